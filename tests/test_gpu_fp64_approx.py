"""The FP32 path's exact-solver Newton iteration takes its FP64 reciprocals and
reciprocal square roots from the hardware approximations refined by two Newton-Raphson
steps (phd_physics.cuh ex_rcp, ex_rsqrt).  Against CUDA's correctly rounded reciprocal
and square root on 4M arguments log-uniform over [1e-20, 1e20]: within 2 units of the
last place (1/sqrt(x) is compared with the correctly rounded 1/(correctly rounded
sqrt(x)), itself up to one unit off the exact value)."""
import os
import shutil
import subprocess

import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def test_ex_rcp_and_rsqrt_within_two_ulp(tmp_path):
    nvcc = next((c for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc"))
                 if c and os.path.exists(c)), None)
    if nvcc is None:
        pytest.skip("nvcc not found")
    exe = str(tmp_path / "fp64_approx_check")
    subprocess.run([nvcc, "-O3", "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a",
                    "-I" + os.path.join(ROOT, "include"), "-I" + os.path.join(ROOT, "phd-code_gb300", "csrc"),
                    os.path.join(HERE, "fp64_approx_check.cu"), "-o", exe], check=True)
    out = subprocess.run([exe, str(1 << 22)], check=True, capture_output=True, text=True).stdout.split()
    n, max_rcp, max_rsqrt = int(out[0]), int(out[1]), int(out[2])
    assert n == 1 << 22
    assert max_rcp <= 2, max_rcp
    assert max_rsqrt <= 2, max_rsqrt
