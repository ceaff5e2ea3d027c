"""The FP32 path's FP64 Newton iteration of the exact solver (phd_physics.cuh,
ex_get_pstar_lean) against the reference's iteration (riemann.pyx:974-1090, restated
verbatim as ex_get_pstar), compiled for the host with nvcc: same convergence flag on
every problem, p* and u* equal to FP64 rounding.  No GPU needed."""
import os
import shutil
import subprocess

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)


def _nvcc():
    for c in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if c and os.path.exists(c):
            return c
    return None


def test_lean_newton_matches_reference_iteration(tmp_path):
    nvcc = _nvcc()
    if nvcc is None:
        pytest.skip("nvcc not found")
    exe = str(tmp_path / "exact_newton_check")
    subprocess.run([nvcc, "-O2", "-std=c++17", "-I" + os.path.join(ROOT, "include"),
                    "-I" + os.path.join(ROOT, "phd-code_gb300", "csrc"), "-x", "cu",
                    os.path.join(HERE, "exact_newton_check.cu"), "-o", exe], check=True)
    out = subprocess.run([exe, "200000"], check=True, capture_output=True, text=True).stdout.split()
    n, n_fail, n_flag = int(out[0]), int(out[1]), int(out[2])
    worst_p, worst_u = float(out[3]), float(out[4])
    assert (int(out[5]), int(out[6])) == (7, 5)
    assert n > 150000
    assert n_flag == 0
    assert n_fail < 0.02 * n
    assert worst_p <= 1e-12, worst_p
    assert worst_u <= 1e-13, worst_u
