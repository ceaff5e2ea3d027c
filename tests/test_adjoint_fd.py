"""The hand-written reverse routines of the adjoint (phd_adjoint.cuh: HLL / HLLC with and
without boost, the exact solver, wave speeds, GIZMO pair limiter, MUSCL-Hancock half
step) against central
finite differences of the forward routines (phd_physics.cuh) on seeded random cases,
compiled for the host with nvcc.  No GPU needed."""
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


def test_reverse_routines_match_finite_differences(tmp_path):
    nvcc = _nvcc()
    if nvcc is None:
        pytest.skip("nvcc not found")
    exe = str(tmp_path / "adjoint_fd_check")
    subprocess.run([nvcc, "-O2", "-std=c++17", "-I" + os.path.join(ROOT, "include"),
                    "-I" + os.path.join(ROOT, "phd-code_gb300", "csrc"), "-x", "cu",
                    os.path.join(HERE, "adjoint_fd_check.cu"), "-o", exe], check=True)
    out = subprocess.run([exe, "4000"], check=True, capture_output=True, text=True).stdout
    rows = {r.split()[0]: r.split()[1:] for r in out.strip().splitlines()}
    assert set(rows) == {"hllc", "hll", "hllc_lab", "exact", "get_waves", "gizmo_pair", "temporal"}
    for name, (n, compared, worst) in rows.items():
        n, compared, worst = int(n), int(compared), float(worst)
        assert n == 4000
        assert compared >= 0.95 * n, (name, compared)        # the rest crossed a branch switch
        assert worst <= 1e-5, (name, worst)
