"""The device exact Riemann solver (phd_riemann_f64, FP64, the reference's iteration)
against samples of the reference's own Toro exact solver (test_suite/sod/riemann.py;
fixture tests/golden/exact_riemann.npz): Toro's tests 1-5 and 400 seeded random
problems, the flux of the exact solution at the face within 1e-8 of each field's
largest flux (the Newton tolerance 1e-6 with quadratic convergence)."""
import numpy as np
import pytest
import torch

from phd_code_gb300 import _lib as L
from phd_code_gb300.device import DeviceClock, DeviceMesh
from _exact_golden import face_mesh, load, rel_err, sample_flux, states

pytestmark = pytest.mark.gpu

TOL = 1e-8


@pytest.mark.parametrize("gamma", [1.4, 5.0 / 3.0])
def test_device_exact_solver_matches_the_exact_solution(gamma):
    d = load()
    sel = np.flatnonzero(np.isclose(d["gamma"], gamma))
    n = len(sel)
    dm = DeviceMesh(face_mesh(n))
    clk = DeviceClock()
    left, right = (torch.as_tensor(np.ascontiguousarray(a), device="cuda") for a in states(d, sel))
    fw = torch.zeros((2, n), dtype=torch.float64, device="cuda")
    out = torch.zeros((4, n), dtype=torch.float64, device="cuda")
    L.check(L.lib().phd_riemann_f64(dm.ref, L.EXACT, gamma, 1, 1000, L.ptr(left), L.ptr(right), L.ptr(fw),
                                    L.ptr(out), clk.ptr, L.stream_handle()), "phd_riemann_f64")
    torch.cuda.synchronize()
    assert clk.read().status == 0
    err = rel_err(out.cpu().numpy(), sample_flux(d, sel))
    assert np.all(err <= TOL), err
