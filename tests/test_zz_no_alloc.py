"""The adjoint step that allocates nothing (phd_adjoint_step_f64_noalloc) against the
allocating one (phd_adjoint_step_f64, work array from the caller).

Callers without a device allocator (a ctypes binding such as the one a maintainer adds
to the reference, or a host program whose device memory belongs to another
framework's pool) use the no-allocation entry point; its work space is a fixed array
inside the library.  Two calls in a row must both reproduce the allocating entry
point's result (FP64 tolerance of the parity tests: 1e-12 normwise relative), and a
mesh too large for the fixed array must be refused before anything runs.  This file is
collected last so a failure here leaves every other test's result standing.
"""
import ctypes

import numpy as np
import pytest
import torch

from phd_code_gb300 import _lib as L
from phd_code_gb300.adjoint import StepRecord, FluxRunRecord
from phd_code_gb300.device import DeviceMesh
from _util import FP64_TOL, lattice_mesh, smooth_state

pytestmark = pytest.mark.gpu


def _inputs(boundary, seed):
    m = lattice_mesh(20, boundary, seed=seed)
    prim = smooth_state(m)
    rng = np.random.default_rng(seed)
    dm = DeviceMesh(m)
    fw = torch.tensor(0.05 * rng.standard_normal((2, m.n_faces)), device="cuda")
    rec = StepRecord(dm, fw, 2e-3)
    run = FluxRunRecord([rec], gamma=1.4, solver="hllc")
    n, nr = dm.n_cells, dm.n_real
    cons = torch.zeros((4, n), dtype=torch.float64, device="cuda")
    p = torch.tensor(prim, device="cuda")
    s = L.stream_handle()
    lib = L.lib()
    L.check(lib.phd_cons_from_prim_f64(2, n, 1.4, L.ptr(dm.vol), L.ptr(p), L.ptr(cons), s), "cons")
    L.check(lib.phd_ghost_cons_f64(dm.ref, L.ptr(cons), s), "ghost")
    prim_d = torch.empty_like(cons)
    L.check(lib.phd_prim_from_cons_f64(2, n, 1.4, L.ptr(dm.vol), L.ptr(cons), L.ptr(prim_d), s), "prim")
    grad = torch.zeros((8, n), dtype=torch.float64, device="cuda")
    L.check(lib.phd_gradients_f64(dm.ref, L.ptr(prim_d), 0, L.ptr(grad), run.clock.ptr, s), "grad")
    lam_next = torch.zeros((4, n), dtype=torch.float64, device="cuda")
    lam_next[:, :nr] = torch.tensor(rng.standard_normal((4, nr)), device="cuda")
    return dm, rec, run, cons, prim_d, grad, fw, lam_next


@pytest.mark.parametrize("boundary", ["periodic", "reflective"])
def test_noalloc_adjoint_matches_allocating_entry_point(boundary):
    dm, rec, run, cons, prim, grad, fw, lam_next = _inputs(boundary, 5)
    lib = L.lib()
    s = L.stream_handle()
    idx = ctypes.byref(rec.index())
    par = ctypes.byref(run.params)
    work = torch.empty(int(lib.phd_adjoint_work_doubles(dm.n_cells, dm.n_faces)), dtype=torch.float64,
                       device="cuda")
    ref = torch.empty_like(lam_next)
    L.check(lib.phd_adjoint_step_f64(dm.ref, idx, par, rec.dt, L.ptr(cons), L.ptr(prim), L.ptr(grad), L.ptr(fw),
                                     L.ptr(lam_next), L.ptr(ref), L.ptr(work), s), "allocating adjoint")
    outs = []
    for _ in range(2):                      # two calls in a row share the fixed work array
        out = torch.full_like(lam_next, float("nan"))
        rc = lib.phd_adjoint_step_f64_noalloc(dm.ref, idx, par, rec.dt, L.ptr(cons), L.ptr(prim), L.ptr(grad),
                                              L.ptr(fw), L.ptr(lam_next), L.ptr(out), s)
        assert rc == L.PHD_OK
        outs.append(out)
    torch.cuda.synchronize()
    r = ref[:, :dm.n_real].cpu().numpy()
    for out in outs:
        o = out[:, :dm.n_real].cpu().numpy()
        assert np.isfinite(o).all()
        assert np.max(np.abs(o - r)) / np.max(np.abs(r)) <= FP64_TOL


def test_noalloc_adjoint_refuses_meshes_beyond_its_array():
    lib = L.lib()
    big = L.PhdMesh()
    big.dim, big.n_cells, big.n_real, big.n_faces = 2, 200000, 190000, 600000   # needs > 4,194,304 doubles
    assert lib.phd_adjoint_work_doubles(big.n_cells, big.n_faces) > L.ADJ_NOALLOC_MAX_DOUBLES
    rc = lib.phd_adjoint_step_f64_noalloc(ctypes.byref(big), None, None, 1e-3, None, None, None, None, None, None,
                                          L.stream_handle())
    assert rc == L.PHD_ERR_SCRATCH_TOO_SMALL


def test_noalloc_adjoint_size_limit_is_exact():
    """A mesh whose work space is exactly the array's size is accepted (the call then
    fails only its argument check, here a missing index table); one face more is
    refused before anything runs."""
    lib = L.lib()
    m = L.PhdMesh()
    m.dim, m.n_cells, m.n_real, m.n_faces = 2, 49712, 49712, 100002    # 32 F + 20 n == the array
    assert lib.phd_adjoint_work_doubles(m.n_cells, m.n_faces) == L.ADJ_NOALLOC_MAX_DOUBLES
    rc = lib.phd_adjoint_step_f64_noalloc(ctypes.byref(m), None, None, 1e-3, None, None, None, None, None, None,
                                          L.stream_handle())
    assert rc == L.PHD_ERR_ARG
    m.n_faces += 1
    assert lib.phd_adjoint_work_doubles(m.n_cells, m.n_faces) == L.ADJ_NOALLOC_MAX_DOUBLES + 32
    rc = lib.phd_adjoint_step_f64_noalloc(ctypes.byref(m), None, None, 1e-3, None, None, None, None, None, None,
                                          L.stream_handle())
    assert rc == L.PHD_ERR_SCRATCH_TOO_SMALL
