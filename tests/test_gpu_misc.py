"""Device utilities and the status word: Hilbert keys, reflective flip bits, and the
reference's error conditions reported without faulting the GPU (bounded inputs; every
kernel checks its indices and sets a status bit instead of trapping)."""
import ctypes

import numpy as np
import pytest
import torch

import phd_code_gb300 as pkg
from phd_code_gb300 import _lib as L
from phd_code_gb300.device import DeviceClock, DeviceMesh
from _util import GOLDEN, lattice_mesh, smooth_state

pytestmark = pytest.mark.gpu


def test_device_hilbert_keys_match_reference():
    d = np.load(GOLDEN + "/hilbert_2d.npz")
    fac = 2.0 ** 18
    # positions whose quantisation (x - 0) * 2^18 truncates to the golden integers
    x = torch.tensor(np.stack([(d["xh"] + 0.25) / fac, (d["yh"] + 0.25) / fac]), dtype=torch.float64,
                     device="cuda")
    keys = torch.empty(x.shape[1], dtype=torch.int64, device="cuda")
    L.check(L.lib().phd_hilbert_keys_2d(x.shape[1], L.ptr(x), 0.0, 0.0, fac, 18, L.ptr(keys),
                                        L.stream_handle()), "keys")
    assert np.array_equal(keys.cpu().numpy(), d["keys"])


def test_device_flip_mask():
    m = lattice_mesh(20, "reflective", seed=2)
    dm = DeviceMesh(m)
    assert np.array_equal(dm.flip.cpu().numpy(), m.flip_mask())
    mp = lattice_mesh(20, "periodic", seed=2)
    assert int(DeviceMesh(mp).flip.abs().sum()) == 0


def test_negative_mass_sets_status_and_raises():
    m = lattice_mesh(12, "periodic", seed=1)
    prim = smooth_state(m)
    pc = pkg.HydroParticleCreator(num=m.n_cells, dim=2)
    it = pkg.StaticMeshMUSCLHancock()
    for setter, obj in (("set_particles", pc), ("set_domain_manager", pkg.DomainManager([0, 0], [1, 1])),
                        ("set_boundary_condition", pkg.Periodic()), ("set_mesh", pkg.Mesh()),
                        ("set_reconstruction", pkg.PieceWiseLinear()), ("set_riemann", pkg.HLLC()),
                        ("set_equation_state", pkg.IdealGas(1.4))):
        getattr(it, setter)(obj)
    it.initialize()
    it.before_loop(m, prim)
    it.riemann.fluxes = None
    it.riemann.initialize("cuda")
    it.riemann.fluxes.resize(m.n_faces)
    it.riemann.fluxes.block("flux")[0] = 1e6          # drains every pair-i cell's mass
    with pytest.raises(RuntimeError, match="Mass less than zero in flux update"):
        it.mesh.update_from_fluxes(pc, it.riemann, 1.0)


def test_exact_iteration_cap_sets_status():
    m = lattice_mesh(16, "reflective", seed=3)
    prim = smooth_state(m, "sod")
    dm = DeviceMesh(m)
    F = m.n_faces
    L_ = torch.tensor(prim[:, m.pair_i], device="cuda")
    R_ = torch.tensor(prim[:, m.pair_j], device="cuda")
    fw = torch.zeros((2, F), dtype=torch.float64, device="cuda")
    out = torch.zeros((4, F), dtype=torch.float64, device="cuda")
    clk = DeviceClock()
    L.check(L.lib().phd_riemann_f64(dm.ref, L.EXACT, 1.4, 1, 1, L.ptr(L_), L.ptr(R_), L.ptr(fw), L.ptr(out),
                                    clk.ptr, L.stream_handle()), "riemann")
    st = clk.read().status
    assert st & L.STATUS_RIEMANN_NONCONVERGED
    with pytest.raises(RuntimeError, match="No convergence in Exact Riemann Solver"):
        L.raise_status(st)


def test_corrupt_neighbour_list_sets_bad_index():
    m = lattice_mesh(12, "periodic", seed=5)
    bad = m.nbr_idx.copy()
    bad[5] = (bad[5] + 7) % m.n_faces          # a face that does not touch that cell
    m2 = pkg.meshgen.HostMesh(**{**m.__dict__, "nbr_idx": bad})
    dm = DeviceMesh(m2)
    prim = torch.tensor(smooth_state(m), device="cuda")
    grad = torch.zeros((8, m.n_cells), dtype=torch.float64, device="cuda")
    clk = DeviceClock()
    L.check(L.lib().phd_gradients_f64(dm.ref, L.ptr(prim), 0, L.ptr(grad), clk.ptr, L.stream_handle()), "grad")
    assert clk.read().status & L.STATUS_BAD_INDEX


def test_out_of_range_face_id_is_rejected_not_read():
    m = lattice_mesh(12, "periodic", seed=6)
    bad = m.nbr_idx.copy()
    bad[3] = m.n_faces + 1000                 # outside the face arrays: checked before any load
    m2 = pkg.meshgen.HostMesh(**{**m.__dict__, "nbr_idx": bad})
    st = pkg.FluxStepper(m2, smooth_state(m), solver="hllc")
    st.step(1)
    assert st.read_clock().status & L.STATUS_BAD_INDEX


def test_mesh_without_faces():
    """Empty face list: every entry point returns PHD_OK without launching over faces;
    gradients of isolated cells are zero and the neighbour lists are empty."""
    lib = L.lib()
    s = L.stream_handle()
    n = 5
    x = torch.tensor(np.random.default_rng(0).uniform(0, 1, (2, n)), device="cuda")
    dcom = torch.zeros((2, n), dtype=torch.float64, device="cuda")
    vol = torch.full((n,), 0.2, dtype=torch.float64, device="cuda")
    tag = torch.zeros(n, dtype=torch.int8, device="cuda")
    mp = torch.arange(n, dtype=torch.int32, device="cuda")
    flip = torch.zeros(n, dtype=torch.int8, device="cuda")
    ptr = torch.full((n + 1,), 9, dtype=torch.int32, device="cuda")
    idx = torch.zeros(1, dtype=torch.int32, device="cuda")
    m = L.PhdMesh()
    m.dim, m.n_cells, m.n_real, m.n_faces = 2, n, n, 0
    for name, t in (("tag", tag), ("map", mp), ("flip", flip), ("x", x), ("dcom", dcom), ("vol", vol),
                    ("nbr_ptr", ptr), ("nbr_idx", idx)):
        setattr(m, name, t.data_ptr())
    work = torch.empty(int(lib.phd_csr_work_ints(n)), dtype=torch.int32, device="cuda")
    L.check(lib.phd_build_csr(ctypes.byref(m), L.ptr(ptr), L.ptr(idx), L.ptr(work), None, s), "csr")
    prim = torch.tensor(np.random.default_rng(1).uniform(0.5, 1.5, (4, n)), device="cuda")
    grad = torch.full((8, n), 7.0, dtype=torch.float64, device="cuda")
    clk = DeviceClock("cuda", dt=1e-3)
    L.check(lib.phd_gradients_f64(ctypes.byref(m), L.ptr(prim), L.LIMITER_AREPO, L.ptr(grad), clk.ptr, s), "grad")
    left = torch.zeros((4, 1), dtype=torch.float64, device="cuda")
    flux = torch.zeros((4, 1), dtype=torch.float64, device="cuda")
    L.check(lib.phd_riemann_f64(ctypes.byref(m), L.HLLC, 1.4, 1, 100, L.ptr(left), L.ptr(left), None, L.ptr(flux),
                                clk.ptr, s), "riemann")
    torch.cuda.synchronize()
    assert np.array_equal(ptr.cpu().numpy(), np.zeros(n + 1, dtype=np.int32))
    assert float(grad.abs().max()) == 0.0
    assert clk.read().status == 0
