"""The headline workloads at their full sizes, through size-independent properties:
the 1024x1024 shear layer (1,048,576 cells, 3.15 M faces) and the 256x256 point
explosion (65,536 cells).  At full size the oracle still takes one FP64 step (a few
seconds on the host), so FP64 parity is checked there too; the rest are properties
that hold at any size -- exact exchange of mass and energy, FP32 tracking FP64,
device-built neighbour lists equal to the host's, the compact hand-over equal to the
full one, bitwise-repeatable steps."""
import numpy as np
import pytest
import torch

import oracle as O
import phd_code_gb300 as pkg
from phd_code_gb300.step import FluxStepper
from _util import FP64_TOL, assert_parity, rel_rows

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def shear():
    mesh, prim, info = pkg.problems.shear_layer(1024, seed=0)
    assert mesh.n_real == 1024 * 1024
    return mesh, prim, info["gamma"]


def test_shear_1024_fp64_step_matches_the_oracle(shear):
    mesh, prim, gamma = shear
    st = FluxStepper(mesh, prim, gamma=gamma, cfl=0.5, solver="hllc", moving=True, precision="fp64")
    st.step(1)
    st.check_status()
    p = prim.copy()
    c = O.cons_from_prim(mesh, p, gamma)
    dt = O.time_step(mesh, p, gamma, 0.5, True)
    assert O.OracleStepper(mesh, gamma=gamma, solver="hllc", moving=True).step(dt, p, c) == 0
    nr = mesh.n_real
    assert_parity(st.cons_host()[:, :nr], c[:, :nr])
    assert_parity(st.prim_host(), p)


def test_shear_1024_fp32_conserves_tracks_fp64_and_repeats(shear):
    mesh, prim, gamma = shear
    nr = mesh.n_real
    runs = []
    for precision in ("fp32", "fp32", "fp64"):
        st = FluxStepper(mesh, prim, gamma=gamma, cfl=0.5, solver="hllc", moving=True, precision=precision)
        c0 = st.cons_host()[:, :nr].sum(axis=1)
        st.step(10)
        st.check_status()
        runs.append((st.cons_host()[:, :nr], c0))
    (a, c0), (b, _), (ref, _) = runs
    assert np.array_equal(a, b)                                  # bitwise repeatable
    c1 = a.sum(axis=1)
    for q in (0, 3):                                             # exact exchange, periodic box
        assert abs(c1[q] - c0[q]) <= 1e-12 * abs(c0[q])
    vol = mesh.vol[:nr]
    assert np.mean(np.abs(a[0] / vol - ref[0] / vol)) <= 1e-5   # L1 density, FP32 vs FP64


def test_shear_1024_device_mesh_data_and_compact_hand_over(shear):
    mesh, prim, gamma = shear
    st = FluxStepper(mesh, prim, gamma=gamma, precision="fp32", handover_records=True)
    geo = [t.clone() for t in (st.face_geo, st.face_ar, st.csr_face, st.csr_nbr, st.cell_geo)]
    e_real = int(mesh.nbr_ptr[mesh.n_real])
    rec = st.entry_rec[:e_real].clone()
    st.load_mesh(st.dmesh.pinned_host_compact(mesh))             # lists, twins, geometry on the device
    torch.cuda.synchronize()
    assert st.dmesh.upload_errors() == 0
    assert np.array_equal(st.dmesh.nbr_ptr.cpu().numpy(), mesh.nbr_ptr)
    assert np.array_equal(st.dmesh.nbr_idx.cpu().numpy(), mesh.nbr_idx)
    assert np.array_equal(st.dmesh.pair_i.cpu().numpy(), mesh.pair_i)
    # the first preparation rounds the host's FP64 normals, the hand-over forms them from
    # the rounded separation: equal to FP32 rounding; everything else bit for bit
    assert torch.equal(geo[0][:, 2:], st.face_geo[:, 2:])
    assert torch.max(torch.abs(geo[0][:, :2] - st.face_geo[:, :2])).item() <= 4e-7
    for old, new in zip(geo[1:4], (st.face_ar, st.csr_face, st.csr_nbr)):
        assert torch.equal(old, new)
    # the gradient records follow the normals: equal to FP32 rounding of the geometry
    assert torch.max(torch.abs(rec - st.entry_rec[:e_real])).item() <= 1e-6 * torch.max(torch.abs(rec)).item()


@pytest.mark.parametrize("solver", ["hllc", "exact"])
def test_explosion_256_fp32_tracks_fp64(solver):
    """The point explosion at its configured size (256x256, E = 1) run to t = 0.05 with
    each solver: FP32 + FP64 accumulation against the FP64 path -- L1 density error
    <= 1e-5 and total-energy drift <= 1e-12 for both precisions.  The exact solver keeps
    its Newton pressure iteration in FP64 inside the FP32 path."""
    mesh, prim, info = pkg.problems.point_explosion(256, seed=0)
    nr, gamma, t_end = mesh.n_real, info["gamma"], info["t_end"]
    out = {}
    for precision in ("fp32", "fp64"):
        st = FluxStepper(mesh, prim, gamma=gamma, cfl=0.5, solver=solver, moving=True, precision=precision,
                         t_end=t_end)
        e0 = st.cons_host()[3, :nr].sum()
        steps = 0
        while st.read_clock().t < t_end * (1.0 - 1e-12) and steps < 2000:
            st.step(25)
            steps += 25
        assert st.read_clock().t >= t_end * (1.0 - 1e-12)
        st.check_status()
        cons = st.cons_host()[:, :nr]
        assert abs(cons[3].sum() - e0) <= 1e-12 * abs(e0)
        out[precision] = cons[0] / mesh.vol[:nr]
    assert np.mean(np.abs(out["fp32"] - out["fp64"])) <= 1e-5


def test_ensemble_256_runs_batch_equals_single_runs():
    """The batching workload at its full size (256 runs, 1,000-65,536 generators each,
    about 4.6 M cells in one batch): runs never interact -- a sample of them, the
    smallest and largest included, evolves bit for bit as it does alone."""
    from phd_code_gb300.ensemble import EnsembleStepper
    runs, _ = pkg.problems.riemann_ensemble(n_runs=256, seed=0)
    sizes = [m.n_real for m, _ in runs]
    assert sum(sizes) > 4_000_000
    ens = EnsembleStepper(runs)
    ens.step(5)
    ens.check_status()
    sample = sorted({int(np.argmin(sizes)), int(np.argmax(sizes)), 7, 100, 200})
    for r in sample:
        m, p = runs[r]
        st = FluxStepper(m, p, precision="fp32", solver="hllc")
        st.step(5)
        assert np.array_equal(ens.run_cons(r), st.cons_host()[:, :m.n_real])
        assert ens.read_clocks()[r].dt == st.read_clock().dt


def test_differentiation_workload_gradient_vs_autograd():
    """The differentiation workload at its full size (128x128 periodic, HLLC, CFL 0.4,
    200 recorded steps, checkpoint every 20; start: the background with 1e-3 seeded
    noise; loss: squared distance of the final density to the evolved Gaussian bump):
    the hand-written adjoint's gradient against PyTorch autograd through the independent
    FP64 step (oracle/torch_step.py) over the same 200 steps.  Autograd follows the
    branches its own forward pass takes, as the adjoint does, so this measures the
    derivative of the piecewise-smooth map on the branch actually taken -- which central
    differences cannot, once the perturbation crosses a limiter switch."""
    import torch_step as T
    from phd_code_gb300.adjoint import FluxRun, FluxRunRecord, StepRecord
    from phd_code_gb300.device import DeviceMesh
    mesh, prim_bump, _ = pkg.problems.gaussian_bump(128, background=False)
    _, prim_bg, _ = pkg.problems.gaussian_bump(128, background=True)
    nr = mesh.n_real
    dm = DeviceMesh(mesh)
    st_t = FluxStepper(dm, prim_bump, gamma=1.4, cfl=0.4, solver="hllc", moving=False)
    st_t.step(200)
    target = st_t.prim[0, :nr].clone()
    rng = np.random.default_rng(3)
    p_init = prim_bg.copy()
    p_init[:, :nr] += 1e-3 * rng.uniform(-1.0, 1.0, (4, nr))
    p_init = pkg.meshgen.fill_ghosts(mesh, p_init)
    st = FluxStepper(dm, p_init, gamma=1.4, cfl=0.4, solver="hllc", moving=False)
    fw = torch.zeros((2, mesh.n_faces), dtype=torch.float64, device="cuda")
    recs = []
    for _ in range(200):
        recs.append(StepRecord(dm, fw, st.read_clock().dt))
        st.step(1)
    run = FluxRunRecord(recs, gamma=1.4, solver="hllc", checkpoint=20)
    p0 = torch.as_tensor(p_init[:, :nr]).cuda().requires_grad_(True)
    ((FluxRun.apply(p0, run) - target) ** 2).sum().backward()
    g = p0.grad.detach()
    # autograd through the PyTorch FP64 step on the device, same dt schedule
    tm = T.TorchMesh(mesh, device="cuda")
    vol = torch.as_tensor(mesh.vol[:nr]).cuda()
    pp = torch.as_tensor(p_init[:, :nr]).cuda().requires_grad_(True)
    U = T.cons_from_prim(pp, vol, 1.4)
    for rec in recs:
        U = T.step(tm, U, fw, rec.dt, 1.4)
    ((U[0] / vol - target) ** 2).sum().backward()
    gr = pp.grad.detach()
    rel = (torch.linalg.norm(g - gr) / torch.linalg.norm(gr)).item()
    print("differentiation workload: adjoint vs autograd, normwise relative difference %.3e" % rel)
    assert rel <= 1e-10, rel
