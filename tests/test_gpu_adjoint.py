"""Hand-written adjoint of the step against PyTorch-FP64 autograd of the same step
(oracle/torch_step.py) and against central finite differences.
Bounds: one step, relative to the largest adjoint component: 1e-9;
multi-step gradient along random directions vs central FD (h = 1e-6): 1e-6."""
import numpy as np
import pytest
import torch

import torch_step as T
import phd_code_gb300 as pkg
from phd_code_gb300.adjoint import FluxRun, FluxRunRecord, StepRecord, cons_from_prim_t
from phd_code_gb300.device import DeviceMesh
from _util import lattice_mesh, smooth_state

pytestmark = pytest.mark.gpu


def one_step_case(boundary, solver, limiter, boost, reconstruction="linear", seed=0, n_side=16):
    m = lattice_mesh(n_side, boundary, seed=seed + 30)
    prim = smooth_state(m)
    rng = np.random.default_rng(seed)
    fw = 0.05 * rng.standard_normal((2, m.n_faces))
    U = T.cons_from_prim(torch.tensor(prim[:, :m.n_real]), torch.tensor(m.vol[:m.n_real]), 1.4)
    lam_next = torch.tensor(rng.standard_normal((4, m.n_real)))
    dt = 2e-3
    # torch autograd
    tm = T.TorchMesh(m)
    Ut = U.clone().requires_grad_(True)
    out = T.step(tm, Ut, torch.tensor(fw), dt, 1.4, solver=solver, limiter=limiter, boost=boost) \
        if reconstruction == "linear" else None
    if out is None:
        pytest.skip("constant reconstruction not in the torch reference")
    (g_ref,) = torch.autograd.grad((out * lam_next).sum(), Ut)
    # device adjoint
    dm = DeviceMesh(m)
    rec = StepRecord(dm, torch.tensor(fw, device="cuda"), dt)
    run = FluxRunRecord([rec], gamma=1.4, solver=solver, limiter=limiter, boost=boost)
    fwd = run._forward_step(rec, U.cuda())
    np.testing.assert_allclose(fwd.cpu().numpy(), out.detach().numpy(), rtol=1e-11, atol=1e-13)
    lam = run._adjoint_step(rec, U.cuda(), lam_next.cuda())
    g = lam.cpu().numpy()
    gr = g_ref.numpy()
    return np.max(np.abs(g - gr)) / np.max(np.abs(gr))


@pytest.mark.parametrize("boundary", ["periodic", "reflective"])
@pytest.mark.parametrize("solver", ["hllc", "hll"])
@pytest.mark.parametrize("limiter", ["arepo", "tess"])
def test_one_step_adjoint_vs_autograd(boundary, solver, limiter):
    assert one_step_case(boundary, solver, limiter, True) <= 1e-9


@pytest.mark.parametrize("boundary", ["periodic", "reflective"])
def test_one_step_adjoint_lab_frame(boundary):
    assert one_step_case(boundary, "hllc", "arepo", False, seed=3) <= 1e-9


def record_static_run(m, prim, n_steps, cfl=0.4, gamma=1.4, solver="hllc"):
    """Forward FP64 run on a fixed mesh recording its dt schedule (static mesh: w = 0)."""
    dm = DeviceMesh(m)
    st = pkg.FluxStepper(dm, prim, gamma=gamma, cfl=cfl, solver=solver, moving=False)
    recs = []
    fw = torch.zeros((2, m.n_faces), dtype=torch.float64, device="cuda")
    for _ in range(n_steps):
        recs.append(StepRecord(dm, fw, st.read_clock().dt))
        st.step(1)
    return recs


def generic_state(m):
    """Bump plus smooth variation in every field at every cell.  The AREPO / TESS
    limiters are ratios of local differences: where a field is flat to ~1e-11 (a bump on
    an exactly uniform background) a 1e-6 perturbation is not small against the field's
    own variation and finite differences stop measuring a derivative there; this state
    keeps every cell's variation O(1) at the mesh scale."""
    x = m.x
    prim = np.stack([1.0 + 0.2 * np.sin(2 * np.pi * x[0]) * np.sin(2 * np.pi * x[1])
                     + 0.1 * np.exp(-((x[0] - 0.4) ** 2 + (x[1] - 0.6) ** 2) / (2 * 0.1 ** 2)),
                     0.1 * np.sin(2 * np.pi * x[1]) + 0.05 * np.cos(2 * np.pi * x[0]),
                     0.1 * np.cos(2 * np.pi * x[0]) + 0.05 * np.sin(4 * np.pi * x[1]),
                     1.0 + 0.1 * np.sin(2 * np.pi * (x[0] + 2 * x[1]))])
    return pkg.meshgen.fill_ghosts(m, prim)


def multistep_case(m, prim, n_steps, limiter="arepo", checkpoint=5, solver="hllc"):
    recs = record_static_run(m, prim, n_steps, solver=solver)
    run = FluxRunRecord(recs, gamma=1.4, solver=solver, limiter=limiter, checkpoint=checkpoint)
    p0 = torch.tensor(prim[:, :m.n_real], device="cuda")
    tgt = torch.tensor(1.0 + 0.02 * np.sin(2 * np.pi * m.x[0, :m.n_real]), device="cuda")

    def loss(p):
        return ((FluxRun.apply(p, run) - tgt) ** 2).sum()

    p = p0.clone().requires_grad_(True)
    loss(p).backward()
    return run, recs, p0, tgt, loss, p.grad.detach()


def test_multistep_gradient_vs_finite_differences():
    """AREPO limiter (the default and the adjoint workload's).  The TESS limiter takes
    one minimum over every field's and face's ratio, so near-ties between candidates
    put kinks within reach of a 1e-6 perturbation; it is checked against autograd
    below, which follows the same branches."""
    m = lattice_mesh(16, "periodic", seed=4)
    run, recs, p0, tgt, loss, g = multistep_case(m, generic_state(m), 12)
    rng = np.random.default_rng(7)
    h = 1e-6
    errs = []
    for _ in range(8):
        d = torch.tensor(rng.standard_normal(p0.shape), device="cuda")
        d = d / torch.linalg.norm(d)
        with torch.no_grad():
            fd = (loss(p0 + h * d) - loss(p0 - h * d)).item() / (2 * h)
        ad = float((g * d).sum())
        errs.append(abs(fd - ad) / max(abs(fd), 1e-12))
    assert max(errs) <= 1e-6, errs


@pytest.mark.parametrize("state,limiter", [("generic", "arepo"), ("noisy_background", "arepo"),
                                           ("generic", "tess")])
def test_multistep_gradient_vs_torch_autograd(state, limiter):
    """The recorded run's gradient (checkpoint-and-recompute through the hand-written
    kernels) against PyTorch autograd through the same steps (oracle/torch_step.py)."""
    m = lattice_mesh(16, "periodic", seed=4)
    if state == "generic":
        prim = generic_state(m)
    else:
        # the adjoint workload's starting point: uniform background plus seeded noise
        # (an exactly uniform state sits on the limiter's non-differentiable point)
        m, prim, _ = pkg.problems.gaussian_bump(16, background=True)
        rng = np.random.default_rng(11)
        prim = prim.copy()
        prim[:, :m.n_real] += 1e-3 * rng.uniform(-1.0, 1.0, (4, m.n_real))
        prim = pkg.meshgen.fill_ghosts(m, prim)
    run, recs, p0, tgt, loss, g = multistep_case(m, prim, 10, limiter=limiter, checkpoint=4)
    tm = T.TorchMesh(m)
    w = torch.zeros((2, m.n_faces), dtype=torch.float64)
    vol = torch.tensor(m.vol[:m.n_real])
    pp = p0.cpu().clone().requires_grad_(True)
    U = T.cons_from_prim(pp, vol, 1.4)
    for rec in recs:
        U = T.step(tm, U, w, rec.dt, 1.4, limiter=limiter)
    ((U[0] / vol - tgt.cpu()) ** 2).sum().backward()
    gr = pp.grad.numpy()
    assert np.max(np.abs(g.cpu().numpy() - gr)) / np.max(np.abs(gr)) <= 1e-9


@pytest.mark.parametrize("limiter", ["arepo", "tess"])
def test_taped_adjoint_equals_recomputing_adjoint(limiter):
    """The reverse step reading the limiter record of a taped forward step gives the same
    result as the one recomputing the limiter's selections (same arithmetic)."""
    m = lattice_mesh(16, "periodic", seed=8)
    prim = generic_state(m)
    run, recs, p0, tgt, loss, g = multistep_case(m, prim, 3, limiter=limiter, checkpoint=3)
    U0 = cons_from_prim_t(p0.detach(), recs[0].dmesh.vol[:m.n_real], 1.4).contiguous()
    run.forward(U0)
    states = run._replay_segment(0, 3)
    lam = torch.tensor(np.random.default_rng(2).standard_normal((4, m.n_real)), device="cuda")
    for k in range(2, -1, -1):
        cons, prim_k, grad, tape = states[k]
        assert tape is not None
        a = run._adjoint(recs[k], (cons, prim_k, grad, tape), lam)
        b = run._adjoint(recs[k], (cons, prim_k, grad, None), lam)
        assert torch.equal(a, b)
        lam = a


@pytest.mark.parametrize("boundary", ["periodic", "reflective"])
def test_exact_solver_gradient_vs_finite_differences(boundary):
    """The exact solver's reverse (p* by implicit differentiation of the converged Newton
    root, every sampled region) through recorded multi-step runs against central
    differences.  The forward's Newton stops at a relative change of 1e-6, so its p*
    carries a ~1e-12 convergence error that a difference quotient at h = 1e-6 turns into
    ~1e-6 noise; the bound allows for that."""
    m = lattice_mesh(16, boundary, seed=9)
    prim = generic_state(m)
    run, recs, p0, tgt, loss, g = multistep_case(m, prim, 6, solver="exact", checkpoint=3)
    rng = np.random.default_rng(13)
    h = 1e-6
    errs = []
    for _ in range(8):
        d = torch.tensor(rng.standard_normal(p0.shape), device="cuda")
        d = d / torch.linalg.norm(d)
        with torch.no_grad():
            fd = (loss(p0 + h * d) - loss(p0 - h * d)).item() / (2 * h)
        ad = float((g * d).sum())
        errs.append(abs(fd - ad) / max(abs(fd), 1e-12))
    assert np.median(errs) <= 1e-5, errs
    assert max(errs) <= 1e-4, errs


def _bump_workload(n_side, n_steps, checkpoint, noise=1e-3):
    """The differentiation workload at a reduced size: periodic box, gamma 1.4, HLLC,
    CFL 0.4; target = a Gaussian density bump evolved n_steps; the differentiated run
    starts from the background plus seeded noise."""
    mesh, prim_bump, _ = pkg.problems.gaussian_bump(n_side, background=False)
    _, prim_bg, _ = pkg.problems.gaussian_bump(n_side, background=True)
    nr = mesh.n_real
    dm = DeviceMesh(mesh)
    st = pkg.FluxStepper(dm, prim_bump, gamma=1.4, cfl=0.4, solver="hllc", moving=False)
    st.step(n_steps)
    target = st.prim[0, :nr].clone()
    rng = np.random.default_rng(3)
    p_init = prim_bg.copy()
    p_init[:, :nr] += noise * rng.uniform(-1.0, 1.0, (4, nr))
    p_init = pkg.meshgen.fill_ghosts(mesh, p_init)
    recs = record_static_run(mesh, p_init, n_steps)
    run = FluxRunRecord(recs, gamma=1.4, solver="hllc", checkpoint=checkpoint)
    p0 = torch.tensor(p_init[:, :nr], device="cuda")
    return run, p0, target


def test_frozen_forward_records_the_forward_run():
    """RECORD is the ordinary step (same final state as the run's forward to rounding);
    REPLAY at the recorded point gives the recorded run bit for bit."""
    run, p0, target = _bump_workload(24, 20, 5)
    U0 = cons_from_prim_t(p0, run.steps[0].dmesh.vol[:run.n_real], 1.4).contiguous()
    a = run.forward(U0)
    b = run.forward_frozen(U0, record=True)
    c = run.forward_frozen(U0, record=False)
    assert torch.max(torch.abs(a - b)).item() <= 1e-13 * torch.max(torch.abs(a)).item()
    assert torch.equal(b, c)


def test_frozen_finite_differences_match_the_adjoint():
    """The differentiation workload (reduced: 32x32, 40 steps, checkpoint every 10):
    central differences at h = 1e-6 through the branch-frozen forward agree with the
    hand-written adjoint's gradient to 1e-6 in every seeded direction.  (Through the
    free forward the same differences cross limiter switches; not asserted here.)"""
    run, p0, target = _bump_workload(32, 40, 10)

    def loss(p):
        return ((FluxRun.apply(p, run) - target) ** 2).sum()

    p = p0.clone().requires_grad_(True)
    loss(p).backward()
    g = p.grad.detach()
    with torch.no_grad():
        run.final_density_frozen(p0, record=True)

        def frozen(pp):
            return float(((run.final_density_frozen(pp) - target) ** 2).sum())

        rng = np.random.default_rng(11)
        h = 1e-6
        errs = []
        for _ in range(6):
            d = torch.tensor(rng.standard_normal(p0.shape), device="cuda")
            d = d / torch.linalg.norm(d)
            fd = (frozen(p0 + h * d) - frozen(p0 - h * d)) / (2 * h)
            ad = float((g * d).sum())
            errs.append(abs(fd - ad) / max(abs(ad), 1e-300))
    assert max(errs) <= 1e-6, errs
