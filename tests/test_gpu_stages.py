"""FP64 plugin path on the GPU against the reference's own outputs (golden fixtures),
stage by stage, through the reference-shaped plugin classes (FP64: 1e-12)."""
import numpy as np
import pytest
import torch

import phd_code_gb300 as pkg
from _util import CONFIGS, FP64_TOL, load_golden, assert_parity, rel_rows, split

pytestmark = pytest.mark.gpu


def build(m, prim, solver, limiter, boost, reconstruction="linear"):
    pc = pkg.HydroParticleCreator(num=m.n_cells, dim=2, device="cuda")
    dm = pkg.DomainManager(xmin=list(m.xmin), xmax=list(m.xmax), initial_radius=0.1)
    bc = pkg.Periodic() if m.boundary == "periodic" else pkg.Reflective()
    mesh = pkg.Mesh()
    if reconstruction == "linear":
        rec = pkg.PieceWiseLinear(limiter=limiter)
    else:
        rec = pkg.PieceWiseConstant()
    rs = {"hll": pkg.HLL, "hllc": pkg.HLLC}[solver](cfl=0.5, boost=boost) if solver != "exact" else pkg.Exact()
    eos = pkg.IdealGas(gamma=1.4)
    integ = pkg.MovingMeshMUSCLHancock()
    integ.set_particles(pc)
    integ.set_domain_manager(dm)
    integ.set_boundary_condition(bc)
    integ.set_mesh(mesh)
    integ.set_reconstruction(rec)
    integ.set_riemann(rs)
    integ.set_equation_state(eos)
    integ.initialize()
    integ.before_loop(m, prim)
    return integ


@pytest.mark.parametrize("boundary", ["periodic", "reflective"])
@pytest.mark.parametrize("cfg", CONFIGS)
def test_plugin_stages(boundary, cfg):
    m, d = load_golden(boundary)
    solver, limiter, boost = split(cfg)
    it = build(m, d["prim0"], solver, limiter, boost)
    pc, mesh = it.particles, it.mesh
    dt = it.compute_time_step()
    assert abs(dt - float(d[cfg + "/dt"])) <= FP64_TOL * dt
    mesh.assign_generator_velocities(pc, it.equation_state)
    assert_parity(pc.block("w").cpu().numpy(), d[cfg + "/w"])
    mesh.assign_face_velocities(pc)
    assert_parity(mesh.faces.block("velocity").cpu().numpy(), d[cfg + "/face_w"])
    it.reconstruction.compute_gradients(pc, mesh, it.domain_manager)
    assert_parity(it.reconstruction.grad.block("primitive").cpu().numpy(), d[cfg + "/grad"])
    it.reconstruction.compute_states(pc, mesh, 1.4, it.domain_manager, 0.5 * dt, it.riemann.boost)
    assert_parity(it.reconstruction.left_states.block("primitive").cpu().numpy(), d[cfg + "/left"])
    assert_parity(it.reconstruction.right_states.block("primitive").cpu().numpy(), d[cfg + "/right"])
    it.riemann.compute_fluxes(pc, mesh, it.reconstruction, it.equation_state)
    assert_parity(it.riemann.fluxes.block("flux").cpu().numpy(), d[cfg + "/flux"])
    mesh.update_from_fluxes(pc, it.riemann, dt)
    n = m.n_real
    assert_parity(pc.block("conservative").cpu().numpy()[:, :n], d[cfg + "/cons1"][:, :n])


@pytest.mark.parametrize("boundary", ["periodic", "reflective"])
def test_spatial_then_temporal_equals_compute_states(boundary):
    m, d = load_golden(boundary)
    it = build(m, d["prim0"], "hllc", "arepo", True)
    pc, mesh, rec = it.particles, it.mesh, it.reconstruction
    dt = it.compute_time_step()
    mesh.assign_generator_velocities(pc, it.equation_state)
    mesh.assign_face_velocities(pc)
    rec.compute_gradients(pc, mesh, it.domain_manager)
    rec.add_spatial(pc, mesh, 1.4, it.domain_manager, 0.5 * dt, True)
    rec.add_temporal(pc, mesh, 1.4, it.domain_manager, 0.5 * dt, True)
    assert_parity(rec.left_states.block("primitive").cpu().numpy(), d["hllc_arepo_boost/left"])
    assert_parity(rec.right_states.block("primitive").cpu().numpy(), d["hllc_arepo_boost/right"])


@pytest.mark.parametrize("boundary", ["periodic", "reflective"])
def test_constant_reconstruction(boundary):
    m, d = load_golden(boundary)
    it = build(m, d["prim0"], "hllc", "arepo", True, reconstruction="constant")
    pc, mesh = it.particles, it.mesh
    dt = it.compute_time_step()
    it.reconstruction.compute_states(pc, mesh, 1.4, it.domain_manager, 0.5 * dt, True)
    assert_parity(it.reconstruction.left_states.block("primitive").cpu().numpy(), d["pwc_hllc/left"])
    it.riemann.compute_fluxes(pc, mesh, it.reconstruction, it.equation_state)
    assert_parity(it.riemann.fluxes.block("flux").cpu().numpy(), d["pwc_hllc/flux"])


@pytest.mark.parametrize("boundary", ["periodic", "reflective"])
@pytest.mark.parametrize("solver", ["hllc", "exact"])
def test_integrator_three_steps(boundary, solver):
    m, d = load_golden(boundary)
    it = build(m, d["prim0"], solver, "arepo", True)
    dts = []
    for _ in range(3):
        dts.append(it.compute_time_step())
        it.evolve_timestep()
    assert_parity(np.array(dts), d["run3_%s/dts" % solver])
    assert_parity(it.particles.block("primitive").cpu().numpy(), d["run3_%s/prim" % solver])
    assert_parity(it.particles.block("conservative").cpu().numpy(), d["run3_%s/cons" % solver])


def test_known_answer_riemann():
    """phd/riemann/test/test_riemann.py:88-122 known answer through the device solvers."""
    from phd_code_gb300 import _lib as L
    from phd_code_gb300.device import DeviceClock, DeviceMesh
    from phd_code_gb300.meshgen import HostMesh
    m = HostMesh(dim=2, n_real=2, x=np.array([[0.0, 1.0], [0.0, 0.0]]), tag=np.zeros(2, np.int8),
                 type=np.full(2, 4, np.int8), map=np.arange(2, dtype=np.int32), vol=np.ones(2),
                 dcom=np.zeros((2, 2)), pair_i=np.array([0], np.int32), pair_j=np.array([1], np.int32),
                 area=np.ones(1), com=np.array([[0.5], [0.0]]), normal=np.array([[1.0], [0.0]]),
                 nbr_ptr=np.array([0, 1, 2], np.int32), nbr_idx=np.array([0, 0], np.int32))
    dm = DeviceMesh(m)
    clk = DeviceClock()
    for u, ans in ((2.0, (2.0, 4.4, 0.0, 6.8)), (-2.0, (-2.0, 4.4, 0.0, -6.8))):
        st = torch.tensor([[1.0], [u], [0.0], [0.4]], dtype=torch.float64, device="cuda")
        fw = torch.zeros((2, 1), dtype=torch.float64, device="cuda")
        for solver, boost in ((L.HLL, 0), (L.HLLC, 0), (L.HLLC, 1), (L.EXACT, 1)):
            out = torch.zeros((4, 1), dtype=torch.float64, device="cuda")
            L.check(L.lib().phd_riemann_f64(dm.ref, solver, 1.4, boost, 1000, L.ptr(st), L.ptr(st), L.ptr(fw),
                                            L.ptr(out), clk.ptr, L.stream_handle()), "riemann")
            np.testing.assert_allclose(out.cpu().numpy()[:, 0], ans, rtol=0, atol=1e-12)
    assert clk.read().status == 0
