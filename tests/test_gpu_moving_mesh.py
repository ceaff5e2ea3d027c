"""Full moving-mesh steps with a host re-tessellation after every step
(MovingMeshMUSCLHancock.evolve_timestep, integrate.py:385-428): the device plugin
integrator against the oracle replaying the same meshes (FP64, 1e-12)."""
import numpy as np
import pytest

import oracle as O
import phd_code_gb300 as pkg
from _util import FP64_TOL, assert_parity, rel_rows

pytestmark = pytest.mark.gpu


def make_integrator(mesh, prim, gamma=1.4):
    pc = pkg.HydroParticleCreator(num=mesh.n_cells, dim=2)
    it = pkg.MovingMeshMUSCLHancock()
    it.set_particles(pc)
    it.set_domain_manager(pkg.DomainManager(list(mesh.xmin), list(mesh.xmax)))
    it.set_boundary_condition(pkg.Reflective() if mesh.boundary == "reflective" else pkg.Periodic())
    it.set_mesh(pkg.Mesh())
    it.set_reconstruction(pkg.PieceWiseLinear())
    it.set_riemann(pkg.HLLC(cfl=0.5))
    it.set_equation_state(pkg.IdealGas(gamma))
    it.initialize()
    it.before_loop(mesh, prim)
    return it


@pytest.mark.parametrize("boundary", ["reflective", "periodic"])
def test_moving_mesh_with_remesh_matches_oracle(boundary):
    if boundary == "reflective":
        mesh, prim, info = pkg.problems.shock_tube(24, seed=2)
    else:
        mesh, prim, info = pkg.problems.gaussian_bump(24, seed=2, background=False)
        x = mesh.x
        prim = prim.copy()
        prim[1] = 0.3 * np.sin(2 * np.pi * x[1])
        prim = pkg.meshgen.fill_ghosts(mesh, prim)
    gamma = info["gamma"]
    meshes = [mesh]

    def remesh(x_moved):
        x_new = x_moved.copy()
        if boundary == "periodic":                       # Periodic.migrate_particles wraps
            x_new = np.mod(x_new, 1.0)
        m, _ = pkg.meshgen.build_mesh(x_new, boundary, hilbert=False)
        meshes.append(m)
        return m

    it = make_integrator(mesh, prim, gamma)
    dts = []
    for _ in range(6):
        dts.append(it.compute_time_step())
        it.evolve_timestep(remesh=remesh)
    gpu_prim = it.particles.block("primitive").cpu().numpy()
    gpu_cons = it.particles.block("conservative").cpu().numpy()

    # the oracle replays: step on mesh k, carry real totals to mesh k+1, refresh ghosts
    p = prim.copy()
    c = O.cons_from_prim(mesh, p, gamma)
    for k in range(6):
        mk = meshes[k]
        dt = O.time_step(mk, p, gamma, 0.5, True)
        assert abs(dt - dts[k]) <= FP64_TOL * dt
        O.OracleStepper(mk, gamma=gamma, solver="hllc", moving=True).step(dt, p, c)
        nxt = meshes[k + 1]
        c_new = np.zeros((4, nxt.n_cells))
        c_new[:, :nxt.n_real] = c[:, :mk.n_real]
        c = O.ghost_refresh_cons(nxt, c_new)
        p = O.prim_from_cons(nxt, c, gamma)
    n = meshes[-1].n_real
    assert_parity(gpu_cons[:, :n], c[:, :n])
    assert_parity(gpu_prim, p)


def test_shock_tube_full_run_to_t_end_matches_oracle():
    """The shock-tube configuration in full: 100x100 jittered lattice, reflective box,
    moving generators re-tessellated after every step, run to t = 0.1 (the last step
    clipped onto t_end as Simulation.compute_time_step does).  The device plugin
    integrator against the oracle replaying the same meshes.  Over the whole run the
    normwise difference stays at round-off level (bound 1e-10: ~50 steps of
    limiter-switching dynamics on top of the per-step 1e-12)."""
    mesh, prim, info = pkg.problems.shock_tube(100, seed=3)
    gamma, t_end = info["gamma"], info["t_end"]
    meshes = [mesh]

    def remesh(x_moved):
        m, _ = pkg.meshgen.build_mesh(x_moved.copy(), "reflective", hilbert=False)
        meshes.append(m)
        return m

    it = make_integrator(mesh, prim, gamma)
    t, dts = 0.0, []
    while t < t_end * (1.0 - 1e-14):
        dt = it.compute_time_step()
        if t + dt >= t_end:
            dt = t_end - t
        it.dt = dt
        dts.append(dt)
        it.evolve_timestep(remesh=remesh)
        t += dt
    assert 20 < len(dts) < 400
    gpu_prim = it.particles.block("primitive").cpu().numpy()
    gpu_cons = it.particles.block("conservative").cpu().numpy()

    p = prim.copy()
    c = O.cons_from_prim(mesh, p, gamma)
    for k, dt in enumerate(dts):
        mk = meshes[k]
        dt_o = O.time_step(mk, p, gamma, 0.5, True)
        if k < len(dts) - 1:
            assert abs(dt_o - dt) <= 1e-10 * dt
        O.OracleStepper(mk, gamma=gamma, solver="hllc", moving=True).step(dt, p, c)
        nxt = meshes[k + 1]
        c_new = np.zeros((4, nxt.n_cells))
        c_new[:, :nxt.n_real] = c[:, :mk.n_real]
        c = O.ghost_refresh_cons(nxt, c_new)
        p = O.prim_from_cons(nxt, c, gamma)
    n = meshes[-1].n_real
    assert_parity(gpu_cons[:, :n], c[:, :n], tol=1e-10)
    assert_parity(gpu_prim, p, tol=1e-10)
