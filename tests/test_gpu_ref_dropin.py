"""The drop-in, exercised: the reference's own integrator (StaticMeshMUSCLHancock,
integrate.py:295-378) steps with GPU subclasses of its own PieceWiseLinear, HLLC and
Mesh classes installed through its check_class setters (integrate.py:148-161), and
matches the same integrator with the plain reference classes to 1e-12.  Needs the
reference's compiled Cython path (oracle/build_ref.py, built by __graft_entry__.build())."""
import os

import numpy as np
import pytest

import phd_code_gb300._lib as L
import ref_harness as rh
from _util import elem_rel, lattice_mesh, smooth_state
from ref_binding import CONS, PRIM, gpu_plugins

pytestmark = pytest.mark.gpu


def _build(R, integrate_mod, mesh, prim, rec_cls, riem_cls, mesh_cls):
    n, F = mesh.n_cells, mesh.n_faces
    pc = R["HydroParticleCreator"](num=n, dim=2)
    dm = R["DomainManager"](xmin=list(mesh.xmin), xmax=list(mesh.xmax), initial_radius=0.1)
    bc = R["Periodic"]() if mesh.boundary == "periodic" else R["Reflective"]()
    m = mesh_cls(regularize=True, eta=0.25)
    rec = rec_cls(limiter="arepo", gizmo_limiter=True)
    rs = riem_cls(cfl=0.5, boost=True)
    eos = R["IdealGas"](gamma=1.4)
    integ = integrate_mod.StaticMeshMUSCLHancock(dt=0.0)
    # the reference's setters, each behind check_class
    integ.set_particles(pc)
    integ.set_mesh(m)
    integ.set_reconstruction(rec)
    integ.set_riemann(rs)
    integ.set_domain_manager(dm)
    integ.set_equation_state(eos)
    integ.set_boundary_condition(bc)
    integ.initialize()
    # the tessellation: this build's host mesh (CGAL is not installed), injected as the
    # reference's Mesh.build_geometry would leave it (mesh.pyx:255-323)
    pc["position-x"][:] = mesh.x[0]
    pc["position-y"][:] = mesh.x[1]
    pc["tag"][:] = mesh.tag
    pc["type"][:] = mesh.type
    pc["map"][:] = mesh.map
    pc["ids"][:] = np.arange(n, dtype=np.int32)
    pc["volume"][:] = mesh.vol
    pc["dcom-x"][:] = mesh.dcom[0]
    pc["dcom-y"][:] = mesh.dcom[1]
    for k, f in enumerate(PRIM):
        pc[f][:] = prim[k]
    m.faces.resize(F)
    for name, val in (("pair-i", mesh.pair_i), ("pair-j", mesh.pair_j), ("area", mesh.area),
                      ("com-x", mesh.com[0]), ("com-y", mesh.com[1]), ("normal-x", mesh.normal[0]),
                      ("normal-y", mesh.normal[1]), ("velocity-x", np.zeros(F)), ("velocity-y", np.zeros(F))):
        m.faces[name][:] = val
    R["set_neighbors"](m, mesh.nbr_ptr.tolist(), mesh.nbr_idx.tolist())
    eos.conservative_from_primitive(pc)
    return integ, pc, m, rec, dm


@pytest.mark.parametrize("boundary", ["periodic", "reflective"])
def test_reference_integrator_with_gpu_plugin_subclasses(boundary):
    if not rh.available():
        pytest.skip("the reference's compiled Cython path is not built on this machine")
    R = rh._import()
    from phd.integrate import integrate as integrate_mod
    from phd.mesh.mesh import Mesh
    GpuPLM, GpuHLLC, GpuMesh = gpu_plugins(R["PieceWiseLinear"], R["HLLC"], Mesh, L.LIB_PATH)
    mesh = lattice_mesh(12, boundary, seed=5)
    prim = smooth_state(mesh, "wave")
    ref, pc_ref, _, _, _ = _build(R, integrate_mod, mesh, prim, R["PieceWiseLinear"], R["HLLC"], Mesh)
    gpu, pc_gpu, m_gpu, rec_gpu, dm_gpu = _build(R, integrate_mod, mesh, prim, GpuPLM, GpuHLLC, GpuMesh)
    csr = (mesh.nbr_ptr, mesh.nbr_idx)
    rec_gpu.csr = csr
    m_gpu.csr, m_gpu.domain_manager = csr, dm_gpu
    assert isinstance(gpu.reconstruction, GpuPLM) and isinstance(gpu.riemann, GpuHLLC)
    with pytest.raises(RuntimeError, match="is not type"):
        gpu.set_riemann(object())                      # the guard the subclasses pass
    for _ in range(3):
        dt_ref, dt_gpu = ref.compute_time_step(), gpu.compute_time_step()
        assert abs(dt_gpu - dt_ref) <= 1e-12 * dt_ref
        ref.evolve_timestep()
        gpu.evolve_timestep()
    nr = mesh.n_real
    for names in (PRIM, CONS):
        a = np.stack([np.asarray(pc_gpu[f])[:nr] for f in names])
        b = np.stack([np.asarray(pc_ref[f])[:nr] for f in names])
        assert elem_rel(a, b) <= 1e-12, names
