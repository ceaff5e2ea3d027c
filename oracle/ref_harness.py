"""Drive the reference's own compiled Cython flux path on a given mesh and state.

TEST INFRASTRUCTURE ONLY (the checker and the timed CPU baseline, never the product
path).  Needs the build made by ``oracle/build_ref.py``: from the reference tree where it
is mounted, or ``--compile-staged`` from the staged Cython output elsewhere.  The GPU
tests never depend on it; they use the committed golden fixtures and the C
restatement.

The reference objects are wired exactly as ``StaticMeshMUSCLHancock.initialize``
does (``phd/integrate/integrate.py:302-338``); the face list and neighbour lists are
injected in place of the CGAL tessellation (``mesh.pyx:255-323``), and ghost volume /
dcom are those of their images, as ``Mesh.build_geometry`` leaves them.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_BUILD = os.path.join(HERE, "_ref", "build")


def available():
    """The reference modules are importable on this machine."""
    import sysconfig
    return os.path.exists(os.path.join(REF_BUILD, "phd", "riemann",
                                       "riemann" + sysconfig.get_config_var("EXT_SUFFIX")))


def _import():
    if REF_BUILD not in sys.path:
        sys.path.insert(0, REF_BUILD)
    import logging
    logging.getLogger("phd").setLevel(logging.WARNING)
    from phd.utils.particle_creator import HydroParticleCreator
    from phd.mesh.mesh import Mesh
    from phd.domain.domain_manager import DomainManager
    from phd.domain.boundary import Reflective, Periodic
    from phd.reconstruction.reconstruction import PieceWiseLinear, PieceWiseConstant
    from phd.riemann.riemann import HLL, HLLC, Exact
    from phd.equation_state.equation_state import IdealGas
    from phd.mesh.refhelper import set_neighbors
    from phd.hilbert.hilbert import py_hilbert_key_2d
    return dict(HydroParticleCreator=HydroParticleCreator, Mesh=Mesh,
                DomainManager=DomainManager, Reflective=Reflective, Periodic=Periodic,
                PieceWiseLinear=PieceWiseLinear, PieceWiseConstant=PieceWiseConstant,
                HLL=HLL, HLLC=HLLC, Exact=Exact, IdealGas=IdealGas,
                set_neighbors=set_neighbors, py_hilbert_key_2d=py_hilbert_key_2d)


PRIM = ["density", "velocity-x", "velocity-y", "pressure"]
CONS = ["mass", "momentum-x", "momentum-y", "energy"]
GRAD = ["density_x", "density_y", "velocity-x_x", "velocity-x_y",
        "velocity-y_x", "velocity-y_y", "pressure_x", "pressure_y"]


class RefStep:
    """The reference plugins assembled around one mesh."""

    def __init__(self, mesh, prim, gamma=1.4, reconstruction="linear", limiter="arepo",
                 gizmo_limiter=True, riemann="hllc", boost=True, cfl=0.5,
                 face_velocity=None, regularize=True, eta=0.25):
        R = _import()
        self.R = R
        n = mesh.n_cells
        pc = R["HydroParticleCreator"](num=n, dim=2)
        dm = R["DomainManager"](xmin=list(mesh.xmin), xmax=list(mesh.xmax),
                                initial_radius=0.1)
        bc = R["Periodic"]() if mesh.boundary == "periodic" else R["Reflective"]()
        dm.set_boundary_condition(bc)
        dm.register_fields(pc)
        dm.initialize()
        m = R["Mesh"](regularize=regularize, eta=eta)
        m.register_fields(pc)
        m.initialize()
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
        F = mesh.n_faces
        m.faces.resize(F)
        m.faces["pair-i"][:] = mesh.pair_i
        m.faces["pair-j"][:] = mesh.pair_j
        m.faces["area"][:] = mesh.area
        m.faces["com-x"][:] = mesh.com[0]
        m.faces["com-y"][:] = mesh.com[1]
        m.faces["normal-x"][:] = mesh.normal[0]
        m.faces["normal-y"][:] = mesh.normal[1]
        fv = np.zeros((2, F)) if face_velocity is None else face_velocity
        m.faces["velocity-x"][:] = fv[0]
        m.faces["velocity-y"][:] = fv[1]
        R["set_neighbors"](m, mesh.nbr_ptr.tolist(), mesh.nbr_idx.tolist())
        if reconstruction == "linear":
            rec = R["PieceWiseLinear"](limiter=limiter, gizmo_limiter=gizmo_limiter)
        else:
            rec = R["PieceWiseConstant"]()
        rec.add_fields(pc)
        rec.initialize()
        if riemann == "hll":
            rs = R["HLL"](cfl=cfl, boost=boost)
        elif riemann == "hllc":
            rs = R["HLLC"](cfl=cfl, boost=boost)
        else:
            rs = R["Exact"](cfl=cfl)
        rs.add_fields(pc)
        rs.initialize()
        eos = R["IdealGas"](gamma=gamma)
        self.pc, self.dm, self.bc, self.mesh, self.rec, self.rs, self.eos = pc, dm, bc, m, rec, rs, eos
        self.gamma = gamma
        # conserved totals from the primitives (integrate.py:226)
        eos.conservative_from_primitive(pc)

    # -- stage wrappers -------------------------------------------------
    def gradients(self):
        self.rec.compute_gradients(self.pc, self.mesh, self.dm)

    def states(self, dt_half):
        self.rec.compute_states(self.pc, self.mesh, self.gamma, self.dm, dt_half, self.rs.boost)

    def fluxes(self):
        self.rs.compute_fluxes(self.pc, self.mesh, self.rec, self.eos)

    def update(self, dt):
        self.mesh.update_from_fluxes(self.pc, self.rs, dt)

    def time_step(self):
        return self.rs.compute_time_step(self.pc, self.eos)

    def generator_velocities(self):
        self.mesh.assign_generator_velocities(self.pc, self.eos)

    def face_velocities(self):
        self.mesh.assign_face_velocities(self.pc)

    def static_step(self, dt):
        """StaticMeshMUSCLHancock.evolve_timestep (integrate.py:349-378)."""
        self.gradients()
        self.states(0.5 * dt)
        self.fluxes()
        self.update(dt)
        self.dm.update_ghost_fields(self.pc, self.pc.carray_named_groups["conservative"], True)
        self.eos.primitive_from_conservative(self.pc)

    def moving_step_fixed_mesh(self, dt):
        """MovingMeshMUSCLHancock.evolve_timestep (integrate.py:385-428) up to the
        host re-mesh: velocities, flux path, conserved update; the generators are not
        moved and the mesh is kept, then ghosts are refreshed and primitives rebuilt
        as the static step does."""
        self.generator_velocities()
        self.face_velocities()
        self.static_step(dt)

    # -- accessors ------------------------------------------------------
    def get(self, names, container=None):
        c = self.pc if container is None else container
        return np.stack([np.array(c[f], dtype=np.float64) for f in names])

    def prim(self):
        return self.get(PRIM)

    def cons(self):
        return self.get(CONS)

    def grad(self):
        return self.get(GRAD, self.rec.grad)

    def left_right(self):
        return self.get(PRIM, self.rec.left_states), self.get(PRIM, self.rec.right_states)

    def flux(self):
        return self.get(CONS, self.rs.fluxes)

    def w(self):
        return self.get(["w-x", "w-y"])

    def face_w(self):
        return self.get(["velocity-x", "velocity-y"], self.mesh.faces)
