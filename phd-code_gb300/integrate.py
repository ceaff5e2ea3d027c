"""Integrators that drive the device plugins stage by stage.

Mirrors ``phd/integrate/integrate.py``: ``StaticMeshMUSCLHancock`` (:287-378) and
``MovingMeshMUSCLHancock`` (:381-428), with the reference's setter checks and stage
order.  Each stage is one device kernel; the host only sequences them.  For the fast
path (one fused launch sequence per step, CUDA graphs, FP32) see ``step.FluxStepper``.
The moving-mesh re-tessellation is the host mesh's job: ``evolve_timestep`` takes a
``remesh`` callback that receives the moved generator positions and returns the new
host mesh.
"""
import numpy as np
import torch

from .domain import BoundaryConditionBase, DomainManager
from .equation_state import EquationStateBase
from .mesh import Mesh
from .reconstruction import ReconstructionBase
from .riemann import RiemannBase


def _check(obj, cls, what):
    if not isinstance(obj, cls):
        raise RuntimeError("%s is not type %s" % (obj.__class__.__name__, cls.__name__))
    return obj


class IntegrateBase:
    def __init__(self, dt=0.0, time=0.0, iteration=0, restart=False):
        self.dt = dt
        self.time = time
        self.iteration = iteration
        self.restart = restart
        self.mesh = self.riemann = self.particles = self.domain_manager = None
        self.equation_state = self.reconstruction = self.boundary_condition = None

    def set_mesh(self, mesh):
        self.mesh = _check(mesh, Mesh, "mesh")

    def set_riemann(self, riemann):
        self.riemann = _check(riemann, RiemannBase, "riemann")

    def set_particles(self, particles):
        self.particles = particles

    def set_domain_manager(self, domain_manager):
        self.domain_manager = _check(domain_manager, DomainManager, "domain_manager")

    def set_boundary_condition(self, boundary_condition):
        self.boundary_condition = _check(boundary_condition, BoundaryConditionBase, "boundary")

    def set_equation_state(self, equation_state):
        self.equation_state = _check(equation_state, EquationStateBase, "equation_state")

    def set_reconstruction(self, reconstruction):
        self.reconstruction = _check(reconstruction, ReconstructionBase, "reconstruction")

    def compute_time_step(self):
        self.dt = self.riemann.compute_time_step(self.particles, self.equation_state, mesh=self.mesh)
        return self.dt


class StaticMeshMUSCLHancock(IntegrateBase):
    def initialize(self, host_mesh=None):
        if not all((self.mesh, self.riemann, self.particles is not None, self.domain_manager,
                    self.equation_state, self.reconstruction, self.boundary_condition)):
            raise RuntimeError("ERROR: Not all setters defined in %s!" % self.__class__.__name__)
        dev = self.particles.device
        self.domain_manager.set_boundary_condition(self.boundary_condition)
        self.domain_manager.register_fields(self.particles)
        self.domain_manager.initialize()
        self.mesh.register_fields(self.particles)
        self.mesh.initialize(dev)
        self.reconstruction.add_fields(self.particles)
        self.reconstruction.initialize(dev)
        self.riemann.add_fields(self.particles)
        self.riemann.initialize(dev)

    def before_loop(self, host_mesh, prim):
        """Adopt the first host mesh and primitive state (all cells, ghosts included),
        then conserved totals (integrate.py:188-231)."""
        self.mesh.load_host_mesh(self.particles, host_mesh)
        self.particles.block("primitive").copy_(torch.as_tensor(np.ascontiguousarray(prim)))
        self.equation_state.conservative_from_primitive(self.particles)

    def _flux_update(self):
        pc, mesh, dm = self.particles, self.mesh, self.domain_manager
        self.reconstruction.compute_gradients(pc, mesh, dm)
        self.reconstruction.compute_states(pc, mesh, self.equation_state.get_gamma(), dm, 0.5 * self.dt,
                                           self.riemann.boost)
        self.riemann.compute_fluxes(pc, mesh, self.reconstruction, self.equation_state)
        mesh.update_from_fluxes(pc, self.riemann, self.dt)

    def evolve_timestep(self):
        self._flux_update()
        self.domain_manager.update_ghost_fields(self.particles,
                                                self.particles.carray_named_groups["conservative"],
                                                True, mesh=self.mesh)
        self.equation_state.primitive_from_conservative(self.particles)
        self.iteration += 1
        self.time += self.dt


class MovingMeshMUSCLHancock(StaticMeshMUSCLHancock):
    def evolve_timestep(self, remesh=None):
        """One moving-mesh step.  ``remesh(x_real_moved) -> host mesh`` rebuilds the
        tessellation on the host (generators moved by dt*w, integrate.py:410-417); with
        ``remesh=None`` the mesh is kept (generators do not move)."""
        pc, mesh = self.particles, self.mesh
        mesh.assign_generator_velocities(pc, self.equation_state)
        mesh.assign_face_velocities(pc)
        self._flux_update()
        if remesh is not None:
            # the host mesh keeps the real cells in their order; ghosts are rebuilt
            n_real = mesh.dmesh.n_real
            x = pc.block("position")[:, :n_real] + self.dt * pc.block("w")[:, :n_real]
            cons_real = pc.block("conservative")[:, :n_real].clone()
            host = remesh(x.cpu().numpy())
            if host.n_real != n_real:
                raise RuntimeError("remesh must keep the real cells")
            mesh.load_host_mesh(pc, host)
            pc.block("conservative")[:, :n_real].copy_(cons_real)
        self.domain_manager.update_ghost_fields(pc, pc.carray_named_groups["conservative"], True,
                                                mesh=mesh)
        self.equation_state.primitive_from_conservative(pc)
        self.iteration += 1
        self.time += self.dt
