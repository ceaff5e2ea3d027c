"""Reconstruction plugins on the device.

Mirrors ``phd/reconstruction/reconstruction.pyx``: ``ReconstructionBase`` (:15-129),
``PieceWiseConstant`` (:131-353) and ``PieceWiseLinear`` (:355-1079) with the same
methods and arguments (``add_fields``, ``initialize``, ``compute_gradients``,
``add_spatial``, ``add_temporal``, ``compute_states``) and the same public containers
(``left_states``, ``right_states``, ``grad``).  Every call launches the FP64 kernel of
that stage through the C ABI; nothing is computed on the host.
"""
from . import _lib as L
from .containers import CarrayContainer
from .device import DeviceClock


class ReconstructionBase:
    def __init__(self):
        self.fields_registered = False
        self.has_passive_scalars = False
        self.left_states = None
        self.right_states = None

    def initialize(self):
        raise NotImplementedError("Reconstruction::initialize called!")

    def add_fields(self, particles):
        raise NotImplementedError("Reconstruction::initialize called!")

    def compute_gradients(self, particles, mesh, domain_manager):
        raise NotImplementedError("Reconstruction::_compute_gradients called!")

    def add_spatial(self, particles, mesh, gamma, domain_manager, dt, boost):
        raise NotImplementedError("Reconstruction::add_spatial called!")

    def add_temporal(self, particles, mesh, gamma, domain_manager, dt, boost):
        raise NotImplementedError("Reconstruction::add_temporal called!")

    def compute_states(self, particles, mesh, gamma, domain_manager, dt, boost):
        raise NotImplementedError("Reconstruction::compute called!")

    # shared helpers ------------------------------------------------------------
    def _register(self, particles):
        if "primitive" not in particles.carray_named_groups or \
                "velocity" not in particles.carray_named_groups:
            raise RuntimeError("ERROR: Missing fields in particles!")
        if "passive-scalars" in particles.carray_named_groups:
            # the reference's passive-scalar branch references attributes it never
            # defines (reconstruction.pyx:194,320-321,537,1005-1006) and cannot run
            raise NotImplementedError("passive scalars are not supported")
        self.prim_fields = list(particles.carray_named_groups["primitive"])
        self.vel_fields = list(particles.carray_named_groups["velocity"])
        self.dim = len(particles.carray_named_groups["position"])
        self.fields_registered = True

    def _state_containers(self, device):
        if not self.fields_registered:
            raise RuntimeError("Reconstruction did not set fields to reconstruct!")
        groups = {"primitive": self.prim_fields, "velocity": self.vel_fields}
        self.left_states = CarrayContainer(0, device=device)
        self.right_states = CarrayContainer(0, device=device)
        for c in (self.left_states, self.right_states):
            c.register_block("primitive", self.prim_fields)
            c.carray_named_groups = dict(groups)

    def _states(self, particles, mesh, gamma, dt, boost, linear, stages, gizmo=False):
        dm = mesh._need()
        if self.left_states is None:
            self._state_containers(particles.device)
        self.left_states.resize(dm.n_faces)
        self.right_states.resize(dm.n_faces)
        grad = self.grad.block("primitive") if linear else None
        L.check(L.lib().phd_states_f64(dm.ref, L.ptr(particles.block("primitive")), L.ptr(grad),
                                       L.ptr(mesh.faces.block("velocity")), float(gamma), float(dt),
                                       int(bool(boost)), L.LINEAR if linear else L.CONSTANT,
                                       int(bool(gizmo)), stages,
                                       L.ptr(self.left_states.block("primitive")),
                                       L.ptr(self.right_states.block("primitive")),
                                       L.stream_handle()), "phd_states_f64")


class PieceWiseConstant(ReconstructionBase):
    def add_fields(self, particles):
        self._register(particles)

    def initialize(self, device=None):
        self._state_containers(device or "cuda")

    def compute_gradients(self, particles, mesh, domain_manager):
        pass   # no gradients for constant reconstruction (:236-252)

    def compute_states(self, particles, mesh, gamma, domain_manager, dt, boost):
        self._states(particles, mesh, gamma, dt, boost, linear=False, stages=3)


class PieceWiseLinear(ReconstructionBase):
    def __init__(self, limiter="arepo", gizmo_limiter=True, **kwargs):
        super().__init__()
        if limiter == "arepo":
            self.slope_limiter = L.LIMITER_AREPO
        elif limiter == "tess":
            self.slope_limiter = L.LIMITER_TESS
        else:
            raise RuntimeError("ERROR: Unrecognized limiter")
        self.limiter = limiter
        self.gizmo_limiter = gizmo_limiter
        self.grad = None

    def add_fields(self, particles):
        self._register(particles)
        axes = "xyz"[:self.dim]
        self.grad_fields = [f + "_" + a for f in self.prim_fields for a in axes]

    def initialize(self, device=None):
        dev = device or "cuda"
        self._state_containers(dev)
        axes = "xyz"[:self.dim]
        g = CarrayContainer(0, device=dev)
        g.register_block("primitive", self.grad_fields)
        groups = {"primitive": list(self.grad_fields),
                  "velocity": [f + "_" + a for f in self.vel_fields for a in axes]}
        for f in self.prim_fields:
            groups[f] = [f + "_" + a for a in axes]
        g.carray_named_groups = groups
        self.grad = g

    def compute_gradients(self, particles, mesh, domain_manager, clock=None):
        dm = mesh._need()
        if self.grad is None:
            self.initialize(particles.device)
        self.grad.resize(dm.n_cells)
        clk = clock or DeviceClock(particles.device)
        L.check(L.lib().phd_gradients_f64(dm.ref, L.ptr(particles.block("primitive")), self.slope_limiter,
                                          L.ptr(self.grad.block("primitive")), clk.ptr, L.stream_handle()),
                "phd_gradients_f64")
        if clock is None:
            clk.check_status()
        domain_manager.update_ghost_gradients(particles, self.grad)

    def add_spatial(self, particles, mesh, gamma, domain_manager, dt, boost):
        self._states(particles, mesh, gamma, dt, boost, True, L.STAGE_SPATIAL, self.gizmo_limiter)

    def add_temporal(self, particles, mesh, gamma, domain_manager, dt, boost):
        self._states(particles, mesh, gamma, dt, boost, True, L.STAGE_TEMPORAL, self.gizmo_limiter)

    def compute_states(self, particles, mesh, gamma, domain_manager, dt, boost):
        self._states(particles, mesh, gamma, dt, boost, True, L.STAGE_SPATIAL | L.STAGE_TEMPORAL,
                     self.gizmo_limiter)
