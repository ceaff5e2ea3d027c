"""Domain bookkeeping the flux path needs: bounds, boundary condition, ghost refresh.

Mirrors the parts of ``phd/domain/domain_manager.pyx`` and ``phd/domain/boundary.pyx``
that sit on the per-step path: ``update_ghost_fields`` for the conserved fields after
the flux update (serial branch :750-774, with ``Reflective.update_fields``
:309-348) and ``update_ghost_gradients`` (:776-835, with ``Reflective.update_gradients``
:265-307).  Ghost creation itself belongs to the host mesh (out of scope here: the
host tessellation supplies ghosts with their image ``map``).
"""
from . import _lib as L


class BoundaryConditionBase:
    name = None


class Reflective(BoundaryConditionBase):
    """Mirror ghosts; normal velocity / momentum / velocity-gradient diagonal flip."""
    name = "reflective"


class Periodic(BoundaryConditionBase):
    """Shifted ghosts; fields and gradients copied unchanged."""
    name = "periodic"


class DomainManager:
    def __init__(self, xmin, xmax, initial_radius=0.1, search_radius_factor=2.0):
        if len(xmin) not in (2, 3):
            raise RuntimeError("Wrong dimension specified")
        if len(xmin) != len(xmax):
            raise RuntimeError("Wrong dimensions for xmin and xmax")
        for a, b in zip(xmin, xmax):
            if b < a:
                raise RuntimeError("ERROR: Boundary inconsistent")
        self.dim = len(xmin)
        self.xmin = list(xmin)
        self.xmax = list(xmax)
        self.initial_radius = initial_radius
        self.search_radius_factor = search_radius_factor
        self.boundary_condition = None
        self.particle_fields_registered = False

    def set_boundary_condition(self, boundary_condition):
        self.boundary_condition = boundary_condition

    def register_fields(self, particles):
        if self.dim != len(particles.carray_named_groups["position"]):
            raise RuntimeError("ERROR: Particle dim does not match")
        n = particles.get_carray_size()
        particles.register_carray(n, "map", "long")
        particles.register_carray(n, "radius", "double")
        particles.register_carray(n, "old_radius", "double")
        self.particle_fields_registered = True

    def initialize(self):
        if not self.particle_fields_registered:
            raise RuntimeError("ERROR: Fields not registered in particles by Mesh!")
        if not self.boundary_condition:
            raise RuntimeError("Not all setters defined in DomainMangaer")

    def update_ghost_fields(self, particles, fields, apply_boundary_condition=False, mesh=None):
        """Ghost conserved fields from their images (+ reflective momentum flip).  Only
        the full conservative group is supported on the device, which is the one call
        the step makes (integrate.py:372-374)."""
        if list(fields) != list(particles.carray_named_groups["conservative"]):
            raise NotImplementedError("device ghost refresh covers the conservative group")
        if mesh is None or mesh.dmesh is None:
            raise RuntimeError("update_ghost_fields needs the device mesh")
        L.check(L.lib().phd_ghost_cons_f64(mesh.dmesh.ref, L.ptr(particles.block("conservative")),
                                           L.stream_handle()), "phd_ghost_cons_f64")

    def update_ghost_gradients(self, particles, gradients):
        """Ghost gradients are produced inside the gradient kernel (each ghost row is
        its image's gradient with the reflective flip), so there is nothing left to do."""
        return None
