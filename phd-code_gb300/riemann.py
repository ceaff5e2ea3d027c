"""Riemann plugins on the device.

Mirrors ``phd/riemann/riemann.pyx``: ``RiemannBase`` (:15-222: ``add_fields``,
``initialize``, ``compute_fluxes``, ``compute_time_step``, public ``cfl``, ``boost``,
``fluxes``), ``HLL`` (:225-504), ``HLLC`` (:507-682) and ``Exact`` (:684-1090; its
constructor forces ``cfl = 0.5`` and ``boost = True`` exactly as the reference's does,
:695-698).  Fluxes are computed in the moving face frame and deboosted to the lab
frame (:190-222).
"""
from . import _lib as L
from .containers import CarrayContainer
from .device import DeviceClock


class RiemannBase:
    solver = None

    def __init__(self, cfl=0.5, **kwargs):
        self.cfl = float(cfl)
        self.fields_registered = False
        self.fluxes = None
        if not hasattr(self, "boost"):
            self.boost = True

    def add_fields(self, particles):
        if "conservative" not in particles.carray_named_groups or \
                "momentum" not in particles.carray_named_groups:
            raise RuntimeError("ERROR: Missing fields in particles!")
        self.flux_fields = list(particles.carray_named_groups["conservative"])
        self.flux_field_groups = {"conservative": list(self.flux_fields),
                                  "momentum": list(particles.carray_named_groups["momentum"])}
        self.fields_registered = True

    def initialize(self, device=None):
        if not self.fields_registered:
            raise RuntimeError("Riemann did not set fields for flux!")
        f = CarrayContainer(0, device=device or "cuda")
        f.register_block("flux", self.flux_fields)
        f.carray_named_groups = {k: list(v) for k, v in self.flux_field_groups.items()}
        self.fluxes = f

    def compute_fluxes(self, particles, mesh, reconstruction, eos, clock=None):
        dm = mesh._need()
        if self.fluxes is None:
            self.initialize(particles.device)
        self.fluxes.resize(dm.n_faces)
        clk = clock or DeviceClock(particles.device)
        L.check(L.lib().phd_riemann_f64(dm.ref, self.solver, eos.get_gamma(), int(bool(self.boost)), 1000,
                                        L.ptr(reconstruction.left_states.block("primitive")),
                                        L.ptr(reconstruction.right_states.block("primitive")),
                                        L.ptr(mesh.faces.block("velocity")), L.ptr(self.fluxes.block("flux")),
                                        clk.ptr, L.stream_handle()), "phd_riemann_f64")
        if clock is None:
            clk.check_status()

    def compute_time_step(self, particles, eos, mesh=None, clock=None):
        """cfl * min over real cells of R/c (boost) or R/(c+|v|) (riemann.pyx:120-188);
        returns a Python float (one device-to-host read)."""
        if mesh is None:
            mesh = getattr(particles, "_mesh", None)
        dm = mesh._need()
        clk = clock or DeviceClock(particles.device)
        L.check(L.lib().phd_time_step_f64(dm.ref, L.ptr(particles.block("primitive")), eos.get_gamma(),
                                          self.cfl, int(bool(self.boost)), 0, clk.ptr, L.stream_handle()),
                "phd_time_step_f64")
        return clk.read().dt


class HLL(RiemannBase):
    solver = L.HLL

    def __init__(self, cfl=0.5, boost=True, **kwargs):
        self.boost = boost
        super().__init__(cfl, **kwargs)


class HLLC(HLL):
    solver = L.HLLC


class Exact(RiemannBase):
    solver = L.EXACT

    def __init__(self, cfl=0.5, **kwargs):
        # the reference ignores its cfl argument here (riemann.pyx:695-698)
        self.boost = True
        self.cfl = 0.5
        self.fields_registered = False
        self.fluxes = None
