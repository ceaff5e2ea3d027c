"""Mesh plugin: face list in HBM, mesh velocities and the face-to-cell update.

Mirrors the per-step part of ``phd/mesh/mesh.pyx``: ``register_fields`` (:100-145),
``initialize`` (:147-166), ``assign_generator_velocities`` (:363-426),
``assign_face_velocities`` (:428-477) and ``update_from_fluxes`` (:479-551).  The
tessellation stays on the host: ``load_host_mesh`` takes the host mesh's cells, ghosts
and face list (what ``build_geometry`` produces, :255-323) and uploads it once.
"""
import torch

from . import _lib as L
from .containers import CarrayContainer
from .device import DeviceMesh


class Mesh:
    def __init__(self, regularize=True, relax_iterations=0, eta=0.25, num_neighbors=128,
                 max_iterations=20):
        self.regularize = regularize
        self.relax_iterations = relax_iterations
        self.eta = eta
        self.num_neighbors = num_neighbors
        self.max_iterations = max_iterations
        self.particle_fields_registered = False
        self.faces = None
        self.dmesh = None

    def register_fields(self, particles):
        dim = len(particles.carray_named_groups["position"])
        n = particles.get_carray_size()
        axes = "xyz"[:dim]
        particles.register_carray(n, "volume", "double")
        particles.register_block("dcom", ["dcom-" + a for a in axes])
        particles.register_block("w", ["w-" + a for a in axes])
        particles.carray_named_groups["dcom"] = ["dcom-" + a for a in axes]
        particles.carray_named_groups["w"] = ["w-" + a for a in axes]
        self.dim = dim
        self.particle_fields_registered = True

    def initialize(self, device=None):
        if not self.particle_fields_registered:
            raise RuntimeError("ERROR: Fields not registered in particles by Mesh!")
        axes = "xyz"[:self.dim]
        dev = device or "cuda"
        f = CarrayContainer(0, device=dev)
        f.register_carray(0, "area", "double")
        f.register_carray(0, "pair-i", "long")
        f.register_carray(0, "pair-j", "long")
        f.register_block("com", ["com-" + a for a in axes])
        f.register_block("velocity", ["velocity-" + a for a in axes])
        f.register_block("normal", ["normal-" + a for a in axes])
        f.carray_named_groups = {"com": ["com-" + a for a in axes],
                                 "velocity": ["velocity-" + a for a in axes],
                                 "normal": ["normal-" + a for a in axes]}
        self.faces = f

    def load_host_mesh(self, particles, host):
        """Adopt one host tessellation (cells real-then-ghost, faces, neighbour lists).
        Particle geometry fields become views of the uploaded mesh; primitive and
        conserved fields keep their first entries and are resized to the new count."""
        dev = particles.device
        self.dmesh = DeviceMesh(host, device=dev)
        dm = self.dmesh
        particles.resize(dm.n_cells)
        particles.attach_block("position", dm.x)
        particles.attach_block("dcom", dm.dcom)
        particles.attach_block("volume", dm.vol.view(1, -1))
        particles.attach_block("tag", dm.tag.view(1, -1))
        particles.attach_block("type", dm.type.view(1, -1))
        if "map" in particles:
            particles.attach_block("map", dm.map.view(1, -1))
        f = self.faces
        f.resize(dm.n_faces)
        f.attach_block("area", dm.area.view(1, -1))
        f.attach_block("pair-i", dm.pair_i.view(1, -1))
        f.attach_block("pair-j", dm.pair_j.view(1, -1))
        f.attach_block("com", dm.com)
        f.attach_block("normal", dm.normal)
        f.block("velocity").zero_()
        particles._mesh = self          # lets compute_time_step(particles, eos) find the cells
        return dm

    @property
    def neighbors(self):
        """Per-cell face lists as CSR (ptr, idx) device tensors (mesh.pxd:34)."""
        return self.dmesh.nbr_ptr, self.dmesh.nbr_idx

    def _need(self):
        if self.dmesh is None:
            raise RuntimeError("no mesh loaded: call load_host_mesh first")
        return self.dmesh

    def assign_generator_velocities(self, particles, equation_state):
        dm = self._need()
        L.check(L.lib().phd_generator_velocities_f64(dm.ref, L.ptr(particles.block("primitive")),
                                                     equation_state.get_gamma(), self.eta,
                                                     int(self.regularize), L.ptr(particles.block("w")),
                                                     L.stream_handle()), "phd_generator_velocities_f64")

    def assign_face_velocities(self, particles):
        dm = self._need()
        L.check(L.lib().phd_face_velocities_f64(dm.ref, L.ptr(particles.block("w")),
                                                L.ptr(self.faces.block("velocity")), L.stream_handle()),
                "phd_face_velocities_f64")

    def update_from_fluxes(self, particles, riemann, dt, clock=None):
        """Segmented conserved update; raises the reference's RuntimeError on negative
        mass or energy (reads the device status, one small device-to-host copy)."""
        from .device import DeviceClock
        dm = self._need()
        clk = clock or DeviceClock(particles.device)
        L.check(L.lib().phd_update_from_fluxes_f64(dm.ref, L.ptr(riemann.fluxes.block("flux")), float(dt),
                                                   L.ptr(particles.block("conservative")), clk.ptr,
                                                   L.stream_handle()), "phd_update_from_fluxes_f64")
        if clock is None:
            clk.check_status()
