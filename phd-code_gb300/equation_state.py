"""Ideal-gas equation of state on the device.

Mirrors ``phd/equation_state/equation_state.pyx``: ``IdealGas.conservative_from_primitive``
(:43-79), ``primitive_from_conservative`` (:81-117), ``sound_speed`` (:119-121),
``get_gamma`` (:123-125).  Both conversions run over all cells (real and ghost), as in
the reference.
"""
import math

from . import _lib as L


class EquationStateBase:
    def conservative_from_primitive(self, particles):
        raise NotImplementedError("EquationStateBase::conservative_from_primitive called!")

    def primitive_from_conservative(self, particles):
        raise NotImplementedError("EquationStateBase::primitive_from_conservative called!")

    def sound_speed(self, density, pressure):
        raise NotImplementedError("EquationStateBase::sound_speed called!")

    def get_gamma(self):
        raise NotImplementedError("EquationStateBase::get_gamma called!")


class IdealGas(EquationStateBase):
    def __init__(self, gamma=1.4):
        self.gamma = float(gamma)

    def conservative_from_primitive(self, particles):
        n = particles.get_carray_size()
        dim = len(particles.carray_named_groups["position"])
        L.check(L.lib().phd_cons_from_prim_f64(dim, n, self.gamma, L.ptr(particles["volume"]),
                                               L.ptr(particles.block("primitive")),
                                               L.ptr(particles.block("conservative")),
                                               L.stream_handle()), "phd_cons_from_prim_f64")

    def primitive_from_conservative(self, particles):
        n = particles.get_carray_size()
        dim = len(particles.carray_named_groups["position"])
        L.check(L.lib().phd_prim_from_cons_f64(dim, n, self.gamma, L.ptr(particles["volume"]),
                                               L.ptr(particles.block("conservative")),
                                               L.ptr(particles.block("primitive")),
                                               L.stream_handle()), "phd_prim_from_cons_f64")

    def sound_speed(self, density, pressure):
        return math.sqrt(self.gamma * pressure / density)

    def get_gamma(self):
        return self.gamma
