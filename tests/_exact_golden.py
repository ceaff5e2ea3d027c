"""Shared helpers for the exact Riemann golden samples (tests/golden/exact_riemann.npz):
a two-cell mesh with one face per problem (normal x, face at rest) and the flux of the
sampled state at x/t = 0."""
import os

import numpy as np

from phd_code_gb300.meshgen import HostMesh

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "exact_riemann.npz")


def load():
    return np.load(GOLDEN)


def face_mesh(n):
    """Cells 0 and 1 joined by n faces with normal x: face m carries problem m."""
    return HostMesh(dim=2, n_real=2, x=np.array([[0.0, 1.0], [0.0, 0.0]]), tag=np.zeros(2, np.int8),
                    type=np.full(2, 4, np.int8), map=np.arange(2, dtype=np.int32), vol=np.ones(2),
                    dcom=np.zeros((2, 2)), pair_i=np.zeros(n, np.int32), pair_j=np.ones(n, np.int32),
                    area=np.ones(n), com=np.tile([[0.5], [0.0]], (1, n)), normal=np.tile([[1.0], [0.0]], (1, n)),
                    nbr_ptr=np.array([0, n, 2 * n], np.int32),
                    nbr_idx=np.concatenate([np.arange(n), np.arange(n)]).astype(np.int32))


def states(d, sel):
    """[4][n] left and right primitive states (rho, v_x, v_y = 0, p) of the selected problems."""
    lo, ro = d["left"][sel], d["right"][sel]
    z = np.zeros(len(lo))
    return (np.stack([lo[:, 0], lo[:, 1], z, lo[:, 2]]), np.stack([ro[:, 0], ro[:, 1], z, ro[:, 2]]))


def sample_flux(d, sel):
    """[4][n] flux of the exact solution at x/t = 0 (mass, momentum x / y, energy)."""
    rho, u, p = d["sample"][sel].T
    g = d["gamma"][sel]
    e = p / (g - 1.0) + 0.5 * rho * u * u
    return np.stack([rho * u, rho * u * u + p, np.zeros_like(u), u * (e + p)])


def rel_err(got, want):
    """Per field: max |got - want| over the problems / the field's largest |want|."""
    scale = np.maximum(np.max(np.abs(want), axis=1, keepdims=True), 1e-300)
    return np.max(np.abs(got - want) / scale, axis=1)
