"""Shared helpers for the test-suite (fixtures, tolerances, states)."""
import os

import numpy as np

import phd_code_gb300 as pkg
from phd_code_gb300.meshgen import HostMesh

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
MESH_KEYS = ("x", "tag", "type", "map", "vol", "dcom", "pair_i", "pair_j", "area", "com", "normal",
             "nbr_ptr", "nbr_idx")
CONFIGS = ["hll_arepo_boost", "hllc_arepo_boost", "hllc_tess_boost", "hllc_arepo_lab", "exact_arepo_boost"]

# FP64 parity bound of the flux path against the reference (normwise relative)
FP64_TOL = 1e-12


def load_golden(boundary):
    d = np.load(os.path.join(GOLDEN, "step_%s_12.npz" % boundary))
    kw = {k: d[k] for k in MESH_KEYS}
    m = HostMesh(dim=2, n_real=int(d["n_real"]), xmin=tuple(d["xmin"]), xmax=tuple(d["xmax"]),
                 boundary=str(d["boundary"]), **kw)
    return m, d


def split(cfg):
    solver, limiter, frame = cfg.split("_")
    return solver, limiter, frame == "boost"


def rel(a, b):
    """Normwise relative difference max|a-b| / max|b| (per call, all fields)."""
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    s = np.max(np.abs(b))
    return float(np.max(np.abs(a - b)) / (s if s > 0 else 1.0))


def rel_rows(a, b):
    """Largest per-field normwise relative difference of [field][index] arrays; a
    field that is identically zero in b is compared with an absolute floor of 1e-300."""
    a = np.atleast_2d(np.asarray(a, dtype=np.float64))
    b = np.atleast_2d(np.asarray(b, dtype=np.float64))
    worst = 0.0
    for r in range(b.shape[0]):
        s = np.max(np.abs(b[r]))
        d = np.max(np.abs(a[r] - b[r]))
        worst = max(worst, d / s if s > 0 else d)
    return worst


def smooth_state(m, kind="wave"):
    x = m.x
    if kind == "wave":
        prim = np.stack([1.0 + 0.5 * np.sin(6 * x[0]) * np.cos(3 * x[1]), 0.3 * np.cos(5 * x[1]),
                         0.2 * np.sin(4 * x[0]), 1.0 + 0.3 * np.cos(3 * x[1]) + 0.2 * (x[0] > 0.5)])
    elif kind == "sod":
        left = x[0] < 0.5
        prim = np.stack([np.where(left, 1.0, 0.125), np.zeros_like(x[0]), np.zeros_like(x[0]),
                         np.where(left, 1.0, 0.1)])
    else:
        raise ValueError(kind)
    return pkg.meshgen.fill_ghosts(m, prim)


def lattice_mesh(n_side, boundary, seed=0, jitter=0.1):
    m, _ = pkg.meshgen.build_mesh(pkg.meshgen.jittered_lattice(n_side, jitter=jitter, seed=seed), boundary)
    return m
