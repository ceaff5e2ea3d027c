"""Shared helpers for the test-suite (fixtures, tolerances, states)."""
import json
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


# Element-wise parity: each element against its own magnitude, down to ELEM_FLOOR times
# its field's largest magnitude (a field's elements that are exactly zero in the
# reference, or cancellation results near zero, are measured against that floor).  On
# the GB300 every parity comparison of the suite holds at 1e-12 element-wise with a
# floor of 1e-14 (worst element 5.8e-13, worst field normwise 5e-15).
ELEM_FLOOR = 1e-14


def elem_rel(a, b, floor=ELEM_FLOOR):
    """Worst element-wise relative difference of [field][index] arrays:
    max |a - b| / max(|b|, floor * max|b_field|); an identically zero field is compared
    with an absolute floor of 1e-300."""
    a = np.atleast_2d(np.asarray(a, dtype=np.float64))
    b = np.atleast_2d(np.asarray(b, dtype=np.float64))
    worst = 0.0
    for r in range(b.shape[0]):
        scale = np.max(np.abs(b[r])) if b[r].size else 0.0
        den = np.maximum(np.abs(b[r]), max(floor * scale, 1e-300))
        if b[r].size:
            worst = max(worst, float(np.max(np.abs(a[r] - b[r]) / den)))
    return worst


def assert_parity(a, b, tol=FP64_TOL, tag=None):
    """FP64 parity of [field][index] arrays: normwise (per field) and element-wise
    (elem_rel) both within tol.  With PHD_PARITY_REPORT set, the figures (and the
    element-wise one at a floor of 1e-14 of the field scale) are appended to that file."""
    nw, ew = rel_rows(a, b), elem_rel(a, b)
    path = os.environ.get("PHD_PARITY_REPORT")
    if path:
        with open(path, "a") as fh:
            fh.write(json.dumps({"tag": tag or os.environ.get("PYTEST_CURRENT_TEST", "?"), "normwise": nw,
                                 "elementwise": ew, "elementwise_floor_1e-14": elem_rel(a, b, 1e-14)}) + "\n")
    assert nw <= tol, "normwise %.3e > %.1e" % (nw, tol)
    assert ew <= tol, "element-wise %.3e > %.1e" % (ew, tol)


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
