"""Periodic twin faces: the same physical face computed once from each side.

With periodic ghosts the reference emits a boundary face twice -- as (i, ghost of k)
while tessellating i and as (k, ghost of i) while tessellating k -- and each copy
updates only its real cell (``mesh.pyx:529-544``; ``tess.cpp:363``).  In FP64 the two
copies agree to rounding; in FP32 they would differ by ~1e-7 and break conservation.
``periodic_twins`` pairs the copies so the FP32 path computes one and hands both real
cells the same flux.
"""
import numpy as np


def periodic_twins(mesh):
    """int32 [F]: for each dropped copy the id of the kept copy (the lower face id),
    -1 elsewhere.  Empty pairing for non-periodic meshes."""
    F = mesh.n_faces
    twin = np.full(F, -1, dtype=np.int32)
    if mesh.boundary != "periodic" or F == 0:
        return twin
    nr = mesh.n_real
    f = np.nonzero(mesh.pair_j >= nr)[0]
    if f.size == 0:
        return twin
    i = mesh.pair_i[f].astype(np.int64)
    g = mesh.pair_j[f].astype(np.int64)
    k = mesh.map[g].astype(np.int64)
    L = np.array(mesh.xmax, dtype=np.float64) - np.array(mesh.xmin, dtype=np.float64)
    s = np.rint((mesh.x[:, g] - mesh.x[:, k]) / L[:, None]).astype(np.int64)
    sx, sy = s[0], s[1]
    key = ((i * nr + k) * 3 + (sx + 1)) * 3 + (sy + 1)
    tkey = ((k * nr + i) * 3 + (1 - sx)) * 3 + (1 - sy)
    o = np.argsort(key, kind="stable")
    ks = key[o]
    pos = np.searchsorted(ks, tkey)
    pos = np.minimum(pos, ks.size - 1)
    hit = (ks[pos] == tkey) & (i != k)
    a = f[hit]                   # this copy
    b = f[o[pos[hit]]]           # its twin
    drop = a > b                 # keep the lower face id
    twin[a[drop]] = b[drop]
    return twin
