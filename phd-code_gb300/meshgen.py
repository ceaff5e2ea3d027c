"""Host-side 2D Voronoi mesh in the reference's face-list conventions.

The reference builds its mesh with CGAL on the host (``phd/mesh/tess.cpp``) and keeps
it there; the flux path consumes the result.  CGAL is not available in this
environment, so this module produces the same *kind* of face list from a Delaunay
triangulation and our own circumcentre construction, following the conventions of
``Tess2d::extract_geometry`` (``tess.cpp:238-398``).  Two builders give the same mesh:
``backend="native"`` (default) is the C++ tessellation of ``include/phdtess.h``
(``tess.py``); ``backend="scipy"`` is a numpy construction on scipy/Qhull's Delaunay
triangulation, kept as the independent check of the native one.  They agree face for
face (geometry to rounding) except where four generators are exactly cocircular --
e.g. a generator, its neighbour and their mirror images at a reflective wall -- where
either diagonal is a valid Delaunay edge and the two builders may emit different
zero-area faces.  Conventions:

* faces are emitted per REAL cell ``i`` for each Voronoi edge shared with a
  neighbour ``j`` where ``i < j`` -- ghost indices follow all real indices, so
  ``pair-i`` is always real and ghost--ghost faces never appear (``tess.cpp:363``);
* ``area`` = edge length, ``com`` = edge midpoint, ``normal = (x_j - x_i)/|x_j - x_i|``
  (``tess.cpp:318-383``);
* cell volume = sum of ``0.25*area*h`` over all incident edges and the centroid
  offset ``dcom = cx/vol - x`` from the triangle centroids ``2f/3 + x/3``
  (``tess.cpp:350-393``);
* every cell's face list (``mesh.neighbors``) holds face ids in ascending order
  (``tess.cpp:378-380``);
* ghosts are copies of real "image" cells (``map``), shifted by the box length
  (periodic, ``boundary.pyx:351-400``) or mirrored in one axis (reflective,
  ``boundary.pyx:66-130``), tagged Ghost with type Exterior, and take the image's
  volume and dcom (``mesh.pyx:323`` -> ``domain_manager.pyx:758-774``).

Within each real cell, faces are emitted in counter-clockwise order of the
neighbour direction (CGAL's edge circulator also runs counter-clockwise; its start
edge is arbitrary).  Results of the flux path depend on face order only through the
order of per-cell sums, and the oracle, the reference and the GPU path are always
fed the same face list.
"""
from dataclasses import dataclass, field
from typing import Optional

import numpy as np

from .hilbert import hilbert_order

REAL, GHOST, EXTERIOR, INTERIOR, UNDEFINED = 0, 1, 2, 3, 4   # particle_tags.py:1-6


@dataclass
class HostMesh:
    """One tessellated state: cells (real then ghost) and the face list."""
    dim: int
    n_real: int
    x: np.ndarray            # (dim, n) float64 generator positions
    tag: np.ndarray          # (n,) int8   REAL / GHOST
    type: np.ndarray         # (n,) int8   EXTERIOR for ghosts
    map: np.ndarray          # (n,) int32  image index (ghosts), own index (real)
    vol: np.ndarray          # (n,) float64
    dcom: np.ndarray         # (dim, n) float64
    pair_i: np.ndarray       # (F,) int32
    pair_j: np.ndarray       # (F,) int32
    area: np.ndarray         # (F,) float64
    com: np.ndarray          # (dim, F) float64
    normal: np.ndarray       # (dim, F) float64
    nbr_ptr: np.ndarray      # (n+1,) int32 CSR of face ids per cell (ascending)
    nbr_idx: np.ndarray      # (2F,) int32
    xmin: tuple = (0.0, 0.0)
    xmax: tuple = (1.0, 1.0)
    boundary: str = "periodic"
    face_velocity: Optional[np.ndarray] = None   # (dim, F) float64, if assigned

    @property
    def n_cells(self):
        return self.x.shape[1]

    @property
    def n_ghost(self):
        return self.n_cells - self.n_real

    @property
    def n_faces(self):
        return self.pair_i.shape[0]

    def flip_mask(self):
        """Bit k set for a reflective ghost lying outside the box in axis k; this is
        where ``Reflective.update_gradients/update_fields`` flip signs
        (``boundary.pyx:265-348``).  Zero for periodic ghosts and real cells."""
        m = np.zeros(self.n_cells, dtype=np.int8)
        if self.boundary != "reflective":
            return m
        ext = self.type == EXTERIOR
        for k in range(self.dim):
            out = (self.x[k] < self.xmin[k]) | (self.x[k] > self.xmax[k])
            m |= np.where(ext & out, np.int8(1 << k), np.int8(0)).astype(np.int8)
        return m


def jittered_lattice(n_side, jitter=0.1, seed=0, xmin=(0.0, 0.0), xmax=(1.0, 1.0)):
    """``n_side**2`` generators on a Cartesian lattice, each coordinate jittered
    uniformly by ``+-jitter`` lattice spacings (seeded)."""
    rng = np.random.default_rng(seed)
    dx = (xmax[0] - xmin[0]) / n_side
    dy = (xmax[1] - xmin[1]) / n_side
    ix, iy = np.meshgrid(np.arange(n_side), np.arange(n_side), indexing="ij")
    x = xmin[0] + (ix.ravel() + 0.5) * dx
    y = xmin[1] + (iy.ravel() + 0.5) * dy
    x = x + rng.uniform(-jitter, jitter, x.size) * dx
    y = y + rng.uniform(-jitter, jitter, y.size) * dy
    return np.stack([x, y])


def _ghosts(x, boundary, xmin, xmax, pad):
    """Ghost positions and image indices for real points ``x`` (2, N)."""
    L = np.array(xmax, dtype=np.float64) - np.array(xmin, dtype=np.float64)
    gx, gmap = [], []
    n = x.shape[1]
    idx = np.arange(n, dtype=np.int32)
    if boundary == "periodic":
        for sx in (-1, 0, 1):
            for sy in (-1, 0, 1):
                if sx == 0 and sy == 0:
                    continue
                xs = x[0] + sx * L[0]
                ys = x[1] + sy * L[1]
                keep = ((xs > xmin[0] - pad) & (xs < xmax[0] + pad) &
                        (ys > xmin[1] - pad) & (ys < xmax[1] + pad))
                gx.append(np.stack([xs[keep], ys[keep]]))
                gmap.append(idx[keep])
    elif boundary == "reflective":
        for k in range(2):
            for lo in (True, False):
                edge = xmin[k] if lo else xmax[k]
                near = (x[k] - edge < pad) if lo else (edge - x[k] < pad)
                xs = x[:, near].copy()
                xs[k] = xs[k] - 2.0 * (xs[k] - edge)      # boundary.pyx:105,126
                gx.append(xs)
                gmap.append(idx[near])
    else:
        raise ValueError("boundary must be 'periodic' or 'reflective'")
    return np.concatenate(gx, axis=1), np.concatenate(gmap)


def _circumcenters(p, simp):
    a = p[simp[:, 0]]
    b = p[simp[:, 1]] - a
    c = p[simp[:, 2]] - a
    d = 2.0 * (b[:, 0] * c[:, 1] - b[:, 1] * c[:, 0])
    b2 = b[:, 0] * b[:, 0] + b[:, 1] * b[:, 1]
    c2 = c[:, 0] * c[:, 0] + c[:, 1] * c[:, 1]
    ux = (c[:, 1] * b2 - b[:, 1] * c2) / d
    uy = (b[:, 0] * c2 - c[:, 0] * b2) / d
    return np.stack([a[:, 0] + ux, a[:, 1] + uy], axis=1)


def build_mesh(x_real, boundary="periodic", xmin=(0.0, 0.0), xmax=(1.0, 1.0),
               pad=None, hilbert=True, backend="native"):
    """Tessellate real generators ``x_real`` (2, N) with ghosts for ``boundary``.

    With ``hilbert=True`` the real cells are first reordered along the reference's
    Hilbert key (``phd/hilbert``), so neighbouring cells sit close in memory; the
    returned mesh is in that order (``order`` gives original indices).
    ``backend``: "native" (C++ tessellation, ``tess.py``) or "scipy".
    Returns ``(mesh, order)``.
    """
    if backend not in ("native", "scipy"):
        raise ValueError("backend must be 'native' or 'scipy'")
    x_real = np.ascontiguousarray(x_real, dtype=np.float64)
    n = x_real.shape[1]
    if hilbert:
        box = max(xmax[0] - xmin[0], xmax[1] - xmin[1])
        if backend == "native":
            from . import tess
            from .hilbert import ORDER, quantize
            keys = tess.hilbert_keys_2d(quantize(x_real[0], xmin[0], box), quantize(x_real[1], xmin[1], box), ORDER)
            order = np.argsort(keys, kind="stable")
        else:
            order = hilbert_order(x_real[0], x_real[1], xmin, box)
        x_real = np.ascontiguousarray(x_real[:, order])
    else:
        order = np.arange(n)
    if pad is None:
        area = (xmax[0] - xmin[0]) * (xmax[1] - xmin[1])
        pad = 3.0 * np.sqrt(area / n)
    if backend == "native":
        return _build_native(x_real, boundary, xmin, xmax, pad), order
    for _attempt in range(6):
        try:
            return _build(x_real, boundary, xmin, xmax, pad), order
        except _OpenCell:
            pad *= 2.0
    raise RuntimeError("Mesh failed to converged!")      # mesh.pyx:240-241


class _OpenCell(Exception):
    pass


def _build_native(x_real, boundary, xmin, xmax, pad):
    from . import tess
    o, _pad_used = tess.build_mesh_native(x_real, boundary, xmin, xmax, pad)
    n = x_real.shape[1]
    n_cells = o["x"].shape[1]
    tag = np.full(n_cells, GHOST, dtype=np.int8)
    tag[:n] = REAL
    typ = np.full(n_cells, EXTERIOR, dtype=np.int8)
    typ[:n] = UNDEFINED
    return HostMesh(dim=2, n_real=n, x=o["x"], tag=tag, type=typ, map=o["map"], vol=o["vol"], dcom=o["dcom"],
                    pair_i=o["pair_i"], pair_j=o["pair_j"], area=o["area"], com=o["com"], normal=o["normal"],
                    nbr_ptr=o["nbr_ptr"], nbr_idx=o["nbr_idx"], xmin=tuple(xmin), xmax=tuple(xmax),
                    boundary=boundary)


def _build(x_real, boundary, xmin, xmax, pad):
    from scipy.spatial import Delaunay

    n = x_real.shape[1]
    gx, gmap = _ghosts(x_real, boundary, xmin, xmax, pad)
    pts = np.concatenate([x_real, gx], axis=1).T.copy()          # (n_all, 2)
    n_all = pts.shape[0]
    tri = Delaunay(pts)
    simp = tri.simplices.astype(np.int64)
    nbr = tri.neighbors.astype(np.int64)
    cc = _circumcenters(pts, simp)

    # half-edges: triangle t, local edge k (opposite vertex k)
    T = simp.shape[0]
    t_idx = np.repeat(np.arange(T), 3)
    k_idx = np.tile(np.arange(3), T)
    va = simp[t_idx, (k_idx + 1) % 3]
    vb = simp[t_idx, (k_idx + 2) % 3]
    tn = nbr[t_idx, k_idx]
    hull = tn < 0
    if np.any((va[hull] < n) | (vb[hull] < n)):
        raise _OpenCell()
    keep = (~hull) & (tn > t_idx)
    ea, eb = va[keep], vb[keep]
    p1 = cc[t_idx[keep]]
    p2 = cc[tn[keep]]
    lo = np.minimum(ea, eb)
    hi = np.maximum(ea, eb)

    # per-cell incident edges (both orientations) for volume / centroid of real cells
    cell = np.concatenate([lo, hi])
    other = np.concatenate([hi, lo])
    q1 = np.concatenate([p1, p1])
    q2 = np.concatenate([p2, p2])
    xr = pts[other, 0] - pts[cell, 0]
    yr = pts[other, 1] - pts[cell, 1]
    h = np.sqrt(xr * xr + yr * yr)
    xe = q2[:, 0] - q1[:, 0]
    ye = q2[:, 1] - q1[:, 1]
    ln = np.sqrt(xe * xe + ye * ye)
    fx = 0.5 * (q1[:, 0] + q2[:, 0])
    fy = 0.5 * (q1[:, 1] + q2[:, 1])
    ang = np.arctan2(yr, xr)
    srt = np.lexsort((ang, cell))
    cell, other, h, ln, fx, fy, xr, yr = (a[srt] for a in (cell, other, h, ln, fx, fy, xr, yr))

    # a real cell whose neighbours include the hull was caught above; every real cell
    # must have at least three edges
    real_e = cell < n
    tri_a = 0.25 * ln * h
    counts = np.bincount(cell[real_e], minlength=n)
    if np.any(counts[:n] < 3):
        raise _OpenCell()
    starts = np.concatenate([[0], np.cumsum(counts)[:-1]])
    ce, ar = cell[real_e], tri_a[real_e]
    tx = 2.0 * fx[real_e] / 3.0 + pts[ce, 0] / 3.0
    ty = 2.0 * fy[real_e] / 3.0 + pts[ce, 1] / 3.0
    vol = np.add.reduceat(ar, starts)
    cxs = np.add.reduceat(ar * tx, starts)
    cys = np.add.reduceat(ar * ty, starts)
    dcx = cxs / vol - x_real[0]
    dcy = cys / vol - x_real[1]

    # faces: edges of real cells to a higher index, in (cell, angle) order
    fsel = real_e & (other > cell)
    pair_i = cell[fsel].astype(np.int32)
    pair_j_all = other[fsel].astype(np.int64)
    area = ln[fsel]
    com = np.stack([fx[fsel], fy[fsel]])
    normal = np.stack([xr[fsel] / h[fsel], yr[fsel] / h[fsel]])

    # prune ghosts without faces, keep ghost creation order
    used = np.zeros(n_all, dtype=bool)
    used[:n] = True
    used[pair_j_all] = True
    newidx = np.cumsum(used) - 1
    pair_j = newidx[pair_j_all].astype(np.int32)
    keep_pts = np.nonzero(used)[0]
    ghost_keep = keep_pts[keep_pts >= n]
    g_map = gmap[ghost_keep - n].astype(np.int32)

    n_cells = keep_pts.size
    x = pts[keep_pts].T.copy()
    tag = np.full(n_cells, GHOST, dtype=np.int8)
    tag[:n] = REAL
    typ = np.full(n_cells, EXTERIOR, dtype=np.int8)
    typ[:n] = UNDEFINED
    mp = np.concatenate([np.arange(n, dtype=np.int32), g_map])
    volume = np.concatenate([vol, vol[g_map]])
    dcom = np.stack([np.concatenate([dcx, dcx[g_map]]), np.concatenate([dcy, dcy[g_map]])])

    F = pair_i.size
    cells = np.concatenate([pair_i, pair_j]).astype(np.int64)
    fids = np.concatenate([np.arange(F), np.arange(F)])
    o = np.lexsort((fids, cells))
    nbr_idx = fids[o].astype(np.int32)
    cnt = np.bincount(cells, minlength=n_cells)
    nbr_ptr = np.concatenate([[0], np.cumsum(cnt)]).astype(np.int32)

    return HostMesh(dim=2, n_real=n, x=x, tag=tag, type=typ, map=mp, vol=volume,
                    dcom=dcom, pair_i=pair_i, pair_j=pair_j, area=area, com=com,
                    normal=normal, nbr_ptr=nbr_ptr, nbr_idx=nbr_idx,
                    xmin=tuple(xmin), xmax=tuple(xmax), boundary=boundary)


def fill_ghosts(mesh, prim):
    """Copy real-cell primitives to ghost columns (``copy_particles_serial``,
    ``domain_manager.pyx:486-539``) and flip reflective ghost velocities
    (``Reflective.update_fields``, ``boundary.pyx:309-348``).  ``prim`` is
    ``(dim+2, n_cells)``; returns a new array."""
    out = np.array(prim, dtype=np.float64, copy=True)
    g = np.arange(mesh.n_real, mesh.n_cells)
    out[:, g] = out[:, mesh.map[g]]
    fm = mesh.flip_mask()
    for k in range(mesh.dim):
        flip = (fm & (1 << k)) != 0
        out[1 + k, flip] = -out[1 + k, flip]
    return out
