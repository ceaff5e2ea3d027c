"""ctypes binding of ``libphdtess.so`` -- the host C++ tessellation of ``include/phdtess.h``.

``Tess2d`` mirrors the reference's ``PyTess2d`` / ``Tess2d`` method set
(``phd/mesh/pytess.pyx:27-57``, ``phd/mesh/tess.h:53-72``) over numpy arrays;
``build_mesh_native`` builds a whole box mesh (real cells, ghost images, faces,
volumes, face lists) in the layout of ``meshgen.HostMesh``.
"""
import ctypes as C
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "libphdtess.so")

ERR_INCOMPLETE, ERR_ARG, ERR_DUPLICATE, ERR_INTERNAL = -1, -2, -3, -4
_MESSAGES = {ERR_INCOMPLETE: "Mesh failed to converged!",      # mesh.pyx:240-241
             ERR_ARG: "bad argument", ERR_DUPLICATE: "duplicate generator position",
             ERR_INTERNAL: "internal tessellation failure"}

_lib = None
_vp, _i32, _f64 = C.c_void_p, C.c_int32, C.c_double
_SIGNATURES = {
    "phd_tess2d_create": ([], _vp),
    "phd_tess2d_destroy": ([_vp], None),
    "phd_tess2d_build_initial": ([_vp, _vp, _vp, _i32, _vp], C.c_int),
    "phd_tess2d_update_initial": ([_vp, _vp, _vp, _i32, _i32], C.c_int),
    "phd_tess2d_count_faces": ([_vp], C.c_int),
    "phd_tess2d_update_radius": ([_vp, _vp, _i32, _vp], C.c_int),
    "phd_tess2d_extract_geometry": ([_vp] * 13, C.c_int),
    "phd_mesh2d_build": ([_vp, _vp, _vp, _i32, _i32, _f64, _f64, _f64, _f64, _f64], C.c_int),
    "phd_mesh2d_build_strips": ([_vp, _vp, _vp, _i32, _i32, _f64, _f64, _f64, _f64, _f64, _i32], C.c_int),
    "phd_mesh2d_sizes": ([_vp, _vp, _vp, _vp], C.c_int),
    "phd_mesh2d_copy": ([_vp] * 16, C.c_int),
    "phd_mesh2d_copy_compact": ([_vp] * 10, C.c_int),
    "phd_mesh2d_copy_compact16": ([_vp] * 4 + [C.c_int32] + [_vp] * 8, C.c_int),
    "phd_hilbert_keys_2d_host": ([_vp, _vp, C.c_int64, C.c_int, _vp], None),
}


def lib():
    """The loaded tessellation library; raises if it was not built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError("phd_code_gb300: %s is missing; run __graft_entry__.build() first" % LIB_PATH)
    L = C.CDLL(LIB_PATH)
    for name, (args, res) in _SIGNATURES.items():
        fn = getattr(L, name)
        fn.argtypes = args
        fn.restype = res
    _lib = L
    return L


def available():
    return os.path.exists(LIB_PATH)


def _p(a):
    return a.ctypes.data_as(C.c_void_p) if a is not None else None


def _check(rc, what):
    if rc < 0:
        raise RuntimeError("%s: %s" % (what, _MESSAGES.get(rc, "error %d" % rc)))
    return rc


class Tess2d:
    """The reference's ``Tess2d`` over numpy arrays (positions ``x`` of shape (2, n))."""

    def __init__(self):
        self._h = lib().phd_tess2d_create()
        if not self._h:
            raise MemoryError("phd_tess2d_create")
        self.n_real = 0
        self.n_total = 0
        self._x = None

    def __del__(self):
        h, self._h = getattr(self, "_h", None), None
        if h and _lib is not None:
            _lib.phd_tess2d_destroy(h)

    def build_initial_tess(self, x, radius, num_real_particles):
        """tess.cpp:35-142; ``radius`` (float64, length >= n) receives 2 * max distance
        to the Voronoi vertices, -1 where the cell is unbounded."""
        self._x = np.ascontiguousarray(x, dtype=np.float64)
        n = int(num_real_particles)
        rc = lib().phd_tess2d_build_initial(self._h, _p(self._x[0]), _p(self._x[1]), n,
                                             _p(radius) if radius is not None else None)
        self.n_real = self.n_total = n
        return rc

    def update_initial_tess(self, x, begin_particles, end_particles):
        """tess.cpp:144-187: insert generators begin..end-1 of ``x``."""
        self._x = np.ascontiguousarray(x, dtype=np.float64)
        rc = lib().phd_tess2d_update_initial(self._h, _p(self._x[0]), _p(self._x[1]), int(begin_particles),
                                              int(end_particles))
        if rc == 0:
            self.n_total = int(end_particles)
        return rc

    def count_number_of_faces(self):
        """tess.cpp:189-236: faces owned by real cells, -1 while a real cell is unbounded."""
        return lib().phd_tess2d_count_faces(self._h)

    def update_radius(self, radius, ids):
        """tess.cpp:400-470 for the generators ``ids``; returns how many stay unbounded."""
        ids = np.ascontiguousarray(ids, dtype=np.int32)
        return lib().phd_tess2d_update_radius(self._h, _p(ids), int(ids.size), _p(radius))

    def extract_geometry(self):
        """tess.cpp:238-398.  Returns a dict: ``volume``, ``dcom`` (real cells),
        ``area``, ``com``, ``normal``, ``pair_i``, ``pair_j``, and the per-cell face lists
        ``nbr_ptr`` / ``nbr_idx`` over all inserted generators."""
        F = _check(self.count_number_of_faces(), "count_number_of_faces")
        n, nt = self.n_real, self.n_total
        out = {"dcom": np.zeros((2, n)), "volume": np.zeros(n), "area": np.zeros(F), "com": np.zeros((2, F)),
               "normal": np.zeros((2, F)), "pair_i": np.zeros(F, np.int32), "pair_j": np.zeros(F, np.int32),
               "nbr_ptr": np.zeros(nt + 1, np.int32), "nbr_idx": np.zeros(2 * F, np.int32)}
        _check(lib().phd_tess2d_extract_geometry(
            self._h, _p(out["dcom"][0]), _p(out["dcom"][1]), _p(out["volume"]), _p(out["area"]),
            _p(out["com"][0]), _p(out["com"][1]), _p(out["normal"][0]), _p(out["normal"][1]),
            _p(out["pair_i"]), _p(out["pair_j"]), _p(out["nbr_ptr"]), _p(out["nbr_idx"])), "extract_geometry")
        return out


def build_mesh_native(x_real, boundary, xmin, xmax, pad, n_strips=0):
    """Real generators ``x_real`` (2, N) in a periodic or reflective box -> the fields of
    ``meshgen.HostMesh`` (x, map, vol, dcom, pair_i, pair_j, area, com, normal,
    nbr_ptr, nbr_idx) and the pad used.  ``n_strips``: strips tessellated on parallel
    host threads (0: chosen by the number of cells)."""
    x = np.ascontiguousarray(x_real, dtype=np.float64)
    n = x.shape[1]
    L = lib()
    h = L.phd_tess2d_create()
    if not h:
        raise MemoryError("phd_tess2d_create")
    try:
        rc = L.phd_mesh2d_build_strips(h, _p(x[0]), _p(x[1]), n, {"periodic": 0, "reflective": 1}[boundary],
                                       float(xmin[0]), float(xmin[1]), float(xmax[0]), float(xmax[1]), float(pad),
                                       int(n_strips))
        _check(rc, "tessellate")
        nc, nf, pad_used = C.c_int32(), C.c_int32(), C.c_double()
        L.phd_mesh2d_sizes(h, C.byref(nc), C.byref(nf), C.byref(pad_used))
        nc, F = nc.value, nf.value
        o = {"x": np.zeros((2, nc)), "map": np.zeros(nc, np.int32), "vol": np.zeros(nc),
             "dcom": np.zeros((2, nc)), "pair_i": np.zeros(F, np.int32), "pair_j": np.zeros(F, np.int32),
             "area": np.zeros(F), "com": np.zeros((2, F)), "normal": np.zeros((2, F)),
             "nbr_ptr": np.zeros(nc + 1, np.int32), "nbr_idx": np.zeros(2 * F, np.int32)}
        _check(L.phd_mesh2d_copy(h, _p(o["x"][0]), _p(o["x"][1]), _p(o["map"]), _p(o["vol"]), _p(o["dcom"][0]),
                                 _p(o["dcom"][1]), _p(o["pair_i"]), _p(o["pair_j"]), _p(o["area"]),
                                 _p(o["com"][0]), _p(o["com"][1]), _p(o["normal"][0]), _p(o["normal"][1]),
                                 _p(o["nbr_ptr"]), _p(o["nbr_idx"])), "copy")
        return o, pad_used.value
    finally:
        L.phd_tess2d_destroy(h)


class CompactMesher:
    """Re-tessellation of the real generators straight into the flux path's compact FP32
    hand-over (``FluxStepper.load_mesh``; ``phd_mesh2d_copy_compact``): the real cells
    keep their order, the ghosts are re-created.  The hand-over lives in pinned host
    buffers reused across calls (grown by 1/8 when a mesh needs more), so the next call
    overwrites them: let the copies of the previous hand-over finish (any
    synchronisation of the stepper's stream) before calling again."""

    def __init__(self, boundary, xmin=(0.0, 0.0), xmax=(1.0, 1.0), n_strips=0, resident=False, pair16=True):
        """``resident``: the device already holds the real cells' positions (from its own
        generator move, ``FluxStepper.move_generators``): hand over ghost codes instead of
        positions (``phd_ghost_positions``).  ``pair16``: pair-j packed as 16-bit
        differences to the owner cell plus a list of the faces that do not fit
        (``pair_dj``, ``pair_x``; 10 B per face instead of 12)."""
        if boundary not in ("periodic", "reflective"):
            raise ValueError("boundary must be 'periodic' or 'reflective'")
        self.boundary, self.xmin, self.xmax, self.n_strips = boundary, tuple(xmin), tuple(xmax), int(n_strips)
        self.resident = bool(resident)
        self.pair16 = bool(pair16)
        self._h = lib().phd_tess2d_create()
        if not self._h:
            raise MemoryError("phd_tess2d_create")
        self._buf = {}

    def __del__(self):
        h, self._h = getattr(self, "_h", None), None
        if h and _lib is not None:
            _lib.phd_tess2d_destroy(h)

    def _pinned(self, name, shape, dtype):
        import torch
        need = int(np.prod(shape))
        b = self._buf.get(name)
        if b is None or b.numel() < need:
            b = torch.empty(need + need // 8 + 16, dtype=dtype, pin_memory=True)
            self._buf[name] = b
        return b[:need].view(shape)

    def __call__(self, x_real, pad=None):
        """Pinned compact hand-over of the tessellation of ``x_real`` (2, N)."""
        import torch
        x = np.ascontiguousarray(x_real, dtype=np.float64)
        n = x.shape[1]
        if pad is None:
            pad = 3.0 * np.sqrt((self.xmax[0] - self.xmin[0]) * (self.xmax[1] - self.xmin[1]) / n)
        L = lib()
        _check(L.phd_mesh2d_build_strips(self._h, _p(x[0]), _p(x[1]), n, {"periodic": 0, "reflective": 1}[self.boundary],
                                         float(self.xmin[0]), float(self.xmin[1]), float(self.xmax[0]),
                                         float(self.xmax[1]), float(pad), self.n_strips), "tessellate")
        nc, nf, pad_used = C.c_int32(), C.c_int32(), C.c_double()
        L.phd_mesh2d_sizes(self._h, C.byref(nc), C.byref(nf), C.byref(pad_used))
        nc, F = nc.value, nf.value
        out = {"map": self._pinned("map", (nc,), torch.int32),
               "tag": self._pinned("tag", (nc,), torch.int8), "type": self._pinned("type", (nc,), torch.int8)}
        if not self.resident:
            out["x"] = self._pinned("x", (2, nc), torch.float64)

        def ptr(k):
            return C.c_void_p(out[k].data_ptr()) if k in out else None

        if not self.pair16:
            out.update(face_ptr=self._pinned("face_ptr", (n + 1,), torch.int32),
                       pair_j=self._pinned("pair_j", (F,), torch.int32),
                       area32=self._pinned("area32", (F,), torch.float32),
                       ct32=self._pinned("ct32", (F,), torch.float32))
            if self.resident:
                out["ghost_code"] = self._pinned("ghost_code", (nc - n,), torch.int8)
            _check(L.phd_mesh2d_copy_compact(self._h, *(ptr(k) for k in ("face_ptr", "pair_j", "area32", "ct32", "x",
                                                                          "map", "tag", "type", "ghost_code"))),
                   "copy_compact")
            return out
        # the small arrays back to back in one pinned block (one copy to the device): the
        # escape list first, in a region of room for `cap` entries, moved to the region's
        # end once its length is known, so that it joins the arrays behind it
        from .device import block_views, compact_block_layout
        out["face32"] = self._pinned("face32", (F, 2), torch.float32)
        cap = getattr(self, "_cap", max(256, F // 64))
        k = C.c_int32()
        for _ in range(2):
            sizes = {"pair_x": 2 * cap, "face_ptr": n + 1, "pair_dj": F, "list_len": nc}
            if self.resident:
                sizes["ghost_code"] = nc - n
            layout, nbytes = compact_block_layout(sizes)
            block = self._pinned("compact_block", (nbytes,), torch.uint8)
            out.update(block_views(block, layout))
            # 16-bit bit patterns held as int16 (the device reads them as uint16)
            rc = L.phd_mesh2d_copy_compact16(self._h, ptr("face_ptr"), ptr("pair_dj"), ptr("pair_x"), cap,
                                             C.byref(k), ptr("list_len"), ptr("face32"), ptr("x"), ptr("map"),
                                             ptr("tag"), ptr("type"), ptr("ghost_code"))
            if rc != -5:                                # -5: the escape list needs room for k
                break
            cap = self._cap = k.value + k.value // 8 + 16
        if rc == -6:                                    # a list longer than 255: counted on the device
            rc = 0
            out.pop("list_len")
        _check(rc, "copy_compact16")
        K = k.value
        start = 8 * (cap - K)                           # byte offset of the moved escape list
        moved = block[start:8 * cap].view(torch.int32)
        moved.copy_(out["pair_x"][:2 * K].clone())
        out["pair_x"] = moved
        out["compact_block"] = block[start:]
        return out


def hilbert_keys_2d(xh, yh, order):
    """hilbert_key_2d (phd/hilbert/hilbert.pyx:9-23) in C++ for int32 arrays."""
    xh = np.ascontiguousarray(xh, dtype=np.int32)
    yh = np.ascontiguousarray(yh, dtype=np.int32)
    keys = np.zeros(xh.shape, dtype=np.int64)
    lib().phd_hilbert_keys_2d_host(_p(xh), _p(yh), int(xh.size), int(order), _p(keys))
    return keys
