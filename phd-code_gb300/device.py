"""Device-resident mesh, clock and state for the GB300 flux path.

``DeviceMesh`` uploads one tessellated state (the face list and cell geometry that
the host mesh produces each step, ``mesh.pyx:255-323``) into HBM as
structure-of-arrays tensors and exposes the ``phd_mesh`` C structure pointing at them.
``DeviceClock`` is the device-side ``phd_clock`` (time step, time, CFL accumulator,
status bits).  All arithmetic happens in ``libphdflux.so``.
"""
import ctypes as C
import math

import numpy as np
import torch

from . import _lib as L

F64 = torch.float64


class _nullctx:
    def __enter__(self):
        return None

    def __exit__(self, *a):
        return False


def _dev(device):
    d = torch.device(device)
    if d.type != "cuda":
        raise RuntimeError("phd_code_gb300 runs on CUDA devices only (got %s)" % d)
    return d


# The small arrays of a packed compact hand-over back to back in one block, in the order
# phd_load_mesh_f32 copies them (each array's offset a multiple of its element size: the
# element sizes do not increase along the block), so the host block and a staging block
# of the same layout go over as one copy.
COMPACT_BLOCK = (("pair_x", torch.int32), ("face_ptr", torch.int32), ("pair_dj", torch.int16),
                 ("list_len", torch.uint8), ("ghost_code", torch.int8))


def compact_block_layout(sizes):
    """{name: (byte offset, count, dtype)} and the block's bytes for the arrays named in
    ``sizes`` (element counts) in COMPACT_BLOCK order."""
    layout, off = {}, 0
    for nm, dt in COMPACT_BLOCK:
        if nm in sizes:
            layout[nm] = (off, int(sizes[nm]), dt)
            off += int(sizes[nm]) * torch.empty((), dtype=dt).element_size()
    return layout, off


def block_views(block, layout):
    """Typed views of a uint8 block at the layout's offsets."""
    out = {}
    for nm, (off, cnt, dt) in layout.items():
        es = torch.empty((), dtype=dt).element_size()
        out[nm] = block[off:off + cnt * es].view(dt)
    return out


class DeviceMesh:
    """One tessellation in HBM (cells real-then-ghost, faces, CSR neighbour lists)."""

    def __init__(self, host, device="cuda", stream=None):
        dev = _dev(device)
        self.device = dev
        self.host = host
        self.dim = host.dim
        self.n_cells = host.n_cells
        self.n_real = host.n_real
        self.n_faces = host.n_faces
        self.boundary = host.boundary
        self.xmin = tuple(host.xmin)
        self.xmax = tuple(host.xmax)

        def up(a, dt):
            return torch.from_numpy(np.ascontiguousarray(a, dtype=dt)).to(dev, non_blocking=False)

        self.tag = up(host.tag, np.int8)
        self.type = up(host.type, np.int8)
        self.map = up(host.map, np.int32)
        self.x = up(host.x, np.float64)
        self.dcom = up(host.dcom, np.float64)
        self.vol = up(host.vol, np.float64)
        self.pair_i = up(host.pair_i, np.int32)
        self.pair_j = up(host.pair_j, np.int32)
        self.area = up(host.area, np.float64)
        self.com = up(host.com, np.float64)
        self.normal = up(host.normal, np.float64)
        self.nbr_ptr = up(host.nbr_ptr, np.int32)
        self.nbr_idx = up(host.nbr_idx, np.int32)
        self.flip = torch.zeros(self.n_cells, dtype=torch.int8, device=dev)
        xmin = (C.c_double * 3)(*(list(self.xmin) + [0.0] * (3 - self.dim)))
        xmax = (C.c_double * 3)(*(list(self.xmax) + [0.0] * (3 - self.dim)))
        L.check(L.lib().phd_flip_mask(self.dim, self.n_cells, L.ptr(self.type), L.ptr(self.x),
                                      xmin, xmax, int(self.boundary == "reflective"),
                                      L.ptr(self.flip), L.stream_handle(stream)), "phd_flip_mask")
        self._real_type = np.ascontiguousarray(host.type[:self.n_real], dtype=np.int8)
        self._store = {}
        s = L.PhdMesh()
        self.struct = s
        self.ref = C.byref(s)
        self._point_struct()

    def _point_struct(self):
        s = self.struct
        s.dim, s.n_cells, s.n_real, s.n_faces = self.dim, self.n_cells, self.n_real, self.n_faces
        for name in ("tag", "map", "flip", "x", "dcom", "vol", "pair_i", "pair_j", "area", "com",
                     "normal", "nbr_ptr", "nbr_idx"):
            setattr(s, name, getattr(self, name).data_ptr())

    # arrays per cell / per face: (name, shape(dim, n_cells, n_faces), dtype)
    _SIZED = (("tag", lambda d, n, F: (n,), torch.int8), ("type", lambda d, n, F: (n,), torch.int8),
              ("map", lambda d, n, F: (n,), torch.int32), ("flip", lambda d, n, F: (n,), torch.int8),
              ("x", lambda d, n, F: (d, n), F64), ("dcom", lambda d, n, F: (d, n), F64),
              ("vol", lambda d, n, F: (n,), F64), ("pair_i", lambda d, n, F: (F,), torch.int32),
              ("pair_j", lambda d, n, F: (F,), torch.int32), ("area", lambda d, n, F: (F,), F64),
              ("com", lambda d, n, F: (d, F), F64), ("normal", lambda d, n, F: (d, F), F64),
              ("nbr_ptr", lambda d, n, F: (n + 1,), torch.int32),
              ("nbr_idx", lambda d, n, F: (2 * F,), torch.int32))

    def resize(self, n_cells, n_faces):
        """Re-shape every per-cell and per-face array for a tessellation with other
        cell / face counts (the real cells stay: only the ghosts and faces change).
        Storage grows with 1/8 headroom and is reused while it is large enough; the
        contents are undefined afterwards (a full upload follows).  Returns True when
        any array moved to new storage."""
        n_cells, n_faces = int(n_cells), int(n_faces)
        if n_cells < self.n_real:
            raise ValueError("a tessellation holds at least its real cells")
        moved = False
        for name, shape_of, dt in self._SIZED:
            shape = shape_of(self.dim, n_cells, n_faces)
            need = int(np.prod(shape))
            store = self._store.get(name)
            if store is None:
                store = getattr(self, name).reshape(-1)
            if store.numel() < max(need, 1):
                store = torch.empty(need + need // 8 + 16, dtype=dt, device=self.device)
                moved = True
            self._store[name] = store
            setattr(self, name, store[:need].view(shape))
        if hasattr(self, "_csr_work"):
            need = int(L.lib().phd_csr_work_ints(n_cells))
            if self._csr_work.numel() < need:
                self._csr_work = torch.empty(need + need // 8 + 16, dtype=torch.int32, device=self.device)
        self.n_cells, self.n_faces = n_cells, n_faces
        self._point_struct()
        return moved

    # --- per-step hand-over of a new tessellation (resize first when its counts differ)
    UPLOAD = (("tag", np.int8), ("type", np.int8), ("map", np.int32), ("x", np.float64),
              ("dcom", np.float64), ("vol", np.float64), ("pair_i", np.int32), ("pair_j", np.int32),
              ("area", np.float64), ("com", np.float64))

    def _check_remesh(self, host):
        nr = self.n_real
        if (host.n_real != nr or not np.array_equal(host.map[:nr], np.arange(nr)) or
                np.any(host.tag[:nr] != 0) or not np.array_equal(host.type[:nr], self._real_type) or
                np.any(host.tag[nr:] != 1) or np.any(host.type[nr:] != 2)):
            raise ValueError("a re-mesh keeps the real cells (same count and order, identity map, tags and "
                             "types) and re-creates the ghosts as Ghost / Exterior rows")

    def pinned_host(self, host=None):
        """Pinned host copies of a host mesh's per-step arrays (the face list and the
        cell geometry a host re-mesh writes, ``mesh.pyx:255-323``).  A re-mesh keeps the
        real cells -- same count and order, identity map, tags and types -- and re-creates
        the ghosts (tagged Ghost, type Exterior); the ghost and face counts may change."""
        host = self.host if host is None else host
        self._check_remesh(host)
        return {nm: torch.from_numpy(np.ascontiguousarray(getattr(host, nm), dtype=dt)).pin_memory()
                for nm, dt in self.UPLOAD}

    def ghost_codes(self, host):
        """How each ghost of ``host`` images its real cell (phd_ghost_positions): a
        periodic shift (sx, sy) -> 1 + 3 (sx + 1) + (sy + 1); a mirror across axis k at
        its low / high wall -> 16 + 2 k + (high)."""
        nr = host.n_real
        g = np.arange(nr, host.n_cells)
        img = host.map[g]
        x = np.asarray(host.x)
        lo, hi = np.asarray(host.xmin, dtype=np.float64), np.asarray(host.xmax, dtype=np.float64)
        d = x[:, g] - x[:, img]
        if host.boundary == "periodic":
            s = np.rint(d / (hi - lo)[:, None]).astype(np.int64)
            code = 1 + 3 * (s[0] + 1) + (s[1] + 1)
        else:
            k = (d[1] != 0.0).astype(np.int64)                 # the mirrored axis
            high = x[k, g] > 0.5 * (lo[k] + hi[k])
            code = 16 + 2 * k + high.astype(np.int64)
        return code.astype(np.int8)

    def pinned_host_compact(self, host, resident=False, pair16=True):
        """The compact hand-over of a re-mesh for the FP32 path, 12 B per face instead of
        32: per-real-cell face ranges ``face_ptr`` instead of pair-i (faces are emitted
        per real cell in ascending order, tess.cpp:363), pair-j, and the area and the
        centroid offset along the face, s = (c . (-dy, dx)) / r with c = com - (x_i +
        x_j)/2, (dx, dy) = x_j - x_i, r = |x_j - x_i| -- formed in FP64 with the device's
        operations, each rounded separately -- rounded once to FP32 (round to nearest even; magnitudes below 2^-126 to signed
        zero, as the device's own rounding does), plus the cells' positions and maps.
        The FP32 face geometry formed from it equals the full hand-over's bit for bit.
        ``resident``: the device already holds the real cells' positions (its own
        generator move); ghost codes replace the positions (``phd_ghost_positions``).
        ``pair16``: pair-j as the 16-bit difference to the owner cell (``pair_dj``, 0 =
        escape) plus the escaped faces' (face id, pair-j) pairs (``pair_x``): 10 B per
        face; each cell's list length (``list_len``, one byte) so the device lays out
        the neighbour lists without counting them; the area and offset interleaved
        (``face32`` [F][2]); and the small arrays back to back in one pinned block
        (``compact_block``), so the hand-over copies them as one."""
        self._check_remesh(host)
        nr = self.n_real
        pi, pj = np.asarray(host.pair_i), np.asarray(host.pair_j)
        if pi.size and (np.any(np.diff(pi) < 0) or pi[0] < 0 or pi[-1] >= nr):
            raise ValueError("faces must be emitted per real cell in ascending cell order")
        face_ptr = np.searchsorted(pi, np.arange(nr + 1)).astype(np.int32)
        x = np.asarray(host.x, dtype=np.float64)
        com = np.asarray(host.com, dtype=np.float64)
        dx, dy = x[0, pj] - x[0, pi], x[1, pj] - x[1, pi]
        cx, cy = com[0] - 0.5 * (x[0, pi] + x[0, pj]), com[1] - 0.5 * (x[1, pi] + x[1, pj])
        r = np.sqrt(dx * dx + dy * dy)
        with np.errstate(divide="ignore", invalid="ignore"):
            s64 = np.where(r > 0.0, (cx * (-dy) + cy * dx) / r, 0.0)

        def round32(a):
            out = a.astype(np.float32)
            return np.where(np.abs(a) < 2.0 ** -126, np.copysign(np.float32(0.0), out), out).astype(np.float32)

        area32, ct32 = round32(np.asarray(host.area, dtype=np.float64)), round32(s64)
        arrays = {"map": np.ascontiguousarray(host.map, dtype=np.int32),
                  "tag": np.ascontiguousarray(host.tag, dtype=np.int8),
                  "type": np.ascontiguousarray(host.type, dtype=np.int8)}
        if resident:            # the device holds the real positions; ghosts from their codes
            ghost_code = self.ghost_codes(host)
        else:
            arrays["x"] = np.ascontiguousarray(x)
        if not pair16:
            arrays.update(face_ptr=face_ptr, pair_j=np.ascontiguousarray(pj, dtype=np.int32), area32=area32,
                          ct32=ct32)
            if resident:
                arrays["ghost_code"] = ghost_code
            return {k: torch.from_numpy(v).pin_memory() for k, v in arrays.items()}
        d = pj.astype(np.int64) - pi.astype(np.int64)
        ok = (d >= 1) & (d <= 65534)
        esc = np.flatnonzero(~ok)
        small = {"face_ptr": face_ptr, "pair_x": np.stack([esc, pj[esc]], axis=1).astype(np.int32).reshape(-1),
                 # the 16-bit patterns as int16 (the device reads them as uint16)
                 "pair_dj": np.where(ok, d, 0).astype(np.uint16).view(np.int16)}
        ln = np.bincount(np.concatenate([pi, pj]).astype(np.int64), minlength=len(host.map))
        if ln.max(initial=0) <= 255:                # else the device counts them
            small["list_len"] = ln.astype(np.uint8)
        if resident:
            small["ghost_code"] = ghost_code
        out = {k: torch.from_numpy(v).pin_memory() for k, v in arrays.items()}
        sizes = {k: v.size for k, v in small.items()}
        layout, nbytes = compact_block_layout(sizes)
        block = torch.empty(max(nbytes, 16), dtype=torch.uint8, pin_memory=True)
        out.update(block_views(block, layout))
        for k, v in small.items():
            out[k].copy_(torch.from_numpy(v))
        out["compact_block"] = block
        out["face32"] = torch.from_numpy(np.stack([area32, ct32], axis=1)).pin_memory()
        return out

    @staticmethod
    def pinned_sizes(pinned):
        """(n_cells, n_faces) of a pinned hand-over (full or compact)."""
        return int(pinned["map"].shape[0]), int((pinned["pair_j"] if "pair_j" in pinned else pinned["pair_dj"]).shape[0])

    def check_upload(self, pinned):
        """Raise unless the pinned arrays have this mesh's cell and face counts."""
        shapes = {"tag": (self.n_cells,), "type": (self.n_cells,), "map": (self.n_cells,),
                  "x": (self.dim, self.n_cells), "dcom": (self.dim, self.n_cells), "vol": (self.n_cells,),
                  "pair_i": (self.n_faces,), "pair_j": (self.n_faces,), "area": (self.n_faces,),
                  "com": (self.dim, self.n_faces), "face_ptr": (self.n_real + 1,), "area32": (self.n_faces,),
                  "ct32": (self.n_faces,), "ghost_code": (self.n_cells - self.n_real,), "pair_dj": (self.n_faces,),
                  "face32": (self.n_faces, 2)}
        if "face_ptr" in pinned:
            names = ("face_ptr", "pair_j" if "pair_j" in pinned else "pair_dj", "map", "tag", "type") + \
                (("face32",) if "face32" in pinned else ("area32", "ct32")) + \
                (("x",) if "x" in pinned else ("ghost_code",))
            if "list_len" in pinned and tuple(pinned["list_len"].shape) != (self.n_cells,):
                raise ValueError("upload: list_len must hold one length per cell")
            if "pair_dj" in pinned:
                px = pinned["pair_x"]
                if px.dim() != 1 or px.numel() % 2 or px.numel() > 2 * self.n_faces:
                    raise ValueError("upload: pair_x must hold (face id, pair-j) pairs of at most n_faces faces")
        else:
            names = [nm for nm, _ in self.UPLOAD]
        for nm in names:
            if tuple(pinned[nm].shape) != shapes[nm]:
                raise ValueError("upload: %s has shape %s, this mesh holds %s" % (nm, tuple(pinned[nm].shape),
                                                                                 shapes[nm]))

    def copy_fields(self, pinned, names, stream=None):
        """Asynchronous host->device copies of the named arrays; returns their bytes."""
        nbytes = 0
        with (torch.cuda.stream(stream) if stream is not None else _nullctx()):
            for nm in names:
                getattr(self, nm).copy_(pinned[nm], non_blocking=True)
                nbytes += pinned[nm].numel() * pinned[nm].element_size()
        return nbytes

    def copy_ghost_map(self, pinned, stream=None):
        """Copy only the ghost part of the image map: real cells keep their order (and
        therefore their identity map, tags and types) across re-meshes, only the ghosts
        are re-created.  Returns the bytes copied."""
        src = pinned["map"][self.n_real:]
        with (torch.cuda.stream(stream) if stream is not None else _nullctx()):
            self.map[self.n_real:].copy_(src, non_blocking=True)
        return src.numel() * src.element_size()

    def reset_errors(self, stream=None):
        lib = L.lib()
        with (torch.cuda.stream(stream) if stream is not None else _nullctx()):
            if not hasattr(self, "_bad"):
                self._bad = torch.zeros(1, dtype=torch.int32, device=self.device)
                self._csr_work = torch.empty(int(lib.phd_csr_work_ints(self.n_cells)), dtype=torch.int32,
                                             device=self.device)
            self._bad.zero_()

    def build_lists(self, stream=None):
        """Neighbour lists from the face pairs on the device (phd_build_csr)."""
        L.check(L.lib().phd_build_csr(self.ref, L.ptr(self.nbr_ptr), L.ptr(self.nbr_idx), L.ptr(self._csr_work),
                                      L.ptr(self._bad), L.stream_handle(stream)), "phd_build_csr")

    def set_flip(self, stream=None):
        xmin = (C.c_double * 3)(*(list(self.xmin) + [0.0] * (3 - self.dim)))
        xmax = (C.c_double * 3)(*(list(self.xmax) + [0.0] * (3 - self.dim)))
        L.check(L.lib().phd_flip_mask(self.dim, self.n_cells, L.ptr(self.type), L.ptr(self.x), xmin, xmax,
                                      int(self.boundary == "reflective"), L.ptr(self.flip),
                                      L.stream_handle(stream)), "phd_flip_mask")

    def set_normals(self, normals, stream=None):
        """"device": FP64 normals formed on the device; "none": the mesh carries no FP64
        normals (FP32 consumers form their own; FP64 entries then refuse the mesh)."""
        if normals == "device":
            self.struct.normal = self.normal.data_ptr()
            L.check(L.lib().phd_face_normals_f64(self.ref, L.ptr(self.normal), L.ptr(self._bad),
                                                 L.stream_handle(stream)), "phd_face_normals_f64")
        elif normals == "none":
            self.struct.normal = None
        else:
            raise ValueError("normals must be 'device' or 'none'")

    def upload(self, pinned, normals="device", stream=None):
        """Hand over a new tessellation with this mesh's cell and face counts (``resize``
        first for other counts).

        Copies the face list (pair-i/j, area, centroid) and the cell geometry (x, dcom,
        vol, tag, type, map) from pinned host buffers, then forms on the device what
        follows from them: the neighbour lists (phd_build_csr), the reflective flip bits
        and, with ``normals="device"``, the FP64 face normals (phd_face_normals_f64).
        ``normals="none"`` leaves the mesh without FP64 normals.  Returns the bytes
        copied."""
        if normals not in ("device", "none"):
            raise ValueError("normals must be 'device' or 'none'")
        self.check_upload(pinned)
        self.reset_errors(stream)
        nbytes = self.copy_fields(pinned, [nm for nm, _ in self.UPLOAD], stream)
        self.build_lists(stream)
        self.set_flip(stream)
        self.set_normals(normals, stream)
        return nbytes

    def upload_errors(self):
        """Faces of the last upload whose cells were out of range (synchronises)."""
        return int(self._bad.item()) if hasattr(self, "_bad") else 0

    def h2d_bytes(self):
        """Bytes of one mesh upload (the per-step host->device face list and geometry)."""
        ts = (self.tag, self.type, self.map, self.x, self.dcom, self.vol, self.pair_i, self.pair_j,
              self.area, self.com, self.normal, self.nbr_ptr, self.nbr_idx)
        return sum(t.numel() * t.element_size() for t in ts)


class DeviceClock:
    """Device ``phd_clock``: dt, t, t_end, CFL accumulator and status bits."""

    def __init__(self, device="cuda", dt=0.0, t=0.0, t_end=0.0):
        self.device = _dev(device)
        self.buf = torch.zeros(L.CLOCK_BYTES, dtype=torch.uint8, device=self.device)
        self.set(dt=dt, t=t, t_end=t_end)

    def set(self, dt=0.0, t=0.0, t_end=0.0, status=0, step=0):
        c = L.PhdClock()
        c.dt, c.t, c.t_end, c.dt_hydro = dt, t, t_end, 0.0
        c.dtmin_bits = np.float64(np.inf).view(np.uint64).item()
        c.arrive, c.status, c.step = 0, status, step
        host = torch.frombuffer(bytearray(bytes(c)), dtype=torch.uint8)
        self.buf.copy_(host)

    def read(self):
        """Copy the clock back to the host (synchronises the current stream)."""
        raw = self.buf.cpu().numpy().tobytes()
        return L.PhdClock.from_buffer_copy(raw)

    @property
    def ptr(self):
        return C.c_void_p(self.buf.data_ptr())

    def check_status(self):
        st = self.read().status
        L.raise_status(st)
        return st


def make_params(gamma=1.4, cfl=0.5, eta=0.25, reconstruction="linear", limiter="arepo",
                gizmo=True, solver="hllc", boost=True, regularize=True, exact_max_iter=1000):
    p = L.PhdParams()
    p.gamma, p.cfl, p.eta = float(gamma), float(cfl), float(eta)
    p.reconstruction = L.LINEAR if reconstruction in ("linear", L.LINEAR) else L.CONSTANT
    p.limiter = {"arepo": L.LIMITER_AREPO, "tess": L.LIMITER_TESS}.get(limiter, limiter)
    p.gizmo = int(bool(gizmo))
    p.solver = {"hll": L.HLL, "hllc": L.HLLC, "exact": L.EXACT}.get(solver, solver)
    p.boost = 1 if p.solver == L.EXACT else int(bool(boost))
    p.regularize = int(bool(regularize))
    p.exact_max_iter = int(exact_max_iter)
    return p
