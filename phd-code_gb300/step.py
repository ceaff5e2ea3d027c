"""Fused device step of the flux path, with optional CUDA-graph replay.

``FluxStepper`` keeps one mesh and one state resident in HBM and advances it by whole
steps, each a short fixed sequence of kernel launches that needs no host round trip:
the time step lives on the device (``phd_clock``), is produced by the CFL reduction at
the end of each step and consumed by the next one.  The step follows
``MovingMeshMUSCLHancock.evolve_timestep`` (``integrate.py:385-428``) up to the host
re-mesh, or ``StaticMeshMUSCLHancock.evolve_timestep`` (``integrate.py:349-378``).

Precision ``"fp64"`` is the parity mode (reference arithmetic); ``"fp32"`` runs
reconstruction and Riemann fluxes in FP32 with FP64 conserved-state accumulation.
"""
import ctypes

import numpy as np
import torch

from . import _lib as L
from .device import DeviceClock, DeviceMesh, make_params
from .twins import periodic_twins


class FluxStepper:
    def __init__(self, mesh, prim, gamma=1.4, cfl=0.5, solver="hllc", reconstruction="linear",
                 limiter="arepo", gizmo=True, boost=True, moving=True, regularize=True, eta=0.25,
                 precision="fp64", t_end=0.0, face_velocity=None, device="cuda", stream=None,
                 dedup_periodic=True, handover_records=False):
        """handover_records (FP32): whether load_mesh also writes the per-entry gradient
        records (entry_rec).  Without them the first steps on a handed-over mesh form
        each entry's record from its face in the gradient kernel (the same bits); that
        is cheaper for a mesh stepped once, as in the moving-mesh loop, while
        build_entry_records() (called by capture()) pays off over many steps."""
        self.device = torch.device(device)
        self.handover_records = bool(handover_records)
        self.records = False        # entry_rec holds the current mesh's records
        self.dmesh = mesh if isinstance(mesh, DeviceMesh) else DeviceMesh(mesh, device=self.device)
        dm = self.dmesh
        self.params = make_params(gamma=gamma, cfl=cfl, eta=eta, reconstruction=reconstruction,
                                  limiter=limiter, gizmo=gizmo, solver=solver, boost=boost,
                                  regularize=regularize)
        self.moving = bool(moving)
        if precision not in ("fp64", "fp32"):
            raise ValueError("precision must be 'fp64' or 'fp32'")
        self.precision = precision
        self.stream = stream
        self.dedup_periodic = bool(dedup_periodic)
        self.launch = None          # FP32 launch shapes (PhdLaunch, e.g. from autotune.tune)
        n, F, d = dm.n_cells, dm.n_faces, dm.dim
        nf = d + 2
        dev = self.device
        f64 = torch.float64
        self.prim = torch.as_tensor(np.ascontiguousarray(prim, dtype=np.float64)).to(dev).contiguous()
        if tuple(self.prim.shape) != (nf, n):
            raise ValueError("prim must be [%d][%d]" % (nf, n))
        self.cons = torch.empty((nf, n), dtype=f64, device=dev)
        self.cons_next = torch.empty((nf, n), dtype=f64, device=dev)
        self.clock = DeviceClock(dev, t_end=t_end)
        self._graph = None
        self._graph_steps = 0
        s = L.stream_handle(stream)
        lib = L.lib()
        L.check(lib.phd_cons_from_prim_f64(d, n, self.params.gamma, L.ptr(dm.vol), L.ptr(self.prim),
                                           L.ptr(self.cons), s), "phd_cons_from_prim_f64")
        if precision == "fp64":
            self.grad = torch.zeros((nf * d, n), dtype=f64, device=dev)
            self.w = torch.zeros((d, n), dtype=f64, device=dev)
            if face_velocity is None:
                self.face_w = torch.zeros((d, F), dtype=f64, device=dev)
            else:
                self.face_w = torch.as_tensor(np.ascontiguousarray(face_velocity, dtype=np.float64)).to(dev)
            self.flux = torch.zeros((nf, max(F, 1)), dtype=f64, device=dev)
            self.initial_time_step()
        else:
            if face_velocity is not None:
                raise ValueError("fp32 steps form face velocities on the device (moving=True)")
            f32 = torch.float32
            self.twin = torch.as_tensor(periodic_twins(dm.host) if dedup_periodic else
                                        np.full(F, -1, np.int32)).to(dev)
            self.face_geo = torch.zeros((max(F, 1), 4), dtype=f32, device=dev)
            self.face_ar = torch.zeros((max(F, 1), 2), dtype=f32, device=dev)
            self.csr_face = torch.zeros(max(2 * F, 1), dtype=torch.int32, device=dev)
            self.csr_nbr = torch.zeros(max(2 * F, 1), dtype=torch.int32, device=dev)
            self.cell_geo = torch.zeros((n, 4), dtype=f32, device=dev)
            self.entry_rec = torch.zeros((max(2 * F, 1), 4), dtype=f32, device=dev)
            out = L.geom32(self._geo_tensors(), out=True)
            L.check(lib.phd_prepare_f32(dm.ref, L.ptr(self.twin), ctypes.byref(out), s), "phd_prepare_f32")
            self.records = True
            self._set_geo()
            self.prim4 = torch.zeros((n, 4), dtype=f32, device=dev)
            self.cellrec = torch.zeros((n, 16), dtype=f32, device=dev)
            self.w2 = torch.zeros((n, 2), dtype=f32, device=dev)
            self.flux4 = torch.zeros((max(F, 1), 4), dtype=f32, device=dev)
            L.check(lib.phd_prim_f32(dm.ref, ctypes.byref(self.params), L.ptr(self.cons), L.ptr(self.prim4),
                                     self.clock.ptr, s), "phd_prim_f32")

    # ------------------------------------------------------------------------------
    def _geo_tensors(self, records=True):
        return (self.face_geo, self.face_ar, self.csr_face, self.csr_nbr, self.cell_geo,
                self.entry_rec if records else None)

    def _set_geo(self):
        """The step's geometry: with entry_rec only while it holds the current mesh's."""
        self.geo = L.geom32(self._geo_tensors(self.records))

    def build_entry_records(self):
        """(FP32) Write the per-entry gradient records of the current mesh, so the steps
        that follow read them instead of forming them from the faces (the same bits,
        about 8 us less per step at 1M cells; the build costs about as much as 7 steps
        save).  A no-op when they are current."""
        if self.precision != "fp32" or self.records:
            return
        out = L.geom32(self._geo_tensors(), out=True)
        L.check(L.lib().phd_prepare_f32_parts(self.dmesh.ref, None, ctypes.byref(out), L.PREP_RECORDS,
                                              L.stream_handle(self.stream)), "phd_prepare_f32_parts")
        self.records = True
        self._set_geo()

    @property
    def grad8(self):
        """FP32 limited gradients [n][8] (d/dx, d/dy of rho, v_x, v_y, p) of the last step:
        a view into the cell records the gradient stage writes."""
        return self.cellrec[:, 4:12]

    def initial_time_step(self):
        """dt for the first step from the current primitives (riemann.pyx:120-188)."""
        p = self.params
        L.check(L.lib().phd_time_step_f64(self.dmesh.ref, L.ptr(self.prim), p.gamma, p.cfl, p.boost, 0,
                                          self.clock.ptr, L.stream_handle(self.stream)), "phd_time_step_f64")

    def _view(self, name, shape, dtype):
        """``shape`` view of the named array's storage, which grows (1/8 headroom) when
        too small; the contents are undefined after growth."""
        if not hasattr(self, "_store"):
            self._store = {}
        need = int(np.prod(shape))
        store = self._store.get(name)
        if store is None and hasattr(self, name):
            store = getattr(self, name).reshape(-1)
        if store is None or store.numel() < need:
            store = torch.empty(need + need // 8 + 16, dtype=dtype, device=self.device)
        self._store[name] = store
        return store[:need].view(shape)

    def _resize(self, n_cells, n_faces):
        """Re-shape the mesh and every state / work array for new ghost and face counts.
        The real cells' conserved totals are carried over (their rows are re-strided
        through the second buffer); everything else is recomputed by the hand-over.
        A captured CUDA graph no longer matches and is dropped."""
        dm = self.dmesh
        nr, d = dm.n_real, dm.dim
        nf = d + 2
        F1 = max(n_faces, 1)
        old_cons = self.cons
        dm.resize(n_cells, n_faces)
        view = self._view

        f64, f32, i32 = torch.float64, torch.float32, torch.int32
        # the two conserved-state buffers swap every step: find which storage holds the
        # current state, re-stride its real rows into the other one
        stores = getattr(self, "_cons_stores", None) or [self.cons.reshape(-1), self.cons_next.reshape(-1)]
        a, b = stores if stores[0].data_ptr() == old_cons.data_ptr() else stores[::-1]
        need = nf * n_cells
        if b.numel() < need:
            b = torch.empty(need + need // 8 + 16, dtype=f64, device=self.device)
        nxt = b[:need].view(nf, n_cells)
        for q in range(nf):
            nxt[q, :nr].copy_(old_cons[q, :nr])
        if a.numel() < need:
            a = torch.empty(need + need // 8 + 16, dtype=f64, device=self.device)
        self.cons, self.cons_next = nxt, a[:need].view(nf, n_cells)
        self._cons_stores = [b, a]
        if self.precision == "fp64":
            self.prim = view("prim", (nf, n_cells), f64)
            self.grad = view("grad", (nf * d, n_cells), f64)
            self.w = view("w", (d, n_cells), f64)
            self.face_w = view("face_w", (d, n_faces), f64)
            if not self.moving:
                self.face_w.zero_()
            self.flux = view("flux", (nf, F1), f64)
        else:
            self.twin = view("twin", (n_faces,), i32)
            self.face_geo = view("face_geo", (F1, 4), f32)
            self.face_ar = view("face_ar", (F1, 2), f32)
            self.csr_face = view("csr_face", (max(2 * n_faces, 1),), i32)
            self.csr_nbr = view("csr_nbr", (max(2 * n_faces, 1),), i32)
            self.cell_geo = view("cell_geo", (n_cells, 4), f32)
            self.entry_rec = view("entry_rec", (max(2 * n_faces, 1), 4), f32)
            self.prim4 = view("prim4", (n_cells, 4), f32)
            self.cellrec = view("cellrec", (n_cells, 16), f32)
            self.w2 = view("w2", (n_cells, 2), f32)
            self.flux4 = view("flux4", (F1, 4), f32)
            self.records = False
            self._set_geo()
        self._graph = None
        self._graph_steps = 0

    def load_mesh(self, pinned):
        """Continue on a new tessellation handed over from pinned host buffers
        (``DeviceMesh.pinned_host`` layout), as after the host re-mesh of
        ``integrate.py:410-417``: the real cells keep their order, tags, types and
        identity map; the ghosts are re-created and their number, like the number of
        faces, may change -- the arrays are then re-shaped (``_resize``) and the tags,
        types and whole map copied, otherwise only the ghost part of the map is.

        The device forms the neighbour lists, flip bits and, for FP32, the periodic twin
        table and FP32 geometry (normals, cell volumes and centroids included, so FP32
        copies neither); FP64 forms its FP64 normals.  The
        ghosts are re-created from their images (``domain_manager.pyx:712-774``), the
        primitives recovered with the new volumes and the next dt taken from them
        (steps 6-8 of the moving-mesh step).  The neighbour lists, twin table, FP32 list
        codes and face geometry are formed on a second stream while the rest of the mesh
        is still being copied.  ``pinned`` is either the full hand-over
        (``DeviceMesh.pinned_host``) or, for FP32 steppers, the compact one
        (``DeviceMesh.pinned_host_compact`` / ``tess.CompactMesher``: 12 B per face, pair-i
        from per-cell face ranges); a compact hand-over without positions keeps the real
        cells' positions on the device -- the last generator move's (``move_generators``)
        or the current ones -- and forms the ghosts' from their codes
        (``phd_ghost_positions``).  Returns the bytes copied."""
        dm, p = self.dmesh, self.params
        main = self.stream if self.stream is not None else torch.cuda.current_stream(self.device)
        resident = "x" not in pinned          # positions stay on the device (ghost codes come instead)
        if resident:
            with torch.cuda.stream(main):
                xr = self._real_positions()
        n_new, f_new = dm.pinned_sizes(pinned)
        resized = (n_new, f_new) != (dm.n_cells, dm.n_faces)
        if resized:
            main.synchronize()            # storage may be released: nothing may still read it
            with torch.cuda.stream(main):
                self._resize(n_new, f_new)
        dm.check_upload(pinned)
        lib = L.lib()
        fp32 = self.precision == "fp32"
        compact = "face_ptr" in pinned
        if compact and not fp32:
            raise ValueError("the compact hand-over carries FP32 face geometry: FP32 steppers only")
        if getattr(self, "_side", None) is None:
            self._side = torch.cuda.Stream(self.device)
            self._side2 = torch.cuda.Stream(self.device)
            self._ev = [torch.cuda.Event() for _ in range(8)]
            for e in self._ev:                        # creates the events' handles
                e.record(main)
        side, ev = self._side, self._ev
        if compact:
            return self._load_mesh_compact(pinned, resized, xr if resident else None, main)
        s, ss = L.stream_handle(main), L.stream_handle(side)
        out = None
        if fp32:
            out = L.geom32(self._geo_tensors(self.handover_records), out=True)
        # copies on the main stream in the order the side stream needs them; the side
        # stream builds the neighbour lists, twins, list codes and face geometry meanwhile
        dm.reset_errors(main)
        nbytes = dm.copy_fields(pinned, ("pair_i", "pair_j"), main)
        ev[0].record(main)
        side.wait_event(ev[0])
        dm.build_lists(side)
        if resized:
            nbytes += dm.copy_fields(pinned, ("tag", "type", "map"), main)
        else:
            nbytes += dm.copy_ghost_map(pinned, main)
        nbytes += dm.copy_fields(pinned, ("x",), main)
        self._x_real_valid = False
        ev[1].record(main)
        if fp32:
            side.wait_event(ev[1])
            box = [b - a for a, b in zip(dm.xmin, dm.xmax)]
            L.check(lib.phd_periodic_twins(dm.ref, int(self.dedup_periodic and dm.boundary == "periodic"),
                                           float(box[0]), float(box[1]), L.ptr(self.twin), ss),
                    "phd_periodic_twins")
            L.check(lib.phd_prepare_f32_parts(dm.ref, L.ptr(self.twin), ctypes.byref(out), L.PREP_LISTS, ss),
                    "phd_prepare_f32_parts")
        nbytes += dm.copy_fields(pinned, ("com", "area"), main)
        if fp32:
            # face geometry, then the cells' volumes and centroids from it (the FP32 path
            # needs neither host volumes nor host centroids)
            ev[2].record(main)
            side.wait_event(ev[2])
            dm.set_normals("none", side)
            L.check(lib.phd_prepare_f32_parts(dm.ref, None, ctypes.byref(out), L.PREP_FACES | L.PREP_CELLS_FROM_FACES |
                                              (L.PREP_RECORDS if self.handover_records else 0), ss),
                    "phd_prepare_f32_parts")
        ev[3].record(side)
        if not fp32:
            nbytes += dm.copy_fields(pinned, ("dcom", "vol"), main)
        dm.set_flip(main)
        main.wait_event(ev[3])
        L.check(lib.phd_ghost_cons_f64(dm.ref, L.ptr(self.cons), s), "phd_ghost_cons_f64")
        if fp32:
            L.check(lib.phd_prim_f32_cells(dm.ref, L.ptr(self.cell_geo), ctypes.byref(p), L.ptr(self.cons),
                                           L.ptr(self.prim4), self.clock.ptr, s), "phd_prim_f32_cells")
        else:
            dm.set_normals("device", main)
            L.check(lib.phd_prim_from_cons_f64(dm.dim, dm.n_cells, p.gamma, L.ptr(dm.vol), L.ptr(self.cons),
                                               L.ptr(self.prim), s), "phd_prim_from_cons_f64")
            self.initial_time_step()
        if fp32:
            self.records = self.handover_records
            self._set_geo()
        return nbytes

    def _load_mesh_compact(self, pinned, resized, xr, main):
        """load_mesh for the compact FP32 hand-over as one C call (phd_load_mesh_f32):
        the copies on the main stream, the derivations on two side streams while the
        face records are in flight.  xr: the real cells' device positions when the
        hand-over carries none."""
        dm, lib = self.dmesh, L.lib()
        nr, ng, nf = dm.n_real, dm.n_cells - dm.n_real, dm.n_faces
        nbytes = 0
        if resized:                                   # tags, types and the whole map are new
            nbytes += dm.copy_fields(pinned, ("tag", "type", "map"), main)
        if not hasattr(dm, "_bad"):
            dm.reset_errors(main)
        packed = "pair_dj" in pinned
        n_x = pinned["pair_x"].numel() // 2 if packed else 0
        small = [k for k in ("pair_x", "face_ptr", "pair_dj", "list_len", "ghost_code")
                 if k in pinned and pinned[k].numel() > 0]
        if xr is None and "ghost_code" in small:
            small.remove("ghost_code")
        stage = {}
        if "compact_block" in pinned:
            # a staging block laid out like the host block: adjacent arrays go over as one copy
            hb = pinned["compact_block"]
            db = self._view("compact_block_in", (hb.numel(),), torch.uint8)
            for k in small:
                off = pinned[k].data_ptr() - hb.data_ptr()
                if not 0 <= off <= hb.numel() - pinned[k].numel() * pinned[k].element_size():
                    raise ValueError("upload: %s lies outside compact_block" % k)
                stage[k] = db.data_ptr() + off
        else:
            for k in small:
                t = pinned[k]
                stage[k] = self._view(k + "_in", (max(t.numel(), 1),), t.dtype).data_ptr()
        if "face32" in pinned:
            stage["face32"] = self._view("face32_in", (nf, 2), torch.float32).data_ptr()
        else:
            stage["area32"] = self._view("area32_in", (nf,), torch.float32).data_ptr()
            stage["ct32"] = self._view("ct32_in", (nf,), torch.float32).data_ptr()
        dm.set_normals("none")
        hp = lambda k: pinned[k].data_ptr() if k in pinned else None
        h = L.PhdHandover32(face_ptr=hp("face_ptr"), pair_j=hp("pair_j"), area32=hp("area32"), ct32=hp("ct32"),
                            ghost_map=None if resized else pinned["map"][nr:].data_ptr(),
                            ghost_code=hp("ghost_code") if xr is not None else None,
                            x=None if xr is not None else hp("x"),
                            x_real=xr.data_ptr() if xr is not None else None, type=dm.type.data_ptr(),
                            d_face_ptr=stage["face_ptr"], d_area32=stage.get("area32"), d_ct32=stage.get("ct32"),
                            d_ghost_code=stage.get("ghost_code"),
                            twin=self.twin.data_ptr(), csr_work=dm._csr_work.data_ptr(), bad=dm._bad.data_ptr(),
                            periodic=int(dm.boundary == "periodic"), dedup_periodic=int(self.dedup_periodic),
                            xmin=(ctypes.c_double * 2)(*dm.xmin[:2]),
                            xmax=(ctypes.c_double * 2)(*dm.xmax[:2]),
                            pair_dj=hp("pair_dj"), pair_x=hp("pair_x") if n_x else None, n_pair_x=n_x,
                            d_pair_dj=stage.get("pair_dj"), d_pair_x=stage.get("pair_x"),
                            list_len=hp("list_len"), d_list_len=stage.get("list_len"),
                            face32=hp("face32"), d_face32=stage.get("face32"))
        out = L.geom32(self._geo_tensors(self.handover_records), out=True)
        events = (ctypes.c_void_p * 8)(*(e.cuda_event for e in self._ev))
        sides = (ctypes.c_void_p * 2)(self._side.cuda_stream, self._side2.cuda_stream)
        L.check(lib.phd_load_mesh_f32(dm.ref, ctypes.byref(h), ctypes.byref(self.params), ctypes.byref(out),
                                      L.ptr(self.cons), L.ptr(self.prim4), self.clock.ptr, L.stream_handle(main),
                                      sides, events), "phd_load_mesh_f32")
        if xr is None:
            self._x_real_valid = False
        self.records = self.handover_records
        self._set_geo()
        # what phd_load_mesh_f32 copied, counted from the arrays themselves
        nb = lambda k: pinned[k].numel() * pinned[k].element_size()
        pair_bytes = nb("pair_dj") + nb("pair_x") if packed else nb("pair_j")
        pair_bytes += nb("list_len") if "list_len" in pinned else 0
        face_bytes = nb("face32") if "face32" in pinned else nb("area32") + nb("ct32")
        nbytes += nb("face_ptr") + pair_bytes + face_bytes + (0 if resized else 4 * ng)
        nbytes += nb("ghost_code") if xr is not None else nb("x")
        return nbytes

    def _launch_step(self, marks=None):
        """One step; marks: optional array of four CUDA events recorded at the stage
        boundaries (before gradients, before faces, before the update, after it)."""
        dm, p = self.dmesh, self.params
        s = L.stream_handle(self.stream)
        if self.precision == "fp64":
            rc = L.lib().phd_step_f64_marked(dm.ref, ctypes.byref(p), int(self.moving), L.ptr(self.prim),
                                             L.ptr(self.cons), L.ptr(self.cons_next), L.ptr(self.grad),
                                             L.ptr(self.w), L.ptr(self.face_w), L.ptr(self.flux), self.clock.ptr, s,
                                             marks)
        else:
            lch = ctypes.byref(self.launch) if self.launch is not None else None
            rc = L.lib().phd_step_f32_batched(dm.ref, ctypes.byref(self.geo), ctypes.byref(p), int(self.moving), lch,
                                              L.ptr(self.prim4), L.ptr(self.cons), L.ptr(self.cons_next),
                                              L.ptr(self.cellrec), L.ptr(self.w2), L.ptr(self.flux4), self.clock.ptr,
                                              1, None, s, marks)
        L.check(rc, "phd_step_" + self.precision)
        self.cons, self.cons_next = self.cons_next, self.cons

    def step_and_fetch(self, host_w):
        """One step whose generator velocities (w2 [n][2] FP32, or w [2][n] FP64) are
        copied into the pinned host buffer ``host_w`` as soon as the step's first stage
        has formed them, on a copy stream that overlaps the rest of the step -- what the
        host needs for the next re-mesh (integrate.py:410-417), without waiting for the
        flux and update kernels.  Returns the copy's CUDA event; ``host_w`` holds the
        velocities once it has completed.  Later work on the stepper's stream waits for
        the copy (the next step overwrites the velocities)."""
        if not self.moving:
            raise RuntimeError("generator velocities exist only in moving-mesh steps")
        main = self.stream if self.stream is not None else torch.cuda.current_stream(self.device)
        if getattr(self, "_fetch", None) is None:
            evs = [torch.cuda.Event() for _ in range(4)]
            for e in evs:                              # creates the events' handles
                e.record(main)
            self._fetch = (torch.cuda.Stream(self.device), evs, torch.cuda.Event())
        copy_stream, evs, done = self._fetch
        w = self.w2 if self.precision == "fp32" else self.w
        self._launch_step(marks=(ctypes.c_void_p * 4)(*(e.cuda_event for e in evs)))
        copy_stream.wait_event(evs[1])                 # recorded after the gradient stage
        with torch.cuda.stream(copy_stream):
            host_w.copy_(w, non_blocking=True)
            done.record(copy_stream)
        main.wait_event(done)
        return done

    def move_generators(self):
        """DomainManager.move_generators + migrate_particles (domain_manager.pyx:566-590,
        boundary.pyx:236-263, 502-538) on the device after a moving step: x + dt * w for the
        real cells with the step's dt and generator velocities, wrapped into a periodic box
        or flagged (PHD_STATUS_LEFT_DOMAIN, raised by check_status) when a generator leaves
        a reflective one.  Returns the [2][n_real] FP64 positions (a device tensor, reused
        by the next call) -- what the host re-tessellation needs."""
        if not self.moving:
            raise RuntimeError("generator velocities exist only in moving-mesh steps")
        dm = self.dmesh
        out = self._view("x_moved", (dm.dim, dm.n_real), torch.float64)
        w2, w = (self.w2, None) if self.precision == "fp32" else (None, self.w)
        L.check(L.lib().phd_move_generators(dm.ref, L.ptr(w2), L.ptr(w), self.clock.ptr,
                                            int(dm.boundary == "periodic"), float(dm.xmin[0]), float(dm.xmin[1]),
                                            float(dm.xmax[0]), float(dm.xmax[1]), L.ptr(out),
                                            L.stream_handle(self.stream)), "phd_move_generators")
        self._x_real_valid = True
        return out

    def _real_positions(self):
        """The [2][n_real] positions of the real cells the next hand-over starts from: the
        last generator move's, else (copied once) the mesh's own."""
        dm = self.dmesh
        out = self._view("x_moved", (dm.dim, dm.n_real), torch.float64)
        if not getattr(self, "_x_real_valid", False):
            for k in range(dm.dim):
                out[k].copy_(dm.x[k, :dm.n_real])
            self._x_real_valid = True
        return out

    def step(self, n=1):
        """Launch n steps (asynchronous; read the clock or state to synchronise)."""
        for _ in range(n):
            self._launch_step()

    def capture(self, n_steps=2):
        """Record n_steps (even, so the double-buffered conserved state returns to the
        same buffer) into a CUDA graph; replay() then launches them as one unit."""
        if n_steps % 2:
            raise ValueError("capture an even number of steps")
        self.build_entry_records()                 # a graph replays many steps on one mesh
        torch.cuda.synchronize(self.device)
        g = torch.cuda.CUDAGraph()
        cap_stream = torch.cuda.Stream(self.device)
        saved = self.stream
        with torch.cuda.graph(g, stream=cap_stream):
            self.stream = cap_stream
            for _ in range(n_steps):
                self._launch_step()
        self.stream = saved
        self._graph = g
        self._graph_steps = n_steps
        return g

    def replay(self):
        self._graph.replay()

    # ------------------------------------------------------------------------------
    def read_clock(self):
        return self.clock.read()

    def check_status(self):
        return self.clock.check_status()

    def prim_host(self):
        if self.precision == "fp32":
            return self.prim4.double().t().contiguous().cpu().numpy()
        return self.prim.double().cpu().numpy()

    def cons_host(self):
        return self.cons.double().cpu().numpy()
