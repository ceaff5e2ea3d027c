"""Many independent runs advanced together: one launch per stage for all of them.

The runs' meshes are concatenated into one block-diagonal mesh -- all real cells
(run by run), then all ghosts (run by run), faces run by run -- so the FP32 step
kernels sweep every run in the same persistent launch; each cell carries its run id
and each run keeps its own clock (time step from its own CFL minimum, its own time).
``EnsembleStepper.capture`` records steps into a CUDA graph.  ``SequentialEnsemble``
is the baseline: one single-run stepper per run, launched one run after another.
"""
import ctypes

import numpy as np
import torch

from . import _lib as L
from .device import DeviceMesh, make_params
from .meshgen import HostMesh

F64 = torch.float64
F32 = torch.float32


def concatenate(meshes):
    """One HostMesh holding every run: reals of all runs first, then their ghosts.
    Returns (mesh, cell_run, real_off, ghost_off)."""
    nr = np.array([m.n_real for m in meshes])
    ng = np.array([m.n_ghost for m in meshes])
    real_off = np.concatenate([[0], np.cumsum(nr)])
    ghost_off = real_off[-1] + np.concatenate([[0], np.cumsum(ng)])
    n_total = int(ghost_off[-1])

    def newidx(r, m):
        idx = np.empty(m.n_cells, dtype=np.int64)
        idx[:m.n_real] = real_off[r] + np.arange(m.n_real)
        idx[m.n_real:] = ghost_off[r] + np.arange(m.n_ghost)
        return idx

    x = np.zeros((2, n_total))
    dcom = np.zeros((2, n_total))
    vol = np.zeros(n_total)
    tag = np.zeros(n_total, np.int8)
    typ = np.zeros(n_total, np.int8)
    mp = np.zeros(n_total, np.int32)
    cell_run = np.zeros(n_total, np.int32)
    pi_l, pj_l, area_l, com_l, nrm_l = [], [], [], [], []
    lists = [None] * n_total
    f_off = 0
    for r, m in enumerate(meshes):
        ni = newidx(r, m)
        x[:, ni] = m.x
        dcom[:, ni] = m.dcom
        vol[ni] = m.vol
        tag[ni] = m.tag
        typ[ni] = m.type
        mp[ni] = ni[m.map]
        cell_run[ni] = r
        pi_l.append(ni[m.pair_i])
        pj_l.append(ni[m.pair_j])
        area_l.append(m.area)
        com_l.append(m.com)
        nrm_l.append(m.normal)
        for c in range(m.n_cells):
            lists[ni[c]] = m.nbr_idx[m.nbr_ptr[c]:m.nbr_ptr[c + 1]] + f_off
        f_off += m.n_faces
    cnt = np.array([len(l) for l in lists])
    nbr_ptr = np.concatenate([[0], np.cumsum(cnt)]).astype(np.int32)
    nbr_idx = np.concatenate(lists).astype(np.int32)
    mesh = HostMesh(dim=2, n_real=int(real_off[-1]), x=x, tag=tag, type=typ, map=mp, vol=vol, dcom=dcom,
                    pair_i=np.concatenate(pi_l).astype(np.int32), pair_j=np.concatenate(pj_l).astype(np.int32),
                    area=np.concatenate(area_l), com=np.concatenate(com_l, axis=1),
                    normal=np.concatenate(nrm_l, axis=1), nbr_ptr=nbr_ptr, nbr_idx=nbr_idx,
                    xmin=meshes[0].xmin, xmax=meshes[0].xmax, boundary=meshes[0].boundary)
    return mesh, cell_run, real_off, ghost_off


class EnsembleStepper:
    """FP32 step (FP64 totals) over all runs at once; per-run clocks."""

    def __init__(self, runs, gamma=1.4, cfl=0.5, solver="hllc", moving=True, device="cuda", launch=None):
        meshes = [m for m, _ in runs]
        if any(m.boundary != meshes[0].boundary or m.xmin != meshes[0].xmin or m.xmax != meshes[0].xmax
               for m in meshes):
            raise ValueError("all runs of an ensemble share the box and boundary type")
        if meshes[0].boundary == "periodic":
            raise ValueError("ensembles use reflective boxes (periodic twin pairing is per run)")
        self.device = torch.device(device)
        host, cell_run, self.real_off, self.ghost_off = concatenate(meshes)
        self.host = host
        self.n_runs = len(runs)
        self.run_faces = np.array([m.n_faces for m in meshes])
        dev = self.device
        self.dmesh = DeviceMesh(host, device=dev)
        dm = self.dmesh
        n, F = dm.n_cells, dm.n_faces
        prim = np.zeros((4, n))
        for r, (m, p) in enumerate(runs):
            prim[:, self.real_off[r]:self.real_off[r + 1]] = p[:, :m.n_real]
            prim[:, self.ghost_off[r]:self.ghost_off[r + 1]] = p[:, m.n_real:]
        self.params = make_params(gamma=gamma, cfl=cfl, solver=solver)
        self.moving = bool(moving)
        self.cell_run = torch.as_tensor(cell_run).to(dev)
        self.clocks = torch.zeros((self.n_runs, L.CLOCK_BYTES), dtype=torch.uint8, device=dev)
        c = L.PhdClock()
        c.dtmin_bits = np.float64(np.inf).view(np.uint64).item()
        one = torch.frombuffer(bytearray(bytes(c)), dtype=torch.uint8)
        self.clocks.copy_(one.expand(self.n_runs, -1))
        s = L.stream_handle()
        lib = L.lib()
        p64 = torch.as_tensor(prim).to(dev)
        self.cons = torch.empty((4, n), dtype=F64, device=dev)
        self.cons_next = torch.empty_like(self.cons)
        L.check(lib.phd_cons_from_prim_f64(2, n, self.params.gamma, L.ptr(dm.vol), L.ptr(p64), L.ptr(self.cons), s),
                "cons")
        twin = torch.full((max(F, 1),), -1, dtype=torch.int32, device=dev)
        self.face_geo = torch.zeros((max(F, 1), 4), dtype=F32, device=dev)
        self.face_ar = torch.zeros((max(F, 1), 2), dtype=F32, device=dev)
        self.csr_face = torch.zeros(max(2 * F, 1), dtype=torch.int32, device=dev)
        self.csr_nbr = torch.zeros(max(2 * F, 1), dtype=torch.int32, device=dev)
        self.cell_geo = torch.zeros((n, 4), dtype=F32, device=dev)
        self.entry_rec = torch.zeros((max(2 * F, 1), 4), dtype=F32, device=dev)
        geo = (self.face_geo, self.face_ar, self.csr_face, self.csr_nbr, self.cell_geo, self.entry_rec)
        out = L.geom32(geo, out=True)
        L.check(lib.phd_prepare_f32(dm.ref, L.ptr(twin), ctypes.byref(out), s), "prepare")
        self.geo = L.geom32(geo)
        self.prim4 = torch.zeros((n, 4), dtype=F32, device=dev)
        self.cellrec = torch.zeros((n, 16), dtype=F32, device=dev)
        self.w2 = torch.zeros((n, 2), dtype=F32, device=dev)
        self.flux4 = torch.zeros((max(F, 1), 4), dtype=F32, device=dev)
        L.check(lib.phd_prim_f32_batched(dm.ref, ctypes.byref(self.params), L.ptr(self.cons), L.ptr(self.prim4),
                                         L.ptr(self.clocks), self.n_runs, L.ptr(self.cell_run), s), "prim")
        self.launch = launch
        self._graph = None

    def _launch_step(self, stream=None, marks=None):
        s = L.stream_handle(stream)
        lch = ctypes.byref(self.launch) if self.launch is not None else None
        rc = L.lib().phd_step_f32_batched(self.dmesh.ref, ctypes.byref(self.geo), ctypes.byref(self.params),
                                          int(self.moving), lch, L.ptr(self.prim4), L.ptr(self.cons),
                                          L.ptr(self.cons_next), L.ptr(self.cellrec), L.ptr(self.w2),
                                          L.ptr(self.flux4), L.ptr(self.clocks), self.n_runs, L.ptr(self.cell_run),
                                          s, marks)
        L.check(rc, "phd_step_f32_batched")
        self.cons, self.cons_next = self.cons_next, self.cons

    def step(self, n=1):
        for _ in range(n):
            self._launch_step()

    def capture(self, n_steps=2):
        if n_steps % 2:
            raise ValueError("capture an even number of steps")
        torch.cuda.synchronize(self.device)
        g = torch.cuda.CUDAGraph()
        cs = torch.cuda.Stream(self.device)
        with torch.cuda.graph(g, stream=cs):
            for _ in range(n_steps):
                self._launch_step(stream=cs)
        self._graph = g
        return g

    def replay(self):
        self._graph.replay()

    def read_clocks(self):
        raw = self.clocks.cpu().numpy()
        return [L.PhdClock.from_buffer_copy(raw[r].tobytes()) for r in range(self.n_runs)]

    def check_status(self):
        st = 0
        for c in self.read_clocks():
            st |= c.status
        L.raise_status(st)
        return st

    def run_cons(self, r):
        """Conserved totals of run r's real cells [4][n_real_r] (host)."""
        return self.cons[:, self.real_off[r]:self.real_off[r + 1]].double().cpu().numpy()

    def run_prim(self, r):
        return self.prim4[self.real_off[r]:self.real_off[r + 1]].double().t().cpu().numpy()

    @property
    def faces(self):
        return self.dmesh.n_faces


class SequentialEnsemble:
    """The baseline: the same runs as separate single-run steppers, launched in turn."""

    def __init__(self, runs, gamma=1.4, cfl=0.5, solver="hllc", moving=True, device="cuda"):
        from .step import FluxStepper
        self.steppers = [FluxStepper(m, p, gamma=gamma, cfl=cfl, solver=solver, moving=moving, precision="fp32",
                                     device=device) for m, p in runs]

    def step(self, n=1):
        for _ in range(n):
            for st in self.steppers:
                st.step(1)

    @property
    def faces(self):
        return sum(st.dmesh.n_faces for st in self.steppers)
