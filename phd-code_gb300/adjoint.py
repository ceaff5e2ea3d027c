"""Hand-written adjoint of the flux path behind a ``torch.autograd.Function``.

The differentiable map is one run of steps ``U_{n+1} = step(U_n; mesh_n, w_n, dt_n)``
on the real cells' conserved totals, with each step's mesh (geometry and neighbour
lists), face velocities and time step recorded from a forward run and held fixed --
the tessellation, the mesh motion and the CFL choice are not differentiated.  The
backward pass runs the reverse-mode kernels of ``phd_adj.cu`` step by step, from the
last step to the first, recomputing each segment's states from checkpoints taken
every ``checkpoint`` steps (checkpoint-and-recompute: memory holds the checkpoints and
one segment).

``FluxRun.apply(prim0, run)`` maps the real cells' initial primitives ``[4][n_real]``
(rho, v_x, v_y, p) to the final densities ``[n_real]``; gradients flow back to
``prim0``.
"""
import ctypes

import numpy as np
import torch

from . import _lib as L
from .device import DeviceClock, DeviceMesh, make_params

F64 = torch.float64


def adjoint_index(host):
    """Partner entries and per-image ghost lists of a host mesh (numpy int32)."""
    ptr, idx = host.nbr_ptr, host.nbr_idx
    E = int(ptr[-1])
    cells = np.repeat(np.arange(host.n_cells), np.diff(ptr))
    faces = idx[:E]
    o = np.lexsort((cells, faces))              # entries grouped by face, two per face
    partner = np.full(E, -1, dtype=np.int32)
    fa = faces[o]
    same = fa[0::2] == fa[1::2]
    if not np.all(same):
        raise RuntimeError("every face must appear in exactly two cells' lists")
    a, b = o[0::2], o[1::2]
    partner[a] = b
    partner[b] = a
    g = np.arange(host.n_real, host.n_cells)
    img = host.map[g]
    og = np.argsort(img, kind="stable")
    ghost_idx = g[og].astype(np.int32)
    cnt = np.bincount(img, minlength=host.n_real)
    ghost_ptr = np.concatenate([[0], np.cumsum(cnt)]).astype(np.int32)
    return partner, ghost_ptr, ghost_idx


class StepRecord:
    """What one step holds fixed: its device mesh, face velocities and dt."""

    def __init__(self, dmesh, face_w, dt):
        self.dmesh = dmesh
        self.face_w = face_w
        self.dt = float(dt)

    def index(self):
        """Partner/ghost index of the step's mesh, built once per device mesh."""
        dm = self.dmesh
        cached = getattr(dm, "_adjoint_index", None)
        if cached is None:
            p, gp, gi = adjoint_index(dm.host)
            tens = [torch.as_tensor(a).to(dm.device) for a in (p, gp, gi)]
            cached = (tens, L.PhdAdjIndex(*(t.data_ptr() for t in tens)))
            dm._adjoint_index = cached
        return cached[1]


class _MeshBuffers:
    """Per-mesh device buffers reused by every step on that mesh."""

    def __init__(self, dm, device):
        n, F = dm.n_cells, max(dm.n_faces, 1)
        self.cons = torch.zeros((4, n), dtype=F64, device=device)
        self.nxt = torch.zeros_like(self.cons)
        self.prim = torch.zeros_like(self.cons)
        self.grad = torch.zeros((8, n), dtype=F64, device=device)
        self.w = torch.zeros((2, n), dtype=F64, device=device)
        self.flux = torch.zeros((4, F), dtype=F64, device=device)
        self.lam_next = torch.zeros_like(self.cons)      # ghost rows stay zero
        self.lam = torch.zeros_like(self.cons)
        self.work = None

    def adjoint_work(self, lib, dm, device):
        if self.work is None:
            self.work = torch.empty(int(lib.phd_adjoint_work_doubles(dm.n_cells, dm.n_faces)), dtype=F64,
                                    device=device)
        return self.work


class FluxRunRecord:
    """A recorded run: the per-step records and the options of the step.

    Consecutive steps on the same device mesh are chained on the device: the update
    kernel already writes the next step's totals and primitives for every cell, ghosts
    included, so only a change of mesh goes back through the real cells (ghost refresh
    and primitive recovery on the new mesh).  Each step owns a row of a device clock
    table (its dt), so no step waits on the host.
    """

    def __init__(self, steps, gamma=1.4, solver="hllc", limiter="arepo", gizmo=True, boost=True,
                 reconstruction="linear", checkpoint=20, final_vol=None):
        if solver not in ("hll", "hllc", "exact"):
            raise ValueError("solver must be 'hll', 'hllc' or 'exact'")
        self.steps = steps
        self.params = make_params(gamma=gamma, solver=solver, limiter=limiter, gizmo=gizmo, boost=boost,
                                  reconstruction=reconstruction)
        self.checkpoint = max(1, int(checkpoint))
        self.final_vol = final_vol if final_vol is not None else steps[-1].dmesh.vol[:steps[-1].dmesh.n_real]
        d0 = steps[0].dmesh
        self.device = d0.device
        self.n_real = d0.n_real
        self.clock = DeviceClock(self.device)
        rows = []
        for rec in steps:
            c = L.PhdClock()
            c.dt = rec.dt
            c.dtmin_bits = np.float64(np.inf).view(np.uint64).item()
            rows.append(np.frombuffer(bytes(c), dtype=np.uint8))
        self._clocks0 = torch.as_tensor(np.stack(rows)).to(self.device)
        self.clocks = self._clocks0.clone()
        self._bufs = {}

    def _buffers(self, dm):
        b = self._bufs.get(id(dm))
        if b is None:
            b = self._bufs[id(dm)] = _MeshBuffers(dm, self.device)
        return b

    def _clock_ptr(self, k):
        return ctypes.c_void_p(self.clocks[k].data_ptr())

    def _load_real(self, dm, U_real, cons, prim):
        """All-cell totals and primitives on mesh dm from the real cells' totals."""
        s = L.stream_handle()
        lib = L.lib()
        cons[:, :dm.n_real].copy_(U_real)
        L.check(lib.phd_ghost_cons_f64(dm.ref, L.ptr(cons), s), "ghost")
        L.check(lib.phd_prim_from_cons_f64(2, dm.n_cells, self.params.gamma, L.ptr(dm.vol), L.ptr(cons),
                                           L.ptr(prim), s), "prim")

    def _step(self, k, prim, cons, nxt, grad, tape=None):
        """Step k: prim is overwritten with the next primitives, nxt receives the next
        totals (all cells), grad the limited gradients of the incoming primitives and,
        with a tape (f64, i32), the limiter's record for the adjoint."""
        rec = self.steps[k]
        b = self._buffers(rec.dmesh)
        lib = L.lib()
        if tape is None:
            L.check(lib.phd_step_f64(rec.dmesh.ref, ctypes.byref(self.params), 0, L.ptr(prim), L.ptr(cons),
                                     L.ptr(nxt), L.ptr(grad), L.ptr(b.w), L.ptr(rec.face_w), L.ptr(b.flux),
                                     self._clock_ptr(k), L.stream_handle()), "step")
        else:
            L.check(lib.phd_step_f64_taped(rec.dmesh.ref, ctypes.byref(self.params), 0, L.ptr(prim), L.ptr(cons),
                                           L.ptr(nxt), L.ptr(grad), L.ptr(b.w), L.ptr(rec.face_w), L.ptr(b.flux),
                                           L.ptr(tape[0]), L.ptr(tape[1]), self._clock_ptr(k),
                                           L.stream_handle()), "step")

    # --- one step in isolation, on real-cell totals (tests use these) ---------------
    def _forward_step(self, rec, U_real):
        dm = rec.dmesh
        cons = torch.zeros((4, dm.n_cells), dtype=F64, device=self.device)
        prim, nxt = torch.empty_like(cons), torch.empty_like(cons)
        grad = torch.zeros((8, dm.n_cells), dtype=F64, device=self.device)
        self._load_real(dm, U_real, cons, prim)
        self.clock.set(dt=rec.dt)
        b = self._buffers(dm)
        L.check(L.lib().phd_step_f64(dm.ref, ctypes.byref(self.params), 0, L.ptr(prim), L.ptr(cons), L.ptr(nxt),
                                     L.ptr(grad), L.ptr(b.w), L.ptr(rec.face_w), L.ptr(b.flux), self.clock.ptr,
                                     L.stream_handle()), "step")
        return nxt[:, :dm.n_real].clone()

    def _adjoint_step(self, rec, U_real, lam_next_real):
        dm = rec.dmesh
        cons = torch.zeros((4, dm.n_cells), dtype=F64, device=self.device)
        prim = torch.empty_like(cons)
        grad = torch.zeros((8, dm.n_cells), dtype=F64, device=self.device)
        self._load_real(dm, U_real, cons, prim)
        if self.params.reconstruction == L.LINEAR:
            L.check(L.lib().phd_gradients_f64(dm.ref, L.ptr(prim), self.params.limiter, L.ptr(grad), self.clock.ptr,
                                              L.stream_handle()), "gradients")
        return self._adjoint(rec, (cons, prim, grad, None), lam_next_real)

    def _adjoint(self, rec, state, lam_next_real):
        """lam_n (real cells) from lam_{n+1} at the step's recorded all-cell state
        (cons, prim, grad, tape); with a limiter tape the reverse reads the forward's
        selections instead of recomputing them."""
        cons, prim, grad, tape = state
        dm = rec.dmesh
        b = self._buffers(dm)
        lib = L.lib()
        b.lam_next[:, :dm.n_real].copy_(lam_next_real)
        common = (dm.ref, ctypes.byref(rec.index()), ctypes.byref(self.params), rec.dt, L.ptr(cons), L.ptr(prim),
                  L.ptr(grad), L.ptr(rec.face_w), L.ptr(b.lam_next), L.ptr(b.lam),
                  L.ptr(b.adjoint_work(lib, dm, self.device)))
        if tape is None:
            L.check(lib.phd_adjoint_step_f64(*common, L.stream_handle()), "phd_adjoint_step_f64")
        else:
            L.check(lib.phd_adjoint_step_f64_taped(*common, L.ptr(tape[0]), L.ptr(tape[1]), L.stream_handle()),
                    "phd_adjoint_step_f64_taped")
        return b.lam[:, :dm.n_real].clone()

    # --- whole run ------------------------------------------------------------------
    def forward(self, U0):
        """Run all steps from U0 [4][n_real]; keep checkpoints; return U_T."""
        self.clocks.copy_(self._clocks0)
        self.ckpt = {0: U0.clone()}
        prev = None
        for k, rec in enumerate(self.steps):
            dm = rec.dmesh
            b = self._buffers(dm)
            if prev is None:
                self._load_real(dm, U0, b.cons, b.prim)
            elif prev is not b:
                self._load_real(dm, prev.cons[:, :dm.n_real], b.cons, b.prim)
            self._step(k, b.prim, b.cons, b.nxt, b.grad)
            b.cons, b.nxt = b.nxt, b.cons
            prev = b
            if (k + 1) % self.checkpoint == 0 and k + 1 < len(self.steps):
                self.ckpt[k + 1] = b.cons[:, :dm.n_real].clone()
        UT = prev.cons[:, :self.steps[-1].dmesh.n_real].clone()
        st = 0
        for row in self.clocks.cpu().numpy():
            st |= L.PhdClock.from_buffer_copy(row.tobytes()).status
        L.raise_status(st)
        return UT

    # --- branch-frozen forward (finite differences on the branch the run takes) ----
    def forward_frozen(self, U0, record):
        """U_T from U0 through phd_step_f64_frozen.  With ``record`` the run from U0 is
        the ordinary forward, and every step's limiter selections and face decisions are
        written to this run's tapes; without it they are read back, so U0 -> U_T is the
        smooth map of the recorded run's branches, whose derivative the adjoint
        computes -- central differences through it check the adjoint even where the
        limited scheme itself has kinks within the difference step."""
        lib = L.lib()
        if record or getattr(self, "_frozen", None) is None:
            if not record:
                raise RuntimeError("forward_frozen: record a run before replaying it")
            self._frozen = []
            for rec in self.steps:
                dm = rec.dmesh
                self._frozen.append((torch.empty((L.GRAD_TAPE_F64_ROWS, dm.n_cells), dtype=F64, device=self.device),
                                     torch.empty((L.GRAD_TAPE_I32_ROWS, dm.n_cells), dtype=torch.int32,
                                                 device=self.device),
                                     torch.zeros(max(dm.n_faces, 1), dtype=torch.int64, device=self.device)))
        self.clock.set(dt=self.steps[0].dt)
        mode = L.FROZEN_RECORD if record else L.FROZEN_REPLAY
        prev = None
        for k, rec in enumerate(self.steps):
            dm = rec.dmesh
            b = self._buffers(dm)
            if prev is None:
                self._load_real(dm, U0, b.cons, b.prim)
            elif prev is not b:
                self._load_real(dm, prev.cons[:, :dm.n_real], b.cons, b.prim)
            tf, ti, fb = self._frozen[k]
            L.check(lib.phd_step_f64_frozen(dm.ref, ctypes.byref(self.params), mode, rec.dt, L.ptr(b.prim),
                                            L.ptr(b.cons), L.ptr(b.nxt), L.ptr(b.grad), L.ptr(rec.face_w),
                                            L.ptr(b.flux), L.ptr(tf), L.ptr(ti), L.ptr(fb), self.clock.ptr,
                                            L.stream_handle()), "phd_step_f64_frozen")
            b.cons, b.nxt = b.nxt, b.cons
            prev = b
        self.clock.check_status()
        return prev.cons[:, :self.steps[-1].dmesh.n_real].clone()

    def final_density_frozen(self, prim0, record=False):
        """Final densities [n_real] from the real cells' initial primitives through the
        branch-frozen forward (see forward_frozen)."""
        vol0 = self.steps[0].dmesh.vol[:self.n_real]
        U0 = cons_from_prim_t(prim0, vol0, self.params.gamma)
        return self.forward_frozen(U0.contiguous(), record)[0] / self.final_vol

    def _replay_segment(self, a, b):
        """Recompute the all-cell states (totals, primitives, gradients and the
        gradients' limiter tape) entering steps a..b-1 from the checkpoint at a."""
        states = []
        lib = L.lib()
        cons = prim = None
        self.clocks[a:b].copy_(self._clocks0[a:b])      # each step's CFL finish overwrote its dt
        for k in range(a, b):
            dm = self.steps[k].dmesh
            n = dm.n_cells
            if k == a or self.steps[k - 1].dmesh is not dm:
                U_real = self.ckpt[a] if k == a else cons[:, :dm.n_real]
                c = torch.empty((4, n), dtype=F64, device=self.device)
                p = torch.empty_like(c)
                self._load_real(dm, U_real, c, p)
                cons, prim = c, p
            grad = torch.zeros((8, n), dtype=F64, device=self.device)
            tape = None
            if self.params.reconstruction == L.LINEAR:
                tape = (torch.empty((L.GRAD_TAPE_F64_ROWS, n), dtype=F64, device=self.device),
                        torch.empty((L.GRAD_TAPE_I32_ROWS, n), dtype=torch.int32, device=self.device))
            states.append((cons, prim, grad, tape))
            if k + 1 < b:
                nxt = torch.empty_like(cons)
                p_next = prim.clone()                   # the step overwrites its primitives
                self._step(k, p_next, cons, nxt, grad, tape)
                cons, prim = nxt, p_next
            elif tape is not None:
                L.check(lib.phd_gradients_f64_taped(dm.ref, L.ptr(prim), self.params.limiter, L.ptr(grad),
                                                    L.ptr(tape[0]), L.ptr(tape[1]), self._clock_ptr(k),
                                                    L.stream_handle()), "gradients")
        return states

    def backward(self, lam_T):
        """dLoss/dU_0 from dLoss/dU_T, segment by segment (recompute from checkpoints)."""
        lam = lam_T
        N = len(self.steps)
        starts = sorted(self.ckpt)
        for si in range(len(starts) - 1, -1, -1):
            a = starts[si]
            b = starts[si + 1] if si + 1 < len(starts) else N
            states = self._replay_segment(a, b)
            for k in range(b - 1, a - 1, -1):
                lam = self._adjoint(self.steps[k], states[k - a], lam)
            del states
        return lam


def cons_from_prim_t(prim, vol, gamma):
    m = prim[0] * vol
    return torch.stack([m, prim[1] * m, prim[2] * m,
                        (0.5 * prim[0] * (prim[1] ** 2 + prim[2] ** 2) + prim[3] / (gamma - 1.0)) * vol])


class FluxRun(torch.autograd.Function):
    """prim0 [4][n_real] -> final densities [n_real] through a recorded run."""

    @staticmethod
    def forward(ctx, prim0, run):
        vol0 = run.steps[0].dmesh.vol[:run.n_real]
        with torch.no_grad():
            U0 = cons_from_prim_t(prim0, vol0, run.params.gamma)
            UT = run.forward(U0.contiguous())
        ctx.run = run
        ctx.save_for_backward(prim0)
        return UT[0] / run.final_vol

    @staticmethod
    def backward(ctx, g_rho):
        run = ctx.run
        (prim0,) = ctx.saved_tensors
        lam_T = torch.zeros((4, run.n_real), dtype=F64, device=prim0.device)
        lam_T[0] = g_rho / run.final_vol
        lam0 = run.backward(lam_T)
        vol0 = run.steps[0].dmesh.vol[:run.n_real]
        # cons_from_prim is local and smooth: its vector-Jacobian product via autograd
        with torch.enable_grad():
            p = prim0.detach().requires_grad_(True)
            U = cons_from_prim_t(p, vol0, run.params.gamma)
            (gp,) = torch.autograd.grad(U, p, grad_outputs=lam0)
        return gp, None
