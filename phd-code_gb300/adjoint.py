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
        self._index = None

    def index(self):
        if self._index is None:
            dev = self.dmesh.device
            p, gp, gi = adjoint_index(self.dmesh.host)
            tens = [torch.as_tensor(a).to(dev) for a in (p, gp, gi)]
            s = L.PhdAdjIndex(*(t.data_ptr() for t in tens))
            self._index = (tens, s)
        return self._index[1]


class FluxRunRecord:
    """A recorded run: the per-step records and the options of the step."""

    def __init__(self, steps, gamma=1.4, solver="hllc", limiter="arepo", gizmo=True, boost=True,
                 reconstruction="linear", checkpoint=20, final_vol=None):
        if solver not in ("hll", "hllc"):
            raise ValueError("the adjoint covers the HLL and HLLC solvers")
        self.steps = steps
        self.params = make_params(gamma=gamma, solver=solver, limiter=limiter, gizmo=gizmo, boost=boost,
                                  reconstruction=reconstruction)
        self.checkpoint = max(1, int(checkpoint))
        self.final_vol = final_vol if final_vol is not None else steps[-1].dmesh.vol[:steps[-1].dmesh.n_real]
        d0 = steps[0].dmesh
        self.device = d0.device
        self.n_real = d0.n_real
        self.clock = DeviceClock(self.device)

    # --- one forward step on all-cell totals [4][n] of the step's mesh ---------------
    def _forward_step(self, rec, U_real):
        dm = rec.dmesh
        n = dm.n_cells
        cons = torch.zeros((4, n), dtype=F64, device=self.device)
        cons[:, :dm.n_real] = U_real
        s = L.stream_handle()
        lib = L.lib()
        L.check(lib.phd_ghost_cons_f64(dm.ref, L.ptr(cons), s), "ghost")
        prim = torch.empty_like(cons)
        L.check(lib.phd_prim_from_cons_f64(2, n, self.params.gamma, L.ptr(dm.vol), L.ptr(cons), L.ptr(prim), s),
                "prim")
        nxt = torch.empty_like(cons)
        grad = torch.zeros((8, n), dtype=F64, device=self.device)
        w = torch.zeros((2, n), dtype=F64, device=self.device)
        flux = torch.zeros((4, max(dm.n_faces, 1)), dtype=F64, device=self.device)
        self.clock.set(dt=rec.dt)
        L.check(lib.phd_step_f64(dm.ref, ctypes.byref(self.params), 0, L.ptr(prim), L.ptr(cons), L.ptr(nxt),
                                 L.ptr(grad), L.ptr(w), L.ptr(rec.face_w), L.ptr(flux), self.clock.ptr, s), "step")
        return nxt[:, :dm.n_real].clone()

    def forward(self, U0):
        """Run all steps from U0 [4][n_real]; keep checkpoints; return U_T."""
        self.ckpt = {0: U0.clone()}
        U = U0
        for k, rec in enumerate(self.steps):
            U = self._forward_step(rec, U)
            if (k + 1) % self.checkpoint == 0 and k + 1 < len(self.steps):
                self.ckpt[k + 1] = U.clone()
        st = self.clock.read().status
        L.raise_status(st)
        return U

    # --- reverse ------------------------------------------------------------------
    def _adjoint_step(self, rec, U_real, lam_next_real):
        dm = rec.dmesh
        n, nr = dm.n_cells, dm.n_real
        lib = L.lib()
        s = L.stream_handle()
        cons = torch.zeros((4, n), dtype=F64, device=self.device)
        cons[:, :nr] = U_real
        L.check(lib.phd_ghost_cons_f64(dm.ref, L.ptr(cons), s), "ghost")
        prim = torch.empty_like(cons)
        L.check(lib.phd_prim_from_cons_f64(2, n, self.params.gamma, L.ptr(dm.vol), L.ptr(cons), L.ptr(prim), s),
                "prim")
        grad = torch.zeros((8, n), dtype=F64, device=self.device)
        if self.params.reconstruction == L.LINEAR:
            L.check(lib.phd_gradients_f64(dm.ref, L.ptr(prim), self.params.limiter, L.ptr(grad), self.clock.ptr, s),
                    "gradients")
        lam_next = torch.zeros((4, n), dtype=F64, device=self.device)
        lam_next[:, :nr] = lam_next_real
        lam = torch.empty_like(lam_next)
        nwork = lib.phd_adjoint_work_doubles(n, dm.n_faces)
        work = torch.empty(int(nwork), dtype=F64, device=self.device)
        L.check(lib.phd_adjoint_step_f64(dm.ref, ctypes.byref(rec.index()), ctypes.byref(self.params), rec.dt,
                                         L.ptr(cons), L.ptr(prim), L.ptr(grad), L.ptr(rec.face_w), L.ptr(lam_next),
                                         L.ptr(lam), L.ptr(work), s), "phd_adjoint_step_f64")
        return lam[:, :nr].clone()

    def backward(self, lam_T):
        """dLoss/dU_0 from dLoss/dU_T, segment by segment (recompute from checkpoints)."""
        lam = lam_T
        N = len(self.steps)
        starts = sorted(self.ckpt)
        for si in range(len(starts) - 1, -1, -1):
            a = starts[si]
            b = starts[si + 1] if si + 1 < len(starts) else N
            states = [self.ckpt[a]]
            for k in range(a, b - 1):
                states.append(self._forward_step(self.steps[k], states[-1]))
            for k in range(b - 1, a - 1, -1):
                lam = self._adjoint_step(self.steps[k], states[k - a], lam)
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
