"""Pure-PyTorch FP64 version of one flux step, differentiable by autograd.

TEST INFRASTRUCTURE ONLY: the reference the hand-written adjoint is checked against
(torch autograd through this function), never the product path.

One step maps the real cells' conserved totals U to U' with the mesh, the face
velocities and dt held fixed (the quantities the adjoint treats as constants):
ghost refresh (domain_manager.pyx:750-774, boundary.pyx:309-348), primitives
(equation_state.pyx:81-117), limited gradients (reconstruction.pyx:563-739 with
ghost gradients :819-835 / boundary.pyx:287-307), face states with the GIZMO limiter
and the MUSCL-Hancock half step (reconstruction.pyx:741-1072), HLLC / HLL fluxes with
deboost (riemann.pyx:190-682) and the conserved update (mesh.pyx:479-551).  Sums use
scatter-adds, so results agree with the reference to rounding, not bit for bit.
"""
import numpy as np
import torch

F64 = torch.float64


class TorchMesh:
    """Index and geometry tensors of one HostMesh for the vectorised step."""

    def __init__(self, m, device="cpu"):
        t = lambda a, dt=F64: torch.as_tensor(np.ascontiguousarray(a), dtype=dt, device=device)
        self.m = m
        self.n, self.nr, self.F = m.n_cells, m.n_real, m.n_faces
        self.pi = t(m.pair_i, torch.long)
        self.pj = t(m.pair_j, torch.long)
        self.map = t(m.map, torch.long)
        self.x = t(m.x)
        self.dcom = t(m.dcom)
        self.vol = t(m.vol)
        self.area = t(m.area)
        self.com = t(m.com)
        self.normal = t(m.normal)
        self.flip = t(m.flip_mask(), torch.long)
        self.real_j = self.pj < self.nr
        # gradient entries of real cells: (cell, neighbour, face)
        ptr, idx = m.nbr_ptr, m.nbr_idx
        cells = np.repeat(np.arange(m.n_cells), np.diff(ptr))
        sel = cells < m.n_real
        cells, faces = cells[sel], idx[ptr[0]:ptr[-1]][sel]
        nb = np.where(m.pair_i[faces] == cells, m.pair_j[faces], m.pair_i[faces])
        self.ec = t(cells, torch.long)
        self.ef = t(faces, torch.long)
        self.en = t(nb, torch.long)
        self.device = device


def full_cons(tm, U):
    """Real-cell totals -> all cells (ghost = image, reflective momentum flip)."""
    Ua = U[:, tm.map]
    sx = torch.where((tm.flip & 1) != 0, -1.0, 1.0).to(F64)
    sy = torch.where((tm.flip & 2) != 0, -1.0, 1.0).to(F64)
    return torch.stack([Ua[0], Ua[1] * sx, Ua[2] * sy, Ua[3]])


def prim_from_cons(U, vol, gamma):
    rho = U[0] / vol
    vx = U[1] / U[0]
    vy = U[2] / U[0]
    p = (U[3] / vol - 0.5 * rho * (vx * vx + vy * vy)) * (gamma - 1.0)
    return torch.stack([rho, vx, vy, p])


def cons_from_prim(prim, vol, gamma):
    m = prim[0] * vol
    return torch.stack([m, prim[1] * m, prim[2] * m,
                        (0.5 * prim[0] * (prim[1] ** 2 + prim[2] ** 2) + prim[3] / (gamma - 1.0)) * vol])


def _safe(d):
    return torch.where(d == 0, torch.ones_like(d), d)


def gradients(tm, prim, limiter="arepo"):
    c, j, f = tm.ec, tm.en, tm.ef
    xi = tm.x[:, c]
    xj = tm.x[:, j]
    cfx = tm.com[:, f] - 0.5 * (xi + xj)
    dr = xi - xj
    r = torch.sqrt((dr * dr).sum(0))
    pc, pj = prim[:, c], prim[:, j]
    d_dif = pj - pc
    d_sum = pj + pc
    fac = tm.area[f] / (r * tm.vol[c])
    nr = tm.nr
    df = torch.zeros((4, 2, nr), dtype=F64, device=prim.device)
    for k in range(2):
        contrib = fac * (d_dif * cfx[k] - 0.5 * d_sum * dr[k])
        df[:, k] = df[:, k].index_add(1, c, contrib)
    pr = prim[:, :nr]
    pmax = pr.clone().scatter_reduce(1, c.expand(4, -1), pj, reduce="amax", include_self=True)
    pmin = pr.clone().scatter_reduce(1, c.expand(4, -1), pj, reduce="amin", include_self=True)
    cx = tm.x[:, :nr] + tm.dcom[:, :nr]
    sep = tm.com[:, f] - cx[:, c]
    dphi = df[:, 0, c] * sep[0] + df[:, 1, c] * sep[1]
    ds = _safe(dphi)
    if limiter == "arepo":
        psi = torch.where(dphi > 0, (pmax[:, c] - pc) / ds,
                          torch.where(dphi < 0, (pmin[:, c] - pc) / ds, torch.ones_like(dphi)))
        val = torch.clamp(psi, min=0.0)
        alpha = torch.ones((4, nr), dtype=F64, device=prim.device).scatter_reduce(
            1, c.expand(4, -1), val, reduce="amin", include_self=True)
    else:
        t_ = (pj - pc) / ds
        psi = torch.where(dphi != 0, torch.clamp(t_, min=0.0), torch.ones_like(dphi))
        a0 = torch.ones(nr, dtype=F64, device=prim.device).scatter_reduce(
            0, c.repeat(4), psi.reshape(-1), reduce="amin", include_self=True)
        alpha = torch.stack([a0, torch.ones_like(a0), torch.ones_like(a0), torch.ones_like(a0)])
    g = alpha[:, None, :] * df                                  # [4 fields][2 dims][nr]
    g = g.reshape(8, nr)[:, tm.map]                             # ghosts = images
    sx = torch.where((tm.flip & 1) != 0, -1.0, 1.0).to(F64)
    sy = torch.where((tm.flip & 2) != 0, -1.0, 1.0).to(F64)
    g = torch.stack([g[0], g[1], g[2] * sx, g[3], g[4], g[5] * sy, g[6], g[7]])
    return g


def face_states(tm, prim, grad, w, gamma, dt_half, boost=True, gizmo=True):
    i, j = tm.pi, tm.pj
    pi_, pj_ = prim[:, i], prim[:, j]
    gi, gj = grad[:, i], grad[:, j]
    shift = torch.stack([torch.zeros_like(w[0]), w[0], w[1], torch.zeros_like(w[0])]) if boost else 0.0
    sl = pi_ - shift
    sr = pj_ - shift
    sepi = tm.com - (tm.x[:, i] + tm.dcom[:, i])
    sepj = tm.com - (tm.x[:, j] + tm.dcom[:, j])
    L = sl + gi[0::2] * sepi[0] + gi[1::2] * sepi[1]
    R = sr + gj[0::2] * sepj[0] + gj[1::2] * sepj[1]
    if gizmo:
        smi = torch.sqrt((sepi * sepi).sum(0))
        smj = torch.sqrt((sepj * sepj).sum(0))
        dm = torch.sqrt(((tm.x[:, j] - tm.x[:, i]) ** 2).sum(0))
        d1 = 0.5 * torch.abs(sl - sr)
        d2 = 0.25 * torch.abs(sl - sr)
        pmn = torch.minimum(sl, sr)
        pmx = torch.maximum(sl, sr)
        bl = sl + smi / dm * (sr - sl)
        br = sr + smj / dm * (sl - sr)
        pplus = torch.where((pmx + d1) * pmx >= 0, pmx + d1, pmx / (1 + d1 / _safe(torch.abs(pmx))))
        pminus = torch.where((pmn - d1) * pmn >= 0, pmn - d1, pmn / (1 + d1 / _safe(torch.abs(pmn))))
        lt = pi_ < pj_
        gt = pi_ > pj_
        Ll = torch.maximum(pminus, torch.minimum(bl + d2, L))
        Rl = torch.minimum(pplus, torch.maximum(br - d2, R))
        Lg = torch.minimum(pplus, torch.maximum(bl - d2, L))
        Rg = torch.maximum(pminus, torch.minimum(br + d2, R))
        L = torch.where(lt, Ll, torch.where(gt, Lg, sl))
        R = torch.where(lt, Rl, torch.where(gt, Rg, sr))
        negL = (L[0] < 0) | (L[3] < 0)
        negR = (R[0] < 0) | (R[3] < 0)
        L = torch.where(negL[None], sl, L)
        R = torch.where(negR[None], sr, R)
    sL, sR = L, R
    vi = pi_[1:3] - (w if boost else 0.0)
    vj = pj_[1:3] - (w if boost else 0.0)
    dt = dt_half
    Lv = [L[1] - dt * gi[6] / pi_[0], L[2] - dt * gi[7] / pi_[0]]
    Rv = [R[1] - dt * gj[6] / pj_[0], R[2] - dt * gj[7] / pj_[0]]
    divi = gi[2] + gi[5]
    divj = gj[2] + gj[5]
    Ld = L[0] - dt * (pi_[0] * gi[2] + vi[0] * gi[0]) - dt * (pi_[0] * gi[5] + vi[1] * gi[1])
    Rd = R[0] - dt * (pj_[0] * gj[2] + vj[0] * gj[0]) - dt * (pj_[0] * gj[5] + vj[1] * gj[1])
    Lp = L[3] - dt * (gamma * pi_[3] * gi[2] + vi[0] * gi[6]) - dt * (gamma * pi_[3] * gi[5] + vi[1] * gi[7])
    Rp = R[3] - dt * (gamma * pj_[3] * gj[2] + vj[0] * gj[6]) - dt * (gamma * pj_[3] * gj[5] + vj[1] * gj[7])
    for k in range(2):
        Lv = [Lv[c] - dt * vi[k] * gi[2 + 2 * c + k] for c in range(2)]
        Rv = [Rv[c] - dt * vj[k] * gj[2 + 2 * c + k] for c in range(2)]
    Lt = torch.stack([Ld, Lv[0], Lv[1], Lp])
    Rt = torch.stack([Rd, Rv[0], Rv[1], Rp])
    del divi, divj
    negL = (Lt[0] < 0) | (Lt[3] < 0)
    negR = (Rt[0] < 0) | (Rt[3] < 0)
    return torch.where(negL[None], sL, Lt), torch.where(negR[None], sR, Rt)


def get_waves(dl, ul, pl, dr, ur, pr, gamma):
    cl = torch.clamp(torch.sqrt(gamma * pl / dl), min=1e-10)
    cr = torch.clamp(torch.sqrt(gamma * pr / dr), min=1e-10)
    d_avg = 0.5 * (dl + dr)
    c_avg = 0.5 * (cl + cr)
    pv = torch.clamp(0.5 * (pl + pr) + 0.5 * (ul - ur) * d_avg * c_avg, min=0.0)
    pmin = torch.minimum(pl, pr)
    pmax = torch.maximum(pl, pr)
    z = (gamma - 1.0) / (2.0 * gamma)
    plr = (pl / pr) ** z
    us = (plr * ul / cl + ur / cr + 2.0 * (plr - 1.0) / (gamma - 1.0)) / (plr / cl + 1.0 / cr)
    a1 = torch.clamp(1.0 + (gamma - 1.0) * (ul - us) / (2.0 * cl), min=1e-300)
    a2 = torch.clamp(1.0 + (gamma - 1.0) * (us - ur) / (2.0 * cr), min=1e-300)
    p_tr = 0.5 * pl * a1 ** (1.0 / z) + 0.5 * pr * a2 ** (1.0 / z)
    Al = 2.0 / ((gamma + 1.0) * dl)
    Ar = 2.0 / ((gamma + 1.0) * dr)
    Bl = pl * ((gamma - 1.0) / (gamma + 1.0))
    Br = pr * ((gamma - 1.0) / (gamma + 1.0))
    gl = torch.sqrt(Al / (pv + Bl))
    gr = torch.sqrt(Ar / (pv + Br))
    p_ts = (gl * pl + gr * pr - (ur - ul)) / (gl + gr)
    pvrs = ((pmax / pmin) < 2.0) & (pmin < pv) & (pv < pmax)
    ps = torch.where(pvrs, pv, torch.where(pv <= pmin, p_tr, p_ts))
    k = (gamma + 1.0) / (2.0 * gamma)
    sl = torch.where(ps <= pl, ul - cl, ul - cl * torch.sqrt(torch.clamp(1.0 + k * (ps / pl - 1.0), min=1e-300)))
    sr = torch.where(ps <= pr, ur + cr, ur + cr * torch.sqrt(torch.clamp(1.0 + k * (ps / pr - 1.0), min=1e-300)))
    sc = (pr - pl + dl * ul * (sl - ul) - dr * ur * (sr - ur)) / (dl * (sl - ul) - dr * (sr - ur))
    return sl, sc, sr


def riemann(tm, L, R, w, gamma, solver="hllc", boost=True):
    n = tm.normal
    dl, pl, dr, pr = L[0], L[3], R[0], R[3]
    Vnl = L[1] * n[0] + L[2] * n[1]
    Vnr = R[1] * n[0] + R[2] * n[1]
    vl2 = L[1] ** 2 + L[2] ** 2
    vr2 = R[1] ** 2 + R[2] ** 2
    wn = torch.zeros_like(dl) if boost else w[0] * n[0] + w[1] * n[1]
    sl, sc, sr = get_waves(dl, Vnl, pl, dr, Vnr, pr, gamma)
    el = 0.5 * dl * vl2 + pl / (gamma - 1.0)
    er = 0.5 * dr * vr2 + pr / (gamma - 1.0)
    FL = [dl * (Vnl - wn), dl * L[1] * (Vnl - wn) + pl * n[0], dl * L[2] * (Vnl - wn) + pl * n[1],
          el * (Vnl - wn) + pl * Vnl]
    FR = [dr * (Vnr - wn), dr * R[1] * (Vnr - wn) + pr * n[0], dr * R[2] * (Vnr - wn) + pr * n[1],
          er * (Vnr - wn) + pr * Vnr]
    if solver == "hll":
        f1, f2, f3 = sr - wn, sl - wn, _safe(sr - sl)
        Fm = [(dl * Vnl * f1 - dr * Vnr * f2 - sl * dl * f1 + sr * dr * f2) / f3]
        for k in range(2):
            Fm.append(((dl * L[1 + k] * Vnl + pl * n[k]) * f1 - (dr * R[1 + k] * Vnr + pr * n[k]) * f2
                       - sl * dl * L[1 + k] * f1 + sr * dr * R[1 + k] * f2) / f3)
        Fm.append(((el + pl) * Vnl * f1 - (er + pr) * Vnr * f2 - sl * el * f1 + sr * er * f2) / f3)
        mid = [Fm[q] for q in range(4)]
    else:
        f1l = dl * (sl - Vnl) / _safe(sl - sc)
        f2l = f1l * (sl - wn) * (sc - Vnl) + pl
        frl = dl * (Vnl - sl) + f1l * (sl - wn)
        EL = (el + pl) * Vnl - sl * el + (sl - wn) * f1l * (el / dl + (sc - Vnl) * (sc + pl / _safe(dl * (sl - Vnl))))
        f1r = dr * (sr - Vnr) / _safe(sr - sc)
        f2r = f1r * (sr - wn) * (sc - Vnr) + pr
        frr = dr * (Vnr - sr) + f1r * (sr - wn)
        ER = (er + pr) * Vnr - sr * er + (sr - wn) * f1r * (er / dr + (sc - Vnr) * (sc + pr / _safe(dr * (sr - Vnr))))
        sL = [frl, frl * L[1] + f2l * n[0], frl * L[2] + f2l * n[1], EL]
        sR = [frr, frr * R[1] + f2r * n[0], frr * R[2] + f2r * n[1], ER]
        mid = [torch.where(wn <= sc, sL[q], sR[q]) for q in range(4)]
    out = []
    for q in range(4):
        out.append(torch.where(wn <= sl, FL[q], torch.where((sl < wn) & (wn <= sr), mid[q], FR[q])))
    f = torch.stack(out)
    if boost:
        fe = f[3] + w[0] * (0.5 * w[0] * f[0] + f[1])
        fmx = f[1] + w[0] * f[0]
        fe = fe + w[1] * (0.5 * w[1] * f[0] + f[2])
        fmy = f[2] + w[1] * f[0]
        f = torch.stack([f[0], fmx, fmy, fe])
    return f


def update(tm, U, flux, dt):
    nr = tm.nr
    inc = dt * tm.area * flux
    Un = U.index_add(1, tm.pi, -inc)
    rj = tm.real_j
    return Un.index_add(1, tm.pj[rj], inc[:, rj])


def step(tm, U, w, dt, gamma, solver="hllc", limiter="arepo", gizmo=True, boost=True):
    """One step U -> U' (real-cell totals), mesh / face velocities / dt fixed."""
    Ua = full_cons(tm, U)
    prim = prim_from_cons(Ua, tm.vol, gamma)
    g = gradients(tm, prim, limiter)
    L, R = face_states(tm, prim, g, w, gamma, 0.5 * dt, boost=boost, gizmo=gizmo)
    f = riemann(tm, L, R, w, gamma, solver=solver, boost=boost)
    return update(tm, U, f, dt)
