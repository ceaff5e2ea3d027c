// phd_adjoint.cuh -- hand-written reverse mode of the per-face and per-cell physics.
//
// Every function recomputes the forward quantities of its routine (same formulas and
// branch decisions as phd_physics.cuh / phd_f64.cu) and then propagates adjoints
// statement by statement in reverse.  Branch decisions (wave-speed estimate,
// flux region, GIZMO clip, positivity reverts, limiter selections) are held fixed:
// the derivative of the active branch.  Naming: aX = dLoss/dX.
#pragma once
#include "phd_physics.cuh"

namespace phd {

// ---- get_waves (riemann.pyx:375-504) --------------------------------------------
// Forward pass with the same formulas and operation order as get_waves in
// phd_physics.cuh (so the same branch decisions), keeping what the reverse needs.
template <typename T>
struct WaveTape {
    T cl, cr, d_avg, c_avg, pv_raw, p_star;
    T z, plr, den, u_star, A1, A2, e, PA1, PA2;       // two-rarefaction branch
    T Al, Ar, Bl, Brr, gl, gr, S;                      // two-shock branch
    T k, sqlv, sqrv, sl, sr, D, sc;
    int br;                                            // 0 PVRS, 1 TRRS, 2 TSRS
    bool cl_fl, cr_fl, l_shock, r_shock;
};

template <typename T>
PHD_HD __forceinline__ void get_waves_fwd(T dl, T ul, T pl, T dr, T ur, T pr, T gamma, WaveTape<T> &t) {
    const T c_floor = T(1.0E-10);
    const T clr = t_sqrt((gamma * pl) / dl), crr = t_sqrt((gamma * pr) / dr);
    t.cl_fl = !(clr >= c_floor);
    t.cr_fl = !(crr >= c_floor);
    t.cl = t_fmax(clr, c_floor);
    t.cr = t_fmax(crr, c_floor);
    const T cl = t.cl, cr = t.cr;
    t.d_avg = T(.5) * (dl + dr);
    t.c_avg = T(.5) * (cl + cr);
    t.pv_raw = (T(.5) * (pl + pr)) + (((T(.5) * (ul - ur)) * t.d_avg) * t.c_avg);
    const T pv = t_fmax(T(0.), t.pv_raw);
    const T p_min = t_fmin(pl, pr), p_max = t_fmax(pl, pr);
    T p_star = pv;
    t.z = t.plr = t.den = t.u_star = t.A1 = t.A2 = t.e = t.PA1 = t.PA2 = T(0);
    t.Al = t.Ar = t.Bl = t.Brr = t.gl = t.gr = t.S = T(0);
    if (((p_max / p_min) < T(2.)) && ((p_min < pv) && (pv < p_max))) {
        t.br = 0;
    } else if (pv <= p_min) {
        t.br = 1;
        t.z = (gamma - T(1.)) / (T(2.) * gamma);
        t.plr = t_pow(pl / pr, t.z);
        const T num = (((t.plr * ul) / cl) + (ur / cr)) + ((T(2.) * (t.plr - T(1.))) / (gamma - T(1.)));
        t.den = (t.plr / cl) + (T(1.) / cr);
        t.u_star = num / t.den;
        t.A1 = T(1.) + (((gamma - T(1.)) * (ul - t.u_star)) / (T(2.) * cl));
        t.A2 = T(1.) + (((gamma - T(1.)) * (t.u_star - ur)) / (T(2.) * cr));
        t.e = T(1.) / t.z;
        t.PA1 = t_pow(t.A1, t.e);
        t.PA2 = t_pow(t.A2, t.e);
        p_star = (T(.5) * pl) * t.PA1;
        p_star = p_star + ((T(.5) * pr) * t.PA2);
    } else {
        t.br = 2;
        t.Al = T(2.) / ((gamma + T(1.)) * dl);
        t.Ar = T(2.) / ((gamma + T(1.)) * dr);
        t.Bl = pl * ((gamma - T(1.)) / (gamma + T(1.)));
        t.Brr = pr * ((gamma - T(1.)) / (gamma + T(1.)));
        t.gl = t_sqrt(t.Al / (pv + t.Bl));
        t.gr = t_sqrt(t.Ar / (pv + t.Brr));
        t.S = t.gl + t.gr;
        p_star = (((t.gl * pl) + (t.gr * pr)) - (ur - ul)) / t.S;
    }
    t.p_star = p_star;
    t.k = (gamma + T(1.)) / (T(2.) * gamma);
    t.l_shock = !(p_star <= pl);
    t.r_shock = !(p_star <= pr);
    t.sqlv = t.sqrv = T(0);
    if (!t.l_shock) t.sl = ul - cl;
    else { t.sqlv = t_sqrt(T(1.) + (t.k * ((p_star / pl) - T(1.)))); t.sl = ul - (cl * t.sqlv); }
    if (!t.r_shock) t.sr = ur + cr;
    else { t.sqrv = t_sqrt(T(1.) + (t.k * ((p_star / pr) - T(1.)))); t.sr = ur + (cr * t.sqrv); }
    const T N = (((pr - pl) + ((dl * ul) * (t.sl - ul))) - ((dr * ur) * (t.sr - ur)));
    t.D = ((dl * (t.sl - ul)) - (dr * (t.sr - ur)));
    t.sc = N / t.D;
}

// Reverse of get_waves_fwd: adjoints of (sl, sc, sr) -> adjoints of the inputs.
// Derivative-only arithmetic (no branch depends on it) uses reciprocals.
template <typename T>
PHD_HD __forceinline__ void get_waves_rev(const WaveTape<T> &t, T dl, T ul, T pl, T dr, T ur, T pr, T gamma,
                                          T a_sl, T a_sc, T a_sr, T &a_dl, T &a_ul, T &a_pl, T &a_dr, T &a_ur,
                                          T &a_pr) {
    const T cl = t.cl, cr = t.cr, sl = t.sl, sr = t.sr, sc = t.sc, p_star = t.p_star, k = t.k;
    const T iD = T(1.) / t.D, ipl = T(1.) / pl, ipr = T(1.) / pr;
    T aN = a_sc * iD, aD = -a_sc * sc * iD;
    T asl = a_sl, asr = a_sr, acl = 0, acr = 0, aps = 0;
    a_pr += aN;
    a_pl -= aN;
    a_dl += aN * ul * (sl - ul) + aD * (sl - ul);
    a_ul += aN * dl * (sl - T(2.) * ul) - aD * dl;
    asl += aN * dl * ul + aD * dl;
    a_dr += -aN * ur * (sr - ur) - aD * (sr - ur);
    a_ur += -aN * dr * (sr - T(2.) * ur) + aD * dr;
    asr += -aN * dr * ur - aD * dr;
    // sl, sr
    a_ul += asl;
    if (!t.l_shock) acl -= asl;
    else {
        acl -= t.sqlv * asl;
        const T aq = (-cl * asl) / (T(2.) * t.sqlv);
        aps += aq * k * ipl;
        a_pl -= aq * k * p_star * ipl * ipl;
    }
    a_ur += asr;
    if (!t.r_shock) acr += asr;
    else {
        acr += t.sqrv * asr;
        const T aq = (cr * asr) / (T(2.) * t.sqrv);
        aps += aq * k * ipr;
        a_pr -= aq * k * p_star * ipr * ipr;
    }
    // p_star
    T apv = 0;
    if (t.br == 0) {
        apv += aps;
    } else if (t.br == 1) {
        const T icl = T(1.) / cl, icr = T(1.) / cr, g1 = gamma - T(1.);
        a_pl += T(.5) * t.PA1 * aps;
        a_pr += T(.5) * t.PA2 * aps;
        // d(A^e)/dA = e A^e / A
        const T aA1 = T(.5) * pl * t.e * (t.PA1 / t.A1) * aps;
        const T aA2 = T(.5) * pr * t.e * (t.PA2 / t.A2) * aps;
        T aus = 0;
        a_ul += aA1 * g1 * T(.5) * icl;
        aus -= aA1 * g1 * T(.5) * icl;
        acl -= aA1 * g1 * (ul - t.u_star) * T(.5) * icl * icl;
        aus += aA2 * g1 * T(.5) * icr;
        a_ur -= aA2 * g1 * T(.5) * icr;
        acr -= aA2 * g1 * (t.u_star - ur) * T(.5) * icr * icr;
        const T iden = T(1.) / t.den;
        const T anum = aus * iden, aden = -aus * t.u_star * iden;
        T aplr = anum * (ul * icl + T(2.) / g1) + aden * icl;
        a_ul += anum * t.plr * icl;
        acl -= (anum * t.plr * ul + aden * t.plr) * icl * icl;
        a_ur += anum * icr;
        acr -= (anum * ur + aden) * icr * icr;
        a_pl += aplr * t.z * t.plr * ipl;
        a_pr -= aplr * t.z * t.plr * ipr;
    } else {
        const T iS = T(1.) / t.S;
        const T aNn = aps * iS, aS = -aps * p_star * iS;
        const T agl = aNn * pl + aS, agr = aNn * pr + aS;
        a_pl += aNn * t.gl;
        a_pr += aNn * t.gr;
        a_ur -= aNn;
        a_ul += aNn;
        const T pv = t_fmax(T(0.), t.pv_raw);
        const T idnl = T(1.) / (pv + t.Bl), idnr = T(1.) / (pv + t.Brr);
        const T ahl = agl / (T(2.) * t.gl), ahr = agr / (T(2.) * t.gr);
        const T aAl = ahl * idnl, aAr = ahr * idnr;
        apv -= ahl * t.Al * idnl * idnl + ahr * t.Ar * idnr * idnr;
        const T aBl = -ahl * t.Al * idnl * idnl, aBr = -ahr * t.Ar * idnr * idnr;
        a_dl -= aAl * t.Al / dl;
        a_dr -= aAr * t.Ar / dr;
        a_pl += aBl * ((gamma - T(1.)) / (gamma + T(1.)));
        a_pr += aBr * ((gamma - T(1.)) / (gamma + T(1.)));
    }
    if (t.pv_raw > T(0.)) {
        a_pl += T(.5) * apv;
        a_pr += T(.5) * apv;
        a_ul += T(.5) * t.d_avg * t.c_avg * apv;
        a_ur -= T(.5) * t.d_avg * t.c_avg * apv;
        const T ada = T(.5) * (ul - ur) * t.c_avg * apv, aca = T(.5) * (ul - ur) * t.d_avg * apv;
        a_dl += T(.5) * ada;
        a_dr += T(.5) * ada;
        acl += T(.5) * aca;
        acr += T(.5) * aca;
    }
    if (!t.cl_fl) {
        const T idl = T(1.) / dl;
        a_pl += acl * gamma * T(.5) * idl / cl;
        a_dl -= acl * cl * T(.5) * idl;
    }
    if (!t.cr_fl) {
        const T idr = T(1.) / dr;
        a_pr += acr * gamma * T(.5) * idr / cr;
        a_dr -= acr * cr * T(.5) * idr;
    }
}

template <typename T>
PHD_HD void get_waves_adj(T dl, T ul, T pl, T dr, T ur, T pr, T gamma, T a_sl, T a_sc, T a_sr,
                              T &a_dl, T &a_ul, T &a_pl, T &a_dr, T &a_ur, T &a_pr) {
    WaveTape<T> t;
    get_waves_fwd<T>(dl, ul, pl, dr, ur, pr, gamma, t);
    get_waves_rev<T>(t, dl, ul, pl, dr, ur, pr, gamma, a_sl, a_sc, a_sr, a_dl, a_ul, a_pl, a_dr, a_ur, a_pr);
}

// Adjoint of the left / right data flux  F = (d u, d v_k u + p n_k, E u + p Vn),
// u = Vn - wn, E = d v^2 / 2 + p/(gamma-1).
template <typename T>
PHD_HD __forceinline__ void data_flux_adj(T d, const T *v, T p, T Vn, T v2, const T *n, T wn, T gamma,
                                              const T *aF, T &ad, T *av, T &ap, T &aVn, T &av2) {
    const T u = Vn - wn;
    const T E = (T(0.5) * d) * v2 + p / (gamma - T(1.));
    ad += aF[0] * u + (aF[1] * v[0] + aF[2] * v[1]) * u + aF[3] * T(0.5) * v2 * u;
    const T au = aF[0] * d + (aF[1] * v[0] + aF[2] * v[1]) * d + aF[3] * E;
    aVn += au + aF[3] * p;
    av[0] += aF[1] * d * u;
    av[1] += aF[2] * d * u;
    ap += aF[1] * n[0] + aF[2] * n[1] + aF[3] * (u / (gamma - T(1.)) + Vn);
    av2 += aF[3] * T(0.5) * d * u;
}

// Adjoint of the HLLC star-state flux of one side (riemann.pyx:636-670):
// (d, v, p, Vn, v2, s = this side's wave speed) ; sc contact speed.
template <typename T>
PHD_HD __forceinline__ void star_flux_adj(T d, const T *v, T p, T Vn, T v2, T s, T sc, const T *n, T wn,
                                              T gamma, const T *aF, T &ad, T *av, T &ap, T &aVn, T &av2, T &as,
                                              T &asc) {
    const T a = s - Vn, b = s - sc;
    const T id = T(1.) / d, ia = T(1.) / a, ib = T(1.) / b, igm1 = T(1.) / (gamma - T(1.0));
    const T f1 = d * a * ib;
    const T frho = (d * (Vn - s)) + (f1 * (s - wn));
    const T el = ((T(0.5) * d) * v2) + (p * igm1);
    const T t = p * id * ia;
    const T Q = (el * id) + ((sc - Vn) * (sc + t));
    const T afrho = aF[0] + aF[1] * v[0] + aF[2] * v[1];
    av[0] += aF[1] * frho;
    av[1] += aF[2] * frho;
    const T af2 = aF[1] * n[0] + aF[2] * n[1];
    // fe = (el + p) Vn - s el + (s - wn) f1 Q
    T ael = aF[3] * (Vn - s);
    ap += aF[3] * Vn;
    aVn += aF[3] * (el + p);
    as += aF[3] * (-el + f1 * Q);
    T af1 = aF[3] * (s - wn) * Q;
    const T aQ = aF[3] * (s - wn) * f1;
    // Q = el/d + (sc - Vn)(sc + t)
    ael += aQ * id;
    ad -= aQ * el * id * id;
    asc += aQ * (sc + t) + aQ * (sc - Vn);
    aVn -= aQ * (sc + t);
    const T at = aQ * (sc - Vn);
    T aa = 0;
    ap += at * id * ia;
    ad -= at * t * id;
    aa -= at * t * ia;
    // frho = d (Vn - s) + f1 (s - wn)
    ad += afrho * (Vn - s);
    aVn += afrho * d;
    as += afrho * (-d + f1);
    af1 += afrho * (s - wn);
    // f2 = f1 (s - wn)(sc - Vn) + p
    af1 += af2 * (s - wn) * (sc - Vn);
    as += af2 * f1 * (sc - Vn);
    asc += af2 * f1 * (s - wn);
    aVn -= af2 * f1 * (s - wn);
    ap += af2;
    // f1 = d a / b
    ad += af1 * a * ib;
    aa += af1 * d * ib;
    const T ab = -af1 * f1 * ib;
    as += aa + ab;
    aVn -= aa;
    asc -= ab;
    // el
    ad += ael * T(0.5) * v2;
    av2 += ael * T(0.5) * d;
    ap += ael * igm1;
}

// Adjoint of hll_family (HLL / HLLC + deboost), 2D.  aF: adjoint of the (deboosted)
// flux; accumulates into aL, aR.
template <typename T>
PHD_HD void hll_family_adj(bool hllc, const T *L, const T *R, const T *n, const T *w, T gamma, bool boost,
                               const T *aFin, T *aL, T *aR) {
    const T _dl = L[0], _pl = L[3], _dr = R[0], _pr = R[3];
    const T vl[2] = {L[1], L[2]}, vr[2] = {R[1], R[2]};
    T Vnl = T(0.0), Vnr = T(0.0), vl_sq = T(0.0), vr_sq = T(0.0), wn = T(0.0);
    for (int k = 0; k < 2; k++) {
        vl_sq = vl_sq + vl[k] * vl[k];
        vr_sq = vr_sq + vr[k] * vr[k];
        Vnl = Vnl + vl[k] * n[k];
        Vnr = Vnr + vr[k] * n[k];
        wn = wn + w[k] * n[k];
    }
    if (boost) wn = T(0.);
    WaveTape<T> wt;
    get_waves_fwd<T>(_dl, Vnl, _pl, _dr, Vnr, _pr, gamma, wt);
    const T sl = wt.sl, sc = wt.sc, sr = wt.sr;
    // deboost reverse
    T aF[4] = {aFin[0], aFin[1], aFin[2], aFin[3]};
    if (boost) {
        aF[0] = aFin[0] + w[0] * aFin[1] + w[1] * aFin[2] + T(0.5) * (w[0] * w[0] + w[1] * w[1]) * aFin[3];
        aF[1] = aFin[1] + w[0] * aFin[3];
        aF[2] = aFin[2] + w[1] * aFin[3];
        aF[3] = aFin[3];
    }
    T adl = 0, apl = 0, aVnl = 0, avl2 = 0, adr = 0, apr = 0, aVnr = 0, avr2 = 0;
    T avl[2] = {0, 0}, avr[2] = {0, 0};
    T asl = 0, asc = 0, asr = 0;
    if (wn <= sl) {
        data_flux_adj<T>(_dl, vl, _pl, Vnl, vl_sq, n, wn, gamma, aF, adl, avl, apl, aVnl, avl2);
    } else if ((sl < wn) && (wn <= sr)) {
        if (!hllc) {
            const T fac1 = sr - wn, fac2 = sl - wn, fac3 = sr - sl;
            const T el = ((T(0.5) * _dl) * vl_sq) + (_pl / (gamma - T(1.0)));
            const T er = ((T(0.5) * _dr) * vr_sq) + (_pr / (gamma - T(1.0)));
            T f[4];
            f[0] = (((((_dl * Vnl) * fac1) - ((_dr * Vnr) * fac2)) - ((sl * _dl) * fac1)) + ((sr * _dr) * fac2)) / fac3;
            for (int k = 0; k < 2; k++)
                f[1 + k] = ((((((((_dl * vl[k]) * Vnl) + (_pl * n[k])) * fac1) - ((((_dr * vr[k]) * Vnr) + (_pr * n[k])) * fac2)) -
                             ((sl * (_dl * vl[k])) * fac1)) + ((sr * (_dr * vr[k])) * fac2))) / fac3;
            f[3] = ((((((el + _pl) * Vnl) * fac1) - (((er + _pr) * Vnr) * fac2)) - ((sl * el) * fac1)) + ((sr * er) * fac2)) / fac3;
            T af1 = 0, af2 = 0, af3 = 0;
            for (int q = 0; q < 4; q++) af3 -= aF[q] * f[q] / fac3;
            const T aNm = aF[0] / fac3;
            adl += aNm * fac1 * (Vnl - sl);
            aVnl += aNm * _dl * fac1;
            af1 += aNm * _dl * (Vnl - sl);
            adr += aNm * fac2 * (sr - Vnr);
            aVnr -= aNm * _dr * fac2;
            af2 += aNm * _dr * (sr - Vnr);
            asl -= aNm * _dl * fac1;
            asr += aNm * _dr * fac2;
            for (int k = 0; k < 2; k++) {
                const T aNk = aF[1 + k] / fac3;
                adl += aNk * vl[k] * fac1 * (Vnl - sl);
                avl[k] += aNk * _dl * fac1 * (Vnl - sl);
                aVnl += aNk * _dl * vl[k] * fac1;
                apl += aNk * n[k] * fac1;
                af1 += aNk * (_dl * vl[k] * Vnl + _pl * n[k] - sl * _dl * vl[k]);
                adr += aNk * vr[k] * fac2 * (sr - Vnr);
                avr[k] += aNk * _dr * fac2 * (sr - Vnr);
                aVnr -= aNk * _dr * vr[k] * fac2;
                apr -= aNk * n[k] * fac2;
                af2 += aNk * (-(_dr * vr[k] * Vnr + _pr * n[k]) + sr * _dr * vr[k]);
                asl -= aNk * _dl * vl[k] * fac1;
                asr += aNk * _dr * vr[k] * fac2;
            }
            const T aNe = aF[3] / fac3;
            const T ael = aNe * fac1 * (Vnl - sl);
            apl += aNe * Vnl * fac1;
            aVnl += aNe * (el + _pl) * fac1;
            af1 += aNe * ((el + _pl) * Vnl - sl * el);
            const T aer = aNe * fac2 * (sr - Vnr);
            apr -= aNe * Vnr * fac2;
            aVnr -= aNe * (er + _pr) * fac2;
            af2 += aNe * (-(er + _pr) * Vnr + sr * er);
            asl -= aNe * el * fac1;
            asr += aNe * er * fac2;
            adl += ael * T(0.5) * vl_sq;
            avl2 += ael * T(0.5) * _dl;
            apl += ael / (gamma - T(1.0));
            adr += aer * T(0.5) * vr_sq;
            avr2 += aer * T(0.5) * _dr;
            apr += aer / (gamma - T(1.0));
            asr += af1 + af3;
            asl += af2 - af3;
        } else {
            // one star-state adjoint for either side of the contact (no divergence)
            const bool left = wn <= sc;
            const T vs[2] = {left ? vl[0] : vr[0], left ? vl[1] : vr[1]};
            T ad = 0, av[2] = {0, 0}, ap = 0, aVn = 0, av2 = 0, as = 0;
            star_flux_adj<T>(left ? _dl : _dr, vs, left ? _pl : _pr, left ? Vnl : Vnr, left ? vl_sq : vr_sq,
                             left ? sl : sr, sc, n, wn, gamma, aF, ad, av, ap, aVn, av2, as, asc);
            const T kl = left ? T(1) : T(0), kr = T(1) - kl;
            adl += kl * ad; adr += kr * ad;
            avl[0] += kl * av[0]; avr[0] += kr * av[0];
            avl[1] += kl * av[1]; avr[1] += kr * av[1];
            apl += kl * ap; apr += kr * ap;
            aVnl += kl * aVn; aVnr += kr * aVn;
            avl2 += kl * av2; avr2 += kr * av2;
            asl += kl * as; asr += kr * as;
        }
    } else {
        data_flux_adj<T>(_dr, vr, _pr, Vnr, vr_sq, n, wn, gamma, aF, adr, avr, apr, aVnr, avr2);
    }
    if (asl != T(0) || asc != T(0) || asr != T(0))
        get_waves_rev<T>(wt, _dl, Vnl, _pl, _dr, Vnr, _pr, gamma, asl, asc, asr, adl, aVnl, apl, adr, aVnr, apr);
    aL[0] += adl;
    aL[3] += apl;
    aR[0] += adr;
    aR[3] += apr;
    for (int k = 0; k < 2; k++) {
        aL[1 + k] += avl[k] + aVnl * n[k] + T(2.) * vl[k] * avl2;
        aR[1 + k] += avr[k] + aVnr * n[k] + T(2.) * vr[k] * avr2;
    }
}

// ---- Exact Riemann solver (riemann.pyx:700-1090), FP64 --------------------------------
// Partial derivatives of the pressure function f_K(p) of ex_p_func (riemann.pyx:1015-1040)
// in p and in the side's data (d_K, p_K, c_K), c_K treated as its own input:
//   rarefaction (p <= p_K): f = 2 c/(g-1) ((p/p_K)^z - 1), z = (g-1)/(2g);
//   shock (p > p_K): f = (p - p_K) sqrt(A/(p + B)), A = 2/((g+1) d_K), B = (g-1) p_K/(g+1).
PHD_HD __forceinline__ void ex_p_func_partials(double d, double pk, double c, double gamma, double p,
                                               double &f_p, double &f_d, double &f_pk, double &f_c) {
    if (p <= pk) {
        const double z = (gamma - 1.) / (2. * gamma);
        const double q = p / pk;
        const double qz = pow(q, z);
        f_c = (2. / (gamma - 1.)) * (qz - 1.);
        f_pk = -((c / gamma) * qz) / pk;
        f_d = 0.;
        f_p = ((c / gamma) * (qz / q)) / pk;
    } else {
        const double A = 2. / (d * (gamma + 1.));
        const double B = (pk * (gamma - 1.)) / (gamma + 1.);
        const double s = sqrt(A / (p + B));
        const double ds = -0.5 * s / (p + B);              // d s / d(p + B)
        f_p = s + (p - pk) * ds;
        f_pk = -s + (p - pk) * ds * ((gamma - 1.) / (gamma + 1.));
        f_d = -0.5 * (p - pk) * s / d;
        f_c = 0.;
    }
}

// Adjoint of exact_flux<double, 2> (the FP64 path's solver: ex_get_pstar, ex_p_func at
// p*, sampling at xi = 0 in the face frame, deboost).  The forward is recomputed with the
// same arithmetic, so every branch (rarefaction / shock per side, the sampled region) is
// the forward's; p* enters through the implicit function F(p*) = f_L(p*) + f_R(p*) +
// (u_R - u_L) = 0 at the converged root: dp* = -dF / F'(p*).  aF: adjoint of the
// deboosted flux; accumulates into aL, aR.
PHD_HD void exact_flux_adj(const double *L, const double *R, const double *n, const double *w, double gamma,
                           int max_iter, const double *aFin, double *aL, double *aR) {
    const double _dl = L[0], _pl = L[3], _dr = R[0], _pr = R[3];
    const double cl = sqrt((gamma * _pl) / _dl), cr = sqrt((gamma * _pr) / _dr);
    double vnl = 0., vnr = 0.;
    for (int k = 0; k < 2; k++) {
        vnl = vnl + L[1 + k] * n[k];
        vnr = vnr + R[1 + k] * n[k];
    }
    bool failed = false;
    const double p_star = ex_get_pstar(_dl, vnl, _pl, cl, _dr, vnr, _pr, cr, gamma, max_iter, &failed);
    const double fl_d = ex_p_func(_dl, _pl, cl, gamma, p_star);
    const double fr_d = ex_p_func(_dr, _pr, cr, gamma, p_star);
    const double u_star = 0.5 * (((vnl + vnr) + fr_d) - fl_d);
    const double g1 = gamma - 1., gp = gamma + 1.;
    // sampling (the forward's branch, with what its reverse needs)
    int kind = 0, how = 0;     // kind 0/1: left/right data; 2: sampled; how: 1 raref. star, 2 fan, 3 shock star
    bool right = false;
    double _d = 0., _p = 0., ushift = 0., c_fan = 0.;
    if (0. <= u_star) {
        if (p_star <= _pl) {
            if (!(0. <= vnl - cl)) {
                const double c_star_l = cl * pow(p_star / _pl, g1 / (2. * gamma));
                if (0. >= u_star - c_star_l) {
                    kind = 2; how = 1; _d = _dl * pow(p_star / _pl, 1. / gamma); _p = p_star; ushift = u_star - vnl;
                } else {
                    c_fan = (2. / gp) * (cl + ((0.5 * g1) * vnl));
                    kind = 2; how = 2; _d = _dl * pow(c_fan / cl, 2. / g1);
                    _p = _pl * pow(c_fan / cl, (2. * gamma) / g1); ushift = c_fan - vnl;
                }
            }
        } else {
            const double sl = vnl - (cl * sqrt((((gp * p_star) / ((2. * gamma) * _pl)) + (g1 / (2. * gamma)))));
            if (!(0. <= sl)) {
                kind = 2; how = 3;
                _d = (_dl * ((p_star / _pl) + (g1 / gp))) / (((p_star * g1) / (gp * _pl)) + 1.);
                _p = p_star; ushift = u_star - vnl;
            }
        }
    } else {
        right = true;
        kind = 1;
        if (p_star >= _pr) {
            const double sr = vnr + (cr * sqrt((((gp * p_star) / ((2. * gamma) * _pr)) + (g1 / (2. * gamma)))));
            if (!(0. >= sr)) {
                kind = 2; how = 3;
                _d = (_dr * ((p_star / _pr) + (g1 / gp))) / (((p_star * g1) / (gp * _pr)) + 1.);
                _p = p_star; ushift = u_star - vnr;
            }
        } else {
            if (!(0. >= vnr + cr)) {
                const double c_star_r = cr * pow(p_star / _pr, g1 / (2. * gamma));
                if (0. <= u_star + c_star_r) {
                    kind = 2; how = 1; _d = _dr * pow(p_star / _pr, 1. / gamma); _p = p_star; ushift = u_star - vnr;
                } else {
                    c_fan = (2. / gp) * (cr - ((0.5 * g1) * vnr));
                    kind = 2; how = 2; _d = _dr * pow(c_fan / cr, 2. / g1);
                    _p = _pr * pow(c_fan / cr, (2. * gamma) / g1);
                    ushift = ((2. / gp) * ((-cr) + ((0.5 * g1) * vnr))) - vnr;
                }
            }
        }
    }
    // deboost reverse (the exact solver always boosts)
    double aF[4];
    aF[0] = aFin[0] + w[0] * aFin[1] + w[1] * aFin[2] + 0.5 * (w[0] * w[0] + w[1] * w[1]) * aFin[3];
    aF[1] = aFin[1] + w[0] * aFin[3];
    aF[2] = aFin[2] + w[1] * aFin[3];
    aF[3] = aFin[3];
    // adjoints of the side data (d, p, c, vn, velocity) and of p*, u*
    double a_d[2] = {0., 0.}, a_p[2] = {0., 0.}, a_c[2] = {0., 0.}, a_vn[2] = {0., 0.};
    double a_v[2][2] = {{0., 0.}, {0., 0.}};
    double a_ps = 0., a_us = 0.;
    const double *side[2] = {L, R};
    const double dK[2] = {_dl, _dr}, pK[2] = {_pl, _pr}, cK[2] = {cl, cr}, vnK[2] = {vnl, vnr};
    if (kind != 2) {                                   // one side's data flux
        const int s = kind;
        const double vs[2] = {side[s][1], side[s][2]};
        const double v2 = vs[0] * vs[0] + vs[1] * vs[1];
        double ad = 0., av[2] = {0., 0.}, ap = 0., aVn = 0., av2 = 0.;
        data_flux_adj<double>(dK[s], vs, pK[s], vnK[s], v2, n, 0., gamma, aF, ad, av, ap, aVn, av2);
        a_d[s] += ad; a_p[s] += ap; a_vn[s] += aVn;
        for (int k = 0; k < 2; k++) a_v[s][k] += av[k] + 2. * vs[k] * av2;
    } else {
        const int s = right ? 1 : 0;
        double v[2], vn = 0., v_sq = 0.;
        for (int k = 0; k < 2; k++) {
            v[k] = side[s][1 + k] + (ushift * n[k]);
            vn = vn + v[k] * n[k];
            v_sq = v_sq + v[k] * v[k];
        }
        double ad = 0., av[2] = {0., 0.}, ap = 0., aVn = 0., av2 = 0.;
        data_flux_adj<double>(_d, v, _p, vn, v_sq, n, 0., gamma, aF, ad, av, ap, aVn, av2);
        double a_ush = 0.;
        for (int k = 0; k < 2; k++) {
            const double avk = av[k] + aVn * n[k] + 2. * v[k] * av2;
            a_v[s][k] += avk;
            a_ush += avk * n[k];
        }
        const double dk = dK[s], pk = pK[s], ck = cK[s];
        if (how == 1) {                                // rarefaction star: d = d_K (p*/p_K)^(1/g)
            const double q = p_star / pk;
            const double aq = ad * dk * (1. / gamma) * pow(q, 1. / gamma - 1.);
            a_d[s] += ad * pow(q, 1. / gamma);
            a_ps += aq / pk + ap;
            a_p[s] += -aq * q / pk;
            a_us += a_ush;
            a_vn[s] -= a_ush;
        } else if (how == 3) {                         // shock star
            const double q = p_star / pk, gg = g1 / gp;
            const double num = dk * (q + gg), den = gg * q + 1.;
            const double anum = ad / den, aden = -ad * num / (den * den);
            a_d[s] += anum * (q + gg);
            const double aq = anum * dk + aden * gg;
            a_ps += aq / pk + ap;
            a_p[s] += -aq * q / pk;
            a_us += a_ush;
            a_vn[s] -= a_ush;
        } else {                                       // inside the rarefaction fan
            const double r = c_fan / ck, e1 = 2. / g1, e2 = (2. * gamma) / g1;
            const double ar = ad * dk * e1 * pow(r, e1 - 1.) + ap * pk * e2 * pow(r, e2 - 1.);
            a_d[s] += ad * pow(r, e1);
            a_p[s] += ap * pow(r, e2);
            double a_cfan = ar / ck;
            a_c[s] += -ar * c_fan / (ck * ck);
            if (s == 0) {                              // c = 2/(g+1) (c_L + (g-1)/2 u_L); shift = c - u_L
                a_cfan += a_ush;
                a_vn[0] -= a_ush;
                a_c[0] += a_cfan * (2. / gp);
                a_vn[0] += a_cfan * (2. / gp) * (0.5 * g1);
            } else {                                   // c = 2/(g+1) (c_R - (g-1)/2 u_R);
                a_c[1] += a_cfan * (2. / gp);          // shift = 2/(g+1) (-c_R + (g-1)/2 u_R) - u_R
                a_vn[1] += -a_cfan * (2. / gp) * (0.5 * g1);
                a_c[1] += -a_ush * (2. / gp);
                a_vn[1] += a_ush * ((2. / gp) * (0.5 * g1) - 1.);
            }
        }
    }
    // u* = ((u_L + u_R) + f_R(p*) - f_L(p*)) / 2
    double fpL, fdL, fpkL, fcL, fpR, fdR, fpkR, fcR;
    ex_p_func_partials(_dl, _pl, cl, gamma, p_star, fpL, fdL, fpkL, fcL);
    ex_p_func_partials(_dr, _pr, cr, gamma, p_star, fpR, fdR, fpkR, fcR);
    if (a_us != 0.) {
        a_vn[0] += 0.5 * a_us;
        a_vn[1] += 0.5 * a_us;
        const double afr = 0.5 * a_us, afl = -0.5 * a_us;
        a_ps += afr * fpR + afl * fpL;
        a_d[0] += afl * fdL; a_p[0] += afl * fpkL; a_c[0] += afl * fcL;
        a_d[1] += afr * fdR; a_p[1] += afr * fpkR; a_c[1] += afr * fcR;
    }
    // p*: the converged root of F(p) = f_L(p) + f_R(p) + (u_R - u_L)
    if (a_ps != 0.) {
        const double sgm = a_ps / (fpL + fpR);
        a_vn[0] += sgm;
        a_vn[1] -= sgm;
        a_d[0] -= sgm * fdL; a_p[0] -= sgm * fpkL; a_c[0] -= sgm * fcL;
        a_d[1] -= sgm * fdR; a_p[1] -= sgm * fpkR; a_c[1] -= sgm * fcR;
    }
    // c_K = sqrt(g p_K / d_K), u_K = v_K . n
    for (int s = 0; s < 2; s++) {
        double *aS = s == 0 ? aL : aR;
        a_p[s] += a_c[s] * 0.5 * cK[s] / pK[s];
        a_d[s] += -a_c[s] * 0.5 * cK[s] / dK[s];
        aS[0] += a_d[s];
        aS[3] += a_p[s];
        for (int k = 0; k < 2; k++) aS[1 + k] += a_v[s][k] + a_vn[s] * n[k];
    }
}

// Adjoint of the GIZMO pair limit of one field (gizmo_pair in phd_physics.cuh).
// Returns adjoints of (sl, sr, xl, xr) given adjoints of the limited (xl, xr).
// si = |sep_i| / |x_j - x_i|, sj = |sep_j| / |x_j - x_i| (the same quotients the forward
// limiter forms, computed once per face by the caller).
template <typename T>
PHD_HD __forceinline__ void gizmo_pair_adj_q(T sl, T sr, T ci, T cj, T si, T sj, T xl, T xr, T axl_out,
                                                 T axr_out, T &asl, T &asr, T &axl, T &axr) {
    const T diff = sl - sr;
    const T sgn = diff > T(0) ? T(1) : (diff < T(0) ? T(-1) : T(0));
    const T delta1 = T(0.5) * t_fabs(diff), delta2 = T(0.25) * t_fabs(diff);
    const bool a_is_min = !(sr < sl);          // fmin(sl, sr) -> sl when sl <= sr
    const T phi_min = t_fmin(sl, sr), phi_max = t_fmax(sl, sr);
    const T phibar_l = sl + si * (sr - sl), phibar_r = sr + sj * (sl - sr);
    const bool plus_lin = ((phi_max + delta1) * phi_max) >= T(0.);
    const bool minus_lin = ((phi_min - delta1) * phi_min) >= T(0.);
    const T phi_plus = plus_lin ? phi_max + delta1 : phi_max / (T(1) + (delta1 / t_fabs(phi_max)));
    const T phi_minus = minus_lin ? phi_min - delta1 : phi_min / (T(1) + (delta1 / t_fabs(phi_min)));
    T a_pp = 0, a_pm = 0, a_bl = 0, a_br = 0, a_d2 = 0;
    if (ci < cj) {
        // xl = max(phi_minus, min(bl + d2, x)); xr = min(phi_plus, max(br - d2, y))
        const T inner = t_fmin(phibar_l + delta2, xl);
        if (phi_minus >= inner) a_pm += axl_out;
        else if (phibar_l + delta2 <= xl) { a_bl += axl_out; a_d2 += axl_out; }
        else axl += axl_out;
        const T inr = t_fmax(phibar_r - delta2, xr);
        if (phi_plus <= inr) a_pp += axr_out;
        else if (phibar_r - delta2 >= xr) { a_br += axr_out; a_d2 -= axr_out; }
        else axr += axr_out;
    } else if (ci > cj) {
        // xl = min(phi_plus, max(bl - d2, x)); xr = max(phi_minus, min(br + d2, y))
        const T inner = t_fmax(phibar_l - delta2, xl);
        if (phi_plus <= inner) a_pp += axl_out;
        else if (phibar_l - delta2 >= xl) { a_bl += axl_out; a_d2 -= axl_out; }
        else axl += axl_out;
        const T inr = t_fmin(phibar_r + delta2, xr);
        if (phi_minus >= inr) a_pm += axr_out;
        else if (phibar_r + delta2 <= xr) { a_br += axr_out; a_d2 += axr_out; }
        else axr += axr_out;
    } else {
        asl += axl_out;
        asr += axr_out;
        return;
    }
    T a_d1 = 0, a_pmax = 0, a_pmin = 0;
    if (plus_lin) { a_pmax += a_pp; a_d1 += a_pp; }
    else {
        const T q = T(1) + delta1 / t_fabs(phi_max);
        a_pmax += a_pp * (T(1) / q + delta1 / (q * q * t_fabs(phi_max)));
        const T sg = phi_max > T(0) ? T(1) : T(-1);
        a_d1 -= a_pp * sg / (q * q);
    }
    if (minus_lin) { a_pmin += a_pm; a_d1 -= a_pm; }
    else {
        const T q = T(1) + delta1 / t_fabs(phi_min);
        a_pmin += a_pm * (T(1) / q + delta1 / (q * q * t_fabs(phi_min)));
        const T sg = phi_min > T(0) ? T(1) : T(-1);
        a_d1 -= a_pm * sg / (q * q);
    }
    // phibar_l = sl + si (sr - sl); phibar_r = sr + sj (sl - sr)
    asl += a_bl * (T(1) - si) + a_br * sj;
    asr += a_bl * si + a_br * (T(1) - sj);
    // delta1 = |sl - sr| / 2, delta2 = |sl - sr| / 4
    const T ad = T(0.5) * a_d1 + T(0.25) * a_d2;
    asl += ad * sgn;
    asr -= ad * sgn;
    if (a_is_min) { asl += a_pmin; asr += a_pmax; }
    else { asr += a_pmin; asl += a_pmax; }
}

template <typename T>
PHD_HD __forceinline__ void gizmo_pair_adj(T sl, T sr, T ci, T cj, T smi, T smj, T dm, T xl, T xr, T axl_out,
                                               T axr_out, T &asl, T &asr, T &axl, T &axr) {
    gizmo_pair_adj_q<T>(sl, sr, ci, cj, smi / dm, smj / dm, xl, xr, axl_out, axr_out, asl, asr, axl, axr);
}

// Adjoint of the 2D temporal extrapolation (temporal<T,2>).  Lin/Rin are the states
// entering it (spatial result); aL/aR the adjoints of its outputs; accumulates into
// aLin/aRin and the cell-value / gradient adjoints.
template <typename T>
PHD_HD void temporal_adj(const T *Lin, const T *Rin, const T *pi, const T *pj, const T *gi, const T *gj,
                             const T *w, T gamma, T dt, bool boost, const T *aL, const T *aR, T *aLin, T *aRin,
                             T *api, T *apj, T *agi, T *agj) {
    // forward (for the revert decisions)
    T L[4], R[4];
    for (int f = 0; f < 4; f++) { L[f] = Lin[f]; R[f] = Rin[f]; }
    temporal<T, 2>(L, R, pi, pj, gi, gj, w, gamma, dt, boost);
    // a side reverted to its input exactly when its output equals its input and the
    // time-extrapolated density or pressure was negative; recompute that test
    const T *sides_p[2] = {pi, pj};
    const T *sides_g[2] = {gi, gj};
    const T *ins[2] = {Lin, Rin};
    const T *as[2] = {aL, aR};
    T *ains[2] = {aLin, aRin};
    T *aps[2] = {api, apj};
    T *ags[2] = {agi, agj};
    for (int s = 0; s < 2; s++) {
        const T *p = sides_p[s];
        const T *g = sides_g[s];
        const T *in = ins[s];
        const T *a = as[s];
        T *ain = ains[s];
        T *ap = aps[s];
        T *ag = ags[s];
        T v[2];
        for (int k = 0; k < 2; k++) v[k] = boost ? p[1 + k] - w[k] : p[1 + k];
        // time-extrapolated density / pressure (same order as temporal<>)
        T Ld = in[0], Lp = in[3];
        for (int k = 0; k < 2; k++) {
            const T div = g[2 + 3 * k];
            Ld = Ld - (dt * ((p[0] * div) + (v[k] * g[k])));
            Lp = Lp - (dt * (((gamma * p[3]) * div) + (v[k] * g[6 + k])));
        }
        if (Ld < T(0.0) || Lp < T(0.0)) {
            for (int f = 0; f < 4; f++) ain[f] += a[f];
            continue;
        }
        for (int f = 0; f < 4; f++) ain[f] += a[f];
        T av[2] = {0, 0};
        for (int c = 0; c < 2; c++) {
            const T aVc = a[1 + c];
            ag[6 + c] -= dt / p[0] * aVc;
            ap[0] += dt * g[6 + c] / (p[0] * p[0]) * aVc;
            for (int k = 0; k < 2; k++) {
                av[k] -= dt * g[2 + 2 * c + k] * aVc;
                ag[2 + 2 * c + k] -= dt * v[k] * aVc;
            }
        }
        for (int k = 0; k < 2; k++) {
            const int dk = 2 + 3 * k;
            ap[0] -= dt * g[dk] * a[0];
            ag[dk] -= dt * p[0] * a[0];
            av[k] -= dt * g[k] * a[0];
            ag[k] -= dt * v[k] * a[0];
            ap[3] -= dt * gamma * g[dk] * a[3];
            ag[dk] -= dt * gamma * p[3] * a[3];
            av[k] -= dt * g[6 + k] * a[3];
            ag[6 + k] -= dt * v[k] * a[3];
        }
        ap[1] += av[0];
        ap[2] += av[1];
    }
}

}  // namespace phd
