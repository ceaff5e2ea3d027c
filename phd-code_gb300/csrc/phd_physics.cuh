// phd_physics.cuh -- per-face / per-cell physics of the flux path as device functions.
//
// Each function restates one routine of the reference with the reference's operation
// order, templated on the arithmetic type T:
//   T = double : the FP64 path (compiled without FMA contraction) reproduces the
//                reference's Cython arithmetic up to libm-vs-CUDA pow/sqrt rounding;
//   T = float  : the FP32 path (spec precision split).
// Field order: prim [rho, v_0..v_{DIM-1}, p], flux [mass, mom_0.., energy].
#pragma once
#include "phd_common.cuh"

namespace phd {

// HLL.get_waves riemann.pyx:375-504 (PVRS guess, TRRS/TSRS switch Q = 2, sound-speed
// floor 1e-10, Toro eq. 10.68-10.70).
template <typename T>
PHD_HD __forceinline__ void get_waves(T dl, T ul, T pl, T dr, T ur, T pr, T gamma,
                                          T &sl, T &sc, T &sr) {
    const T Q = T(2.), c_floor = T(1.0E-10);
    T p_star;
    const T cl = t_fmax(t_sqrt((gamma * pl) / dl), c_floor);
    const T cr = t_fmax(t_sqrt((gamma * pr) / dr), c_floor);
    const T d_avg = T(.5) * (dl + dr);
    const T c_avg = T(.5) * (cl + cr);
    p_star = t_fmax(T(0.), ((T(.5) * (pl + pr)) + (((T(.5) * (ul - ur)) * d_avg) * c_avg)));
    const T p_min = t_fmin(pl, pr);
    const T p_max = t_fmax(pl, pr);
    if (((p_max / p_min) < Q) && ((p_min < p_star) && (p_star < p_max))) {
        // PVRS estimate stands (u_star is not used by the wave speeds)
    } else if (p_star <= p_min) {
        const T z = (gamma - T(1.)) / (T(2.) * gamma);
        const T plr = t_pow(pl / pr, z);
        const T u_star = ((((plr * ul) / cl) + (ur / cr)) + ((T(2.) * (plr - T(1.))) / (gamma - T(1.)))) /
                         ((plr / cl) + (T(1.) / cr));
        p_star = (T(.5) * pl) * t_pow((T(1.) + (((gamma - T(1.)) * (ul - u_star)) / (T(2.) * cl))), (T(1.) / z));
        p_star = p_star + ((T(.5) * pr) * t_pow((T(1.) + (((gamma - T(1.)) * (u_star - ur)) / (T(2.) * cr))), (T(1.) / z)));
    } else {
        const T Al = T(2.) / ((gamma + T(1.)) * dl);
        const T Ar = T(2.) / ((gamma + T(1.)) * dr);
        const T Bl = pl * ((gamma - T(1.)) / (gamma + T(1.)));
        const T Br = pr * ((gamma - T(1.)) / (gamma + T(1.)));
        const T gl = t_sqrt(Al / (p_star + Bl));
        const T gr = t_sqrt(Ar / (p_star + Br));
        p_star = (((gl * pl) + (gr * pr)) - (ur - ul)) / (gl + gr);
    }
    if (p_star <= pl) sl = ul - cl;
    else sl = ul - (cl * t_sqrt((T(1.) + (((gamma + T(1.)) / (T(2.) * gamma)) * ((p_star / pl) - T(1.))))));
    if (p_star <= pr) sr = ur + cr;
    else sr = ur + (cr * t_sqrt((T(1.) + (((gamma + T(1.)) / (T(2.) * gamma)) * ((p_star / pr) - T(1.))))));
    sc = (((pr - pl) + ((dl * ul) * (sl - ul))) - ((dr * ur) * (sr - ur))) /
         ((dl * (sl - ul)) - (dr * (sr - ur)));
}

// RiemannBase.deboost riemann.pyx:190-222 (Pakmor & Springel 2011 eq. 17).
template <typename T, int DIM>
PHD_HD __forceinline__ void deboost(const T *w, T *f) {
#pragma unroll
    for (int k = 0; k < DIM; k++) {
        f[DIM + 1] = f[DIM + 1] + (w[k] * (((T(0.5) * w[k]) * f[0]) + f[1 + k]));
        f[1 + k] = f[1 + k] + (w[k] * f[0]);
    }
}

// HLL.riemann_solver riemann.pyx:243-373 (hllc = false) and HLLC.riemann_solver
// riemann.pyx:521-682 (hllc = true); L/R are face states, n the unit normal, w the
// face velocity.  Velocities stay in lab axes; only v.n enters the wave structure.
template <typename T, int DIM>
PHD_HD __forceinline__ void hll_family(bool hllc, const T *L, const T *R, const T *n,
                                           const T *w, T gamma, bool boost, T *f) {
    const int E = DIM + 1;
    const T _dl = L[0], _pl = L[E], _dr = R[0], _pr = R[E];
    T Vnl = T(0.0), Vnr = T(0.0), vl_sq = T(0.0), vr_sq = T(0.0), wn = T(0.0);
#pragma unroll
    for (int k = 0; k < DIM; k++) {
        vl_sq = vl_sq + L[1 + k] * L[1 + k];
        vr_sq = vr_sq + R[1 + k] * R[1 + k];
        Vnl = Vnl + L[1 + k] * n[k];
        Vnr = Vnr + R[1 + k] * n[k];
        wn = wn + w[k] * n[k];
    }
    if (boost) wn = T(0.);
    T sl, sc, sr;
    get_waves<T>(_dl, Vnl, _pl, _dr, Vnr, _pr, gamma, sl, sc, sr);
    if (wn <= sl) {
        f[0] = _dl * (Vnl - wn);
        f[E] = ((((T(0.5) * _dl) * vl_sq) + (_pl / (gamma - T(1.0)))) * (Vnl - wn)) + (_pl * Vnl);
#pragma unroll
        for (int k = 0; k < DIM; k++) f[1 + k] = ((_dl * L[1 + k]) * (Vnl - wn)) + (_pl * n[k]);
    } else if ((sl < wn) && (wn <= sr)) {
        if (!hllc) {
            const T fac1 = sr - wn, fac2 = sl - wn, fac3 = sr - sl;
            f[0] = (((((_dl * Vnl) * fac1) - ((_dr * Vnr) * fac2)) - ((sl * _dl) * fac1)) + ((sr * _dr) * fac2)) / fac3;
#pragma unroll
            for (int k = 0; k < DIM; k++) {
                const T vl = L[1 + k], vr = R[1 + k];
                f[1 + k] = ((((((((_dl * vl) * Vnl) + (_pl * n[k])) * fac1) -
                               ((((_dr * vr) * Vnr) + (_pr * n[k])) * fac2)) -
                              ((sl * (_dl * vl)) * fac1)) + ((sr * (_dr * vr)) * fac2))) / fac3;
            }
            const T el = ((T(0.5) * _dl) * vl_sq) + (_pl / (gamma - T(1.0)));
            const T er = ((T(0.5) * _dr) * vr_sq) + (_pr / (gamma - T(1.0)));
            f[E] = ((((((el + _pl) * Vnl) * fac1) - (((er + _pr) * Vnr) * fac2)) - ((sl * el) * fac1)) +
                    ((sr * er) * fac2)) / fac3;
        } else if (wn <= sc) {
            const T factor_1 = (_dl * (sl - Vnl)) / (sl - sc);
            const T factor_2 = ((factor_1 * (sl - wn)) * (sc - Vnl)) + _pl;
            const T frho = (_dl * (Vnl - sl)) + (factor_1 * (sl - wn));
            const T el = ((T(0.5) * _dl) * vl_sq) + (_pl / (gamma - T(1.0)));
            f[0] = frho;
            f[E] = (((el + _pl) * Vnl) - (sl * el)) +
                   (((sl - wn) * factor_1) * ((el / _dl) + ((sc - Vnl) * (sc + (_pl / (_dl * (sl - Vnl)))))));
#pragma unroll
            for (int k = 0; k < DIM; k++) f[1 + k] = (frho * L[1 + k]) + (factor_2 * n[k]);
        } else {
            const T factor_1 = (_dr * (sr - Vnr)) / (sr - sc);
            const T factor_2 = ((factor_1 * (sr - wn)) * (sc - Vnr)) + _pr;
            const T frho = (_dr * (Vnr - sr)) + (factor_1 * (sr - wn));
            const T er = ((T(0.5) * _dr) * vr_sq) + (_pr / (gamma - T(1.0)));
            f[0] = frho;
            f[E] = (((er + _pr) * Vnr) - (sr * er)) +
                   (((sr - wn) * factor_1) * ((er / _dr) + ((sc - Vnr) * (sc + (_pr / (_dr * (sr - Vnr)))))));
#pragma unroll
            for (int k = 0; k < DIM; k++) f[1 + k] = (frho * R[1 + k]) + (factor_2 * n[k]);
        }
    } else {
        f[0] = _dr * (Vnr - wn);
        f[E] = ((((T(0.5) * _dr) * vr_sq) + (_pr / (gamma - T(1.0)))) * (Vnr - wn)) + (_pr * Vnr);
#pragma unroll
        for (int k = 0; k < DIM; k++) f[1 + k] = ((_dr * R[1 + k]) * (Vnr - wn)) + (_pr * n[k]);
    }
    if (boost) deboost<T, DIM>(w, f);
}

// ---- Exact solver: Newton iteration on p* always in FP64 (riemann.pyx:974-1090) ----
PHD_HD __forceinline__ double ex_p_guess(double dl, double ul, double pl, double cl, double dr,
                                             double ur, double pr, double cr, double gamma) {
    const double ppv = (.5 * (pl + pr)) - (((.125 * (ur - ul)) * (dl + dr)) * (cl + cr));
    const double p_max = (pr > pl) ? pr : pl;
    const double p_min = (pr < pl) ? pr : pl;
    const double q_max = p_max / p_min;
    if ((q_max <= 2.) && (p_min <= ppv && ppv <= p_max)) return ppv;
    if (ppv <= p_min) {
        const double p_lr = pow(pl / pr, (gamma - 1.) / (2. * gamma));
        double u_star = (((p_lr * ul) / cl) + (ur / cr)) + ((2. * (p_lr - 1.)) / (gamma - 1.));
        u_star = u_star / ((p_lr / cl) + (1. / cr));
        const double p_tl = pow((1. + (((gamma - 1.) * (ul - u_star)) / (2. * cl))), ((2. * gamma) / (gamma - 1.)));
        const double p_tr = pow((1. + (((gamma - 1.) * (u_star - ur)) / (2. * cr))), ((2. * gamma) / (gamma - 1.)));
        return .5 * ((pl * p_tl) + (pr * p_tr));
    }
    const double gl = sqrt((2. / (dl * (gamma + 1.))) / ((((gamma - 1.) * pl) / (gamma + 1.)) + ppv));
    const double gr = sqrt((2. / (dr * (gamma + 1.))) / ((((gamma - 1.) * pr) / (gamma + 1.)) + ppv));
    return (((gl * pl) + (gr * pr)) - (ur - ul)) / (gr + gl);
}

PHD_HD __forceinline__ double ex_p_func(double d, double p, double c, double gamma, double p_old) {
    if (p_old <= p) return ((2. * c) / (gamma - 1.)) * (pow(p_old / p, (gamma - 1.) / (2. * gamma)) - 1.);
    const double Ak = 2. / (d * (gamma + 1.));
    const double Bk = (p * (gamma - 1.)) / (gamma + 1.);
    return (p_old - p) * sqrt(Ak / (p_old + Bk));
}

PHD_HD __forceinline__ double ex_p_func_deriv(double d, double p, double c, double gamma, double p_old) {
    if (p_old <= p) return pow(p_old / p, ((-(gamma + 1.)) / (2. * gamma))) / (c * d);
    const double Ak = 2. / (d * (gamma + 1.));
    const double Bk = (p * (gamma - 1.)) / (gamma + 1.);
    return sqrt(Ak / (p_old + Bk)) * (1. - ((.5 * (p_old - p)) / (Bk + p_old)));
}

// Returns p*; sets *failed when max_iter Newton steps did not converge.
PHD_HD __forceinline__ double ex_get_pstar(double dl, double ul, double pl, double cl, double dr,
                                               double ur, double pr, double cr, double gamma,
                                               int max_iter, bool *failed) {
    const double TOL = 1.0e-6;
    double p_old = ex_p_guess(dl, ul, pl, cl, dr, ur, pr, cr, gamma), p_new = p_old;
    for (int it = 0; it < max_iter; it++) {
        const double fl = ex_p_func(dl, pl, cl, gamma, p_old);
        const double fr = ex_p_func(dr, pr, cr, gamma, p_old);
        const double dfl = ex_p_func_deriv(dl, pl, cl, gamma, p_old);
        const double dfr = ex_p_func_deriv(dr, pr, cr, gamma, p_old);
        p_new = p_old - ((((fl + fr) + ur) - ul) / (dfl + dfr));
        if ((2. * fabs((p_new - p_old) / (p_new + p_old))) <= TOL) return p_new;
        if (p_new < 0.) p_new = TOL;
        p_old = p_new;
    }
    *failed = true;
    return p_new;
}

// The same Newton iteration for the FP32 path (its pressure iteration stays in FP64),
// arranged for GB300's narrow FP64 pipe, where each pow, division and square root is a
// long instruction sequence.  On the face states of smooth and shocked flows alike,
// 99% of faces converge after one Newton step, so the initial guess and the final
// evaluation at p* cost as much as the iteration itself; all three are trimmed:
//  * gamma-only constants (2/(g-1), 2/(g+1), (g-1)/(g+1), (g-1)/2, z = (g-1)/(2g),
//    1/z) come from the host (ExGas64);
//  * (1 + d)^z for |d| <= 1/64 is the binomial series sum_{k=0..8} C(z,k) d^k: for
//    0 < z < 1, |C(z,k)| <= z/k, so the dropped tail is below (1/9)(1/64)^9 / (1 - 1/64)
//    < 1e-17 relative -- FP64 rounding level;
//  * b^(1/z) in the two-rarefaction guess is a product of squarings when 1/z =
//    2g/(g-1) is an integer (5 for g = 5/3, 7 for g = 1.4), else pow;
//  * on a rarefaction side the function and its derivative share one power,
//    (p/p_K)^((-(g+1))/(2g)) = (p/p_K)^z * (p_K/p), and each side keeps the reciprocal
//    of the last pressure it evaluated with that power: the next evaluation multiplies
//    the power by (p_new/p_old)^z (series) when the ratio is within 1/64 of 1;
//  * on a shock side s(p) = sqrt(A_K/(p + B_K)) takes one division and gives
//    1/(p + B_K) = s^2 d (g+1)/2 without a second one; the final evaluation at p*
//    continues from the last Newton point, s(p*) = s(p_old) (1 + e)^(-1/2),
//    e = (p* - p_old)/(p_old + B_K), by its binomial series (six terms for
//    |e| <= 2^-12: tail below 1e-19);
//  * one reciprocal of the iterate per Newton step serves both sides, the shock-branch
//    guess takes one division and one square root per side, and the convergence test
//    2|dp|/(p_new + p_old) <= TOL is evaluated as 2|dp| <= TOL |p_new + p_old|;
//  * on the device every FP64 reciprocal and reciprocal square root of the iteration
//    is the hardware approximation (rcp.approx.ftz.f64, rsqrt.approx.ftz.f64) refined
//    by two Newton-Raphson steps (ex_rcp, ex_rsqrt): full FP64 precision for the
//    positive normal arguments the iteration takes, in a few fused multiply-adds
//    instead of the correctly rounded division and square root sequences.
// Results agree with ex_get_pstar to FP64 rounding of the guess (the converged p*
// within 1e-12 relative; iteration counts can differ by one only where the relative
// change sits within rounding of TOL).
// The FP32 path (exact_flux<float>) also starts the iteration from the guess formed in
// FP32 from its FP32 states (ex_p_guess32: the guess is an estimate, not part of the
// iteration; the FP64 guess stands in where the FP32 one is not positive and finite),
// and forms the side functions at p*, which only u* needs, from the last Newton step's
// values and slopes, f_K(p*) = f_K(p_old) + f_K'(p_old) (p* - p_old): converged to
// 2|dp| <= 1e-6 (p_old + p*), the dropped term (f_K'' dp^2 / 2) is below 1e-12 of
// f_K, far below the FP32 rounding of the sampled state.
struct ExGas64 {
    double two_gm1, two_gp1, gm1_gp1, gm1_2, gp1_2, z, inv_z;
    int n_inv_z;              // 1/z when it is an integer in [1, 64], else 0
    double c[9];              // C(z, k), k = 0..8
    double sq_two_gp1;        // sqrt(2/(g+1))
    float zf, inv_zf, two_gm1f, gm1_2f, gm1_gp1f, sq_two_gp1f;   // the same in FP32 (ex_p_guess32)
};

inline ExGas64 ex_gas64(double gamma) {
    ExGas64 X;
    X.two_gm1 = 2. / (gamma - 1.);
    X.two_gp1 = 2. / (gamma + 1.);
    X.gm1_gp1 = (gamma - 1.) / (gamma + 1.);
    X.gm1_2 = .5 * (gamma - 1.);
    X.gp1_2 = .5 * (gamma + 1.);
    X.z = (gamma - 1.) / (2. * gamma);
    X.inv_z = (2. * gamma) / (gamma - 1.);
    const double r = X.inv_z + 0.5;
    const int n = (r >= 1. && r < 65.) ? int(r) : 0;
    X.n_inv_z = (n > 0 && fabs(X.inv_z - double(n)) <= 1e-12 * X.inv_z) ? n : 0;
    X.sq_two_gp1 = sqrt(X.two_gp1);
    X.zf = (float)X.z;
    X.inv_zf = (float)X.inv_z;
    X.two_gm1f = (float)X.two_gm1;
    X.gm1_2f = (float)X.gm1_2;
    X.gm1_gp1f = (float)X.gm1_gp1;
    X.sq_two_gp1f = (float)X.sq_two_gp1;
    X.c[0] = 1.;
    for (int k = 1; k < 9; k++) X.c[k] = X.c[k - 1] * (X.z - double(k - 1)) / double(k);
    return X;
}

// 1/x and 1/sqrt(x) for positive normal x: on the device the hardware approximations
// refined by two Newton-Raphson steps, y <- y (2 - x y) and y <- y (3 - x y^2) / 2 (each
// squares the relative error, so the approximations' error reaches FP64 rounding),
// written as a small correction added to y, y + y e with e = 1 - x y, resp.
// e = 1/2 - (x/2) y^2, formed by fused multiply-adds so that the last rounding falls on
// the correction; on the host (the check program) IEEE division and square root.
PHD_HD __forceinline__ double ex_rcp(double x) {
#ifdef __CUDA_ARCH__
    double y;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
    double e = fma(-x, y, 1.0);
    y = fma(y, e, y);
    e = fma(-x, y, 1.0);
    return fma(y, e, y);
#else
    return 1.0 / x;
#endif
}

PHD_HD __forceinline__ double ex_rsqrt(double x) {
#ifdef __CUDA_ARCH__
    double y;
    asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
    const double h = 0.5 * x;
    double e = fma(-h * y, y, 0.5);
    y = fma(y, e, y);
    e = fma(-h * y, y, 0.5);
    return fma(y, e, y);
#else
    return 1.0 / sqrt(x);
#endif
}

constexpr double EX_NEAR_ONE = 0.015625;

// (1 + d)^z, |d| <= 1/64
PHD_HD __forceinline__ double ex_pow_near_one(const ExGas64 &X, double d) {
    double s = X.c[8];
#pragma unroll
    for (int k = 7; k >= 0; k--) s = fma(s, d, X.c[k]);
    return s;
}

// q^z: the series near 1, else pow
PHD_HD __forceinline__ double ex_pow_z(const ExGas64 &X, double q) {
    return (fabs(q - 1.) <= EX_NEAR_ONE) ? ex_pow_near_one(X, q - 1.) : pow(q, X.z);
}

// b^(1/z): squarings for an integer exponent, else pow
PHD_HD __forceinline__ double ex_pow_inv_z(const ExGas64 &X, double b) {
    int n = X.n_inv_z;
    if (n == 0) return pow(b, X.inv_z);
    double r = 1., x = b;
    while (n) {
        if (n & 1) r *= x;
        n >>= 1;
        if (n) x *= x;
    }
    return r;
}

// (1 + e)^(-1/2), |e| <= 2^-12
PHD_HD __forceinline__ double ex_rsqrt_near_one(double e) {
    return fma(fma(fma(fma(fma(-63. / 256., e, 35. / 128.), e, -5. / 16.), e, 3. / 8.), e, -.5), e, 1.);
}

// ex_p_guess with the gamma constants of X: PVRS, then the two-rarefaction (TRRS) or
// two-shock (TSRS) estimate (riemann.pyx p_guess, Toro 9.4.1-9.4.3).
PHD_HD __forceinline__ double ex_p_guess_lean(double dl, double ul, double pl, double cl, double dr, double ur,
                                              double pr, double cr, const ExGas64 &X) {
    const double ppv = (.5 * (pl + pr)) - (((.125 * (ur - ul)) * (dl + dr)) * (cl + cr));
    const double p_max = (pr > pl) ? pr : pl;
    const double p_min = (pr < pl) ? pr : pl;
    if ((p_max <= 2. * p_min) && (p_min <= ppv && ppv <= p_max)) return ppv;
    if (ppv <= p_min) {
        const double inv_cl = ex_rcp(cl), inv_cr = ex_rcp(cr);
        const double p_lr = ex_pow_z(X, pl * ex_rcp(pr));
        const double u_star = (((p_lr * ul) * inv_cl + ur * inv_cr) + X.two_gm1 * (p_lr - 1.)) *
                              ex_rcp(p_lr * inv_cl + inv_cr);
        const double p_tl = ex_pow_inv_z(X, 1. + (X.gm1_2 * (ul - u_star)) * inv_cl);
        const double p_tr = ex_pow_inv_z(X, 1. + (X.gm1_2 * (u_star - ur)) * inv_cr);
        return .5 * ((pl * p_tl) + (pr * p_tr));
    }
    const double gl = X.sq_two_gp1 * ex_rsqrt(dl * (X.gm1_gp1 * pl + ppv));
    const double gr = X.sq_two_gp1 * ex_rsqrt(dr * (X.gm1_gp1 * pr + ppv));
    return (((gl * pl) + (gr * pr)) - (ur - ul)) * ex_rcp(gr + gl);
}

#ifdef __CUDACC__
// ex_p_guess_lean in FP32 from the FP32 path's states (fast-math powers and
// reciprocal square roots): PVRS, else the two-rarefaction or two-shock estimate.
__device__ __forceinline__ float ex_p_guess32(float dl, float ul, float pl, float cl, float dr, float ur, float pr,
                                              float cr, const ExGas64 &X) {
    const float ppv = (.5f * (pl + pr)) - (((.125f * (ur - ul)) * (dl + dr)) * (cl + cr));
    const float p_max = fmaxf(pl, pr), p_min = fminf(pl, pr);
    if ((p_max <= 2.f * p_min) && (p_min <= ppv && ppv <= p_max)) return ppv;
    if (ppv <= p_min) {
        const float inv_cl = 1.f / cl, inv_cr = 1.f / cr;
        const float p_lr = __powf(pl / pr, X.zf);
        const float u_star = (((p_lr * ul) * inv_cl + ur * inv_cr) + X.two_gm1f * (p_lr - 1.f)) /
                             (p_lr * inv_cl + inv_cr);
        const float p_tl = __powf(1.f + (X.gm1_2f * (ul - u_star)) * inv_cl, X.inv_zf);
        const float p_tr = __powf(1.f + (X.gm1_2f * (u_star - ur)) * inv_cr, X.inv_zf);
        return .5f * ((pl * p_tl) + (pr * p_tr));
    }
    const float gl = X.sq_two_gp1f * rsqrtf(dl * (X.gm1_gp1f * pl + ppv));
    const float gr = X.sq_two_gp1f * rsqrtf(dr * (X.gm1_gp1f * pr + ppv));
    return (((gl * pl) + (gr * pr)) - (ur - ul)) / (gr + gl);
}
#endif

struct ExSide {
    double d, p, c, Bk;
    double inv_cd;            // 1/(c d); 0 until first needed
    double inv_ref, qz_ref;   // 1/p and (p/p_K)^z of the last rarefaction evaluation (inv_ref 0: none)
    double ps_ref, s_ref, u_ref;  // p, s(p) and 1/(p + B_K) of the last shock evaluation (s_ref 0: none)
};

PHD_HD __forceinline__ double ex_side_power(ExSide &S, const ExGas64 &X, double p_old) {
    const double r = fma(p_old, S.inv_ref, -1.);
    if (fabs(r) <= EX_NEAR_ONE) return S.qz_ref * ex_pow_near_one(X, r);
    return ex_pow_z(X, p_old * ex_rcp(S.p));
}

// f_K(p_old) and f_K'(p_old) of ex_p_func / ex_p_func_deriv; inv_pold = 1 / p_old
PHD_HD __forceinline__ void ex_side_eval(ExSide &S, const ExGas64 &X, double p_old, double inv_pold, double &f,
                                         double &df) {
    if (p_old <= S.p) {
        const double qz = ex_side_power(S, X, p_old);
        S.inv_ref = inv_pold;
        S.qz_ref = qz;
        if (S.inv_cd == 0.) S.inv_cd = ex_rcp(S.c * S.d);
        f = (S.c * X.two_gm1) * (qz - 1.);
        df = (qz * (S.p * inv_pold)) * S.inv_cd;
    } else {
        const double s = X.sq_two_gp1 * ex_rsqrt(S.d * (p_old + S.Bk));
        const double u = ((s * s) * S.d) * X.gp1_2;         // 1/(p_old + B_K)
        S.ps_ref = p_old;
        S.s_ref = s;
        S.u_ref = u;
        f = (p_old - S.p) * s;
        df = s * (1. - (.5 * (p_old - S.p)) * u);
    }
}

// f_K(p) alone (the final evaluation at p*)
PHD_HD __forceinline__ double ex_side_f(ExSide &S, const ExGas64 &X, double p) {
    if (p <= S.p) return (S.c * X.two_gm1) * (ex_side_power(S, X, p) - 1.);
    const double e = (p - S.ps_ref) * S.u_ref;
    if (S.s_ref != 0. && fabs(e) <= 0.000244140625) return (p - S.p) * (S.s_ref * ex_rsqrt_near_one(e));
    return (p - S.p) * (X.sq_two_gp1 * ex_rsqrt(S.d * (p + S.Bk)));
}

// p* of ex_get_pstar, and the two side functions at p* (for u*).
PHD_HD __forceinline__ double ex_get_pstar_lean(double dl, double ul, double pl, double cl, double dr,
                                                double ur, double pr, double cr, const ExGas64 &X, int max_iter,
                                                bool *failed, double &fl_star, double &fr_star,
                                                float guess32 = -1.f) {
    // guess32 > 0: the FP32 path's guess, and the side functions at p* linearised
    const double TOL = 1.0e-6;
    ExSide Ls{dl, pl, cl, pl * X.gm1_gp1, 0., 0., 0., 0., 0., 0.};
    ExSide Rs{dr, pr, cr, pr * X.gm1_gp1, 0., 0., 0., 0., 0., 0.};
    const bool f32 = guess32 > 0.f && guess32 < INFINITY;
    double p_old = f32 ? double(guess32) : ex_p_guess_lean(dl, ul, pl, cl, dr, ur, pr, cr, X);
    double p_new = p_old;
    for (int it = 0; it < max_iter; it++) {
        double fl, fr, dfl, dfr;
        const double inv_pold = (p_old <= pl || p_old <= pr) ? ex_rcp(p_old) : 0.;
        ex_side_eval(Ls, X, p_old, inv_pold, fl, dfl);
        ex_side_eval(Rs, X, p_old, inv_pold, fr, dfr);
        p_new = p_old - ((((fl + fr) + ur) - ul) * ex_rcp(dfl + dfr));
        const double sum = p_new + p_old;
        if (2. * fabs(p_new - p_old) <= TOL * fabs(sum) && sum != 0.) {
            if (f32) {
                const double dp = p_new - p_old;
                fl_star = fma(dfl, dp, fl);
                fr_star = fma(dfr, dp, fr);
            } else {
                fl_star = ex_side_f(Ls, X, p_new);
                fr_star = ex_side_f(Rs, X, p_new);
            }
            return p_new;
        }
        if (p_new < 0.) p_new = TOL;
        p_old = p_new;
    }
    *failed = true;
    fl_star = ex_side_f(Ls, X, p_new);
    fr_star = ex_side_f(Rs, X, p_new);
    return p_new;
}

// Exact.riemann_solver riemann.pyx:700-972: exact solution sampled at xi = 0 in the
// face frame, then deboosted (the Exact solver always boosts, riemann.pyx:695-698).
// X: the FP32 path's gamma constants (unused by the FP64 path).
template <typename T, int DIM>
PHD_HD __forceinline__ void exact_flux(const T *L, const T *R, const T *n, const T *w, T gamma,
                                           int max_iter, T *f, bool *failed, const ExGas64 *X = nullptr) {
    const int E = DIM + 1;
    const T _dl = L[0], _pl = L[E], _dr = R[0], _pr = R[E];
    const T cl = t_sqrt((gamma * _pl) / _dl);
    const T cr = t_sqrt((gamma * _pr) / _dr);
    T vnl = T(0.0), vnr = T(0.0), vl_sq = T(0.0), vr_sq = T(0.0);
#pragma unroll
    for (int k = 0; k < DIM; k++) {
        vnl = vnl + L[1 + k] * n[k];
        vnr = vnr + R[1 + k] * n[k];
        vl_sq = vl_sq + L[1 + k] * L[1 + k];
        vr_sq = vr_sq + R[1 + k] * R[1 + k];
    }
    const double g = double(gamma);
    T p_star, u_star;
    if constexpr (sizeof(T) == sizeof(double)) {   // FP64 path: the reference's iteration verbatim
        const double p_star_d = ex_get_pstar(double(_dl), double(vnl), double(_pl), double(cl), double(_dr),
                                             double(vnr), double(_pr), double(cr), g, max_iter, failed);
        const double fl_d = ex_p_func(double(_dl), double(_pl), double(cl), g, p_star_d);
        const double fr_d = ex_p_func(double(_dr), double(_pr), double(cr), g, p_star_d);
        p_star = T(p_star_d);
        u_star = T(0.5 * (((double(vnl) + double(vnr)) + fr_d) - fl_d));
    } else {                                  // FP32 path: FP64 Newton, powers reused across steps
        double fl_d, fr_d;
#ifdef __CUDA_ARCH__
        const float g32 = ex_p_guess32(float(_dl), float(vnl), float(_pl), float(cl), float(_dr), float(vnr),
                                       float(_pr), float(cr), *X);
#else
        const float g32 = -1.f;
#endif
        const double p_star_d = ex_get_pstar_lean(double(_dl), double(vnl), double(_pl), double(cl),
                                                  double(_dr), double(vnr), double(_pr), double(cr), *X, max_iter,
                                                  failed, fl_d, fr_d, g32);
        p_star = T(p_star_d);
        u_star = T(0.5 * (((double(vnl) + double(vnr)) + fr_d) - fl_d));
    }
    int kind;            // 0: left data, 1: right data, 2: sampled (d, p, velocity shift)
    T _d = T(0), _p = T(0), ushift = T(0);
    bool right_side = false;
    if (T(0.0) <= u_star) {
        if (p_star <= _pl) {
            const T s_hl = vnl - cl;
            if (T(0.0) <= s_hl) kind = 0;
            else {
                const T c_star_l = cl * t_pow(p_star / _pl, (gamma - T(1.0)) / (T(2.0) * gamma));
                const T s_tl = u_star - c_star_l;
                if (T(0.0) >= s_tl) {
                    kind = 2; _d = _dl * t_pow(p_star / _pl, T(1.0) / gamma); _p = p_star; ushift = u_star - vnl;
                } else {
                    const T c = (T(2.0) / (gamma + T(1.0))) * (cl + ((T(0.5) * (gamma - T(1.0))) * vnl));
                    kind = 2; _d = _dl * t_pow(c / cl, T(2.0) / (gamma - T(1.0)));
                    _p = _pl * t_pow(c / cl, (T(2.0) * gamma) / (gamma - T(1.0))); ushift = c - vnl;
                }
            }
        } else {
            const T sl = vnl - (cl * t_sqrt(((((gamma + T(1.0)) * p_star) / ((T(2.0) * gamma) * _pl)) +
                                             ((gamma - T(1.0)) / (T(2.0) * gamma)))));
            if (T(0.0) <= sl) kind = 0;
            else {
                kind = 2;
                _d = (_dl * ((p_star / _pl) + ((gamma - T(1.0)) / (gamma + T(1.0))))) /
                     (((p_star * (gamma - T(1.0))) / ((gamma + T(1.0)) * _pl)) + T(1.0));
                _p = p_star; ushift = u_star - vnl;
            }
        }
    } else {
        right_side = true;
        if (p_star >= _pr) {
            const T sr = vnr + (cr * t_sqrt(((((gamma + T(1.0)) * p_star) / ((T(2.0) * gamma) * _pr)) +
                                             ((gamma - T(1.0)) / (T(2.0) * gamma)))));
            if (T(0.0) >= sr) kind = 1;
            else {
                kind = 2;
                _d = (_dr * ((p_star / _pr) + ((gamma - T(1.0)) / (gamma + T(1.0))))) /
                     (((p_star * (gamma - T(1.0))) / ((gamma + T(1.0)) * _pr)) + T(1.0));
                _p = p_star; ushift = u_star - vnr;
            }
        } else {
            const T s_hr = vnr + cr;
            if (T(0.0) >= s_hr) kind = 1;
            else {
                const T c_star_r = cr * t_pow(p_star / _pr, (gamma - T(1.0)) / (T(2.0) * gamma));
                const T s_tr = u_star + c_star_r;
                if (T(0.0) <= s_tr) {
                    kind = 2; _d = _dr * t_pow(p_star / _pr, T(1.0) / gamma); _p = p_star; ushift = u_star - vnr;
                } else {
                    const T c = (T(2.0) / (gamma + T(1.0))) * (cr - ((T(0.5) * (gamma - T(1.0))) * vnr));
                    const T u_tmp = (T(2.0) / (gamma + T(1.0))) * ((-cr) + ((T(0.5) * (gamma - T(1.0))) * vnr));
                    kind = 2; _d = _dr * t_pow(c / cr, T(2.0) / (gamma - T(1.0)));
                    _p = _pr * t_pow(c / cr, (T(2.0) * gamma) / (gamma - T(1.0))); ushift = u_tmp - vnr;
                }
            }
        }
    }
    if (kind == 0) {
        f[0] = _dl * vnl;
        f[E] = (((T(0.5) * _dl) * vl_sq) + ((gamma * _pl) / (gamma - T(1.0)))) * vnl;
#pragma unroll
        for (int k = 0; k < DIM; k++) f[1 + k] = ((_dl * L[1 + k]) * vnl) + (_pl * n[k]);
    } else if (kind == 1) {
        f[0] = _dr * vnr;
        f[E] = (((T(0.5) * _dr) * vr_sq) + ((gamma * _pr) / (gamma - T(1.0)))) * vnr;
#pragma unroll
        for (int k = 0; k < DIM; k++) f[1 + k] = ((_dr * R[1 + k]) * vnr) + (_pr * n[k]);
    } else {
        const T *st = right_side ? R : L;
        T v[DIM];
        T vn = T(0.), v_sq = T(0.);
#pragma unroll
        for (int k = 0; k < DIM; k++) {
            v[k] = st[1 + k] + (ushift * n[k]);
            vn = vn + v[k] * n[k];
            v_sq = v_sq + v[k] * v[k];
        }
        f[0] = _d * vn;
        f[E] = (((T(0.5) * _d) * v_sq) + ((gamma * _p) / (gamma - T(1.0)))) * vn;
#pragma unroll
        for (int k = 0; k < DIM; k++) f[1 + k] = ((_d * v[k]) * vn) + (_p * n[k]);
    }
    deboost<T, DIM>(w, f);
}

template <typename T, int DIM>
PHD_HD __forceinline__ void riemann_flux(int solver, const T *L, const T *R, const T *n, const T *w,
                                             T gamma, bool boost, int max_iter, T *f, bool *failed) {
    if (solver == PHD_EXACT) exact_flux<T, DIM>(L, R, n, w, gamma, max_iter, f, failed);
    else hll_family<T, DIM>(solver == PHD_HLLC, L, R, n, w, gamma, boost, f);
}

// GIZMO pair limiter (Hopkins 2015 appendix B4) as in add_spatial
// reconstruction.pyx:877-921.  X = extrapolated state (in/out), S = constant state of
// the same side, ci/cj = unboosted cell values that decide the limiting direction.
template <typename T>
PHD_HD __forceinline__ void gizmo_pair(T sl, T sr, T ci, T cj, T sepi_mag, T sepj_mag, T diff_mag,
                                           T &xl, T &xr) {
    const T psi1 = T(0.5), psi2 = T(0.25);
    const T delta1 = psi1 * t_fabs(sl - sr);
    const T delta2 = psi2 * t_fabs(sl - sr);
    const T phi_min = t_fmin(sl, sr);
    const T phi_max = t_fmax(sl, sr);
    const T phibar_l = sl + ((sepi_mag / diff_mag) * (sr - sl));
    const T phibar_r = sr + ((sepj_mag / diff_mag) * (sl - sr));
    T phi_plus, phi_minus;
    if (((phi_max + delta1) * phi_max) >= T(0.)) phi_plus = phi_max + delta1;
    else phi_plus = phi_max / (T(1) + (delta1 / t_fabs(phi_max)));
    if (((phi_min - delta1) * phi_min) >= T(0.)) phi_minus = phi_min - delta1;
    else phi_minus = phi_min / (T(1) + (delta1 / t_fabs(phi_min)));
    if (ci < cj) {
        xl = t_fmax(phi_minus, t_fmin(phibar_l + delta2, xl));
        xr = t_fmin(phi_plus, t_fmax(phibar_r - delta2, xr));
    } else if (ci > cj) {
        xl = t_fmin(phi_plus, t_fmax(phibar_l - delta2, xl));
        xr = t_fmax(phi_minus, t_fmin(phibar_r + delta2, xr));
    } else {
        xl = sl;
        xr = sr;
    }
}

// add_temporal reconstruction.pyx:923-1072 for one face; dt is the half step.
// L/R enter as spatially extrapolated states and leave time-extrapolated (or reverted
// to the spatial state where density or pressure would turn negative).
template <typename T, int DIM>
PHD_HD __forceinline__ void temporal(T *L, T *R, const T *pi, const T *pj, const T *gi, const T *gj,
                                         const T *w, T gamma, T dt, bool boost) {
    const int NF = DIM + 2, E = DIM + 1;
    T sl[NF], sr[NF], vi[DIM], vj[DIM];
#pragma unroll
    for (int f = 0; f < NF; f++) { sl[f] = L[f]; sr[f] = R[f]; }
    // grad rows: density k, velocity c*DIM+k at DIM + c*DIM + k, pressure at (DIM+1)*DIM + k
#pragma unroll
    for (int k = 0; k < DIM; k++) {
        if (boost) { vi[k] = pi[1 + k] - w[k]; vj[k] = pj[1 + k] - w[k]; }
        else { vi[k] = pi[1 + k]; vj[k] = pj[1 + k]; }
        L[1 + k] = L[1 + k] - ((dt * gi[E * DIM + k]) / pi[0]);
        R[1 + k] = R[1 + k] - ((dt * gj[E * DIM + k]) / pj[0]);
    }
#pragma unroll
    for (int k = 0; k < DIM; k++) {
        const T divi = gi[DIM + (DIM + 1) * k], divj = gj[DIM + (DIM + 1) * k];
        L[0] = L[0] - (dt * ((pi[0] * divi) + (vi[k] * gi[k])));
        R[0] = R[0] - (dt * ((pj[0] * divj) + (vj[k] * gj[k])));
        L[E] = L[E] - (dt * (((gamma * pi[E]) * divi) + (vi[k] * gi[E * DIM + k])));
        R[E] = R[E] - (dt * (((gamma * pj[E]) * divj) + (vj[k] * gj[E * DIM + k])));
#pragma unroll
        for (int c = 0; c < DIM; c++) {
            L[1 + c] = L[1 + c] - ((dt * vi[k]) * gi[DIM + c * DIM + k]);
            R[1 + c] = R[1 + c] - ((dt * vj[k]) * gj[DIM + c * DIM + k]);
        }
    }
    if (L[0] < T(0.0) || L[E] < T(0.0)) {
#pragma unroll
        for (int f = 0; f < NF; f++) L[f] = sl[f];
    }
    if (R[0] < T(0.0) || R[E] < T(0.0)) {
#pragma unroll
        for (int f = 0; f < NF; f++) R[f] = sr[f];
    }
}

}  // namespace phd
