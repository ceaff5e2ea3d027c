// phd_frozen.cu -- the FP64 step with its branch decisions recorded and replayed.
//
// The limited scheme is piecewise smooth: limiter minima over faces and neighbours,
// GIZMO clamps, positivity reverts, the wave-speed estimate and the Riemann region are
// all discrete choices.  A central difference of a multi-step loss crosses such
// switches and then measures no derivative.  phd_step_f64_frozen computes the step of
// phd_step_f64 (static mesh) in two modes:
//   RECORD: the ordinary step -- same formulas, same operation order, no FMA
//           contraction -- that also writes every decision of its face stage (64 bits
//           per face) and, through phd_gradients_f64_taped, the limiter's selections;
//   REPLAY: the same arithmetic with every decision read back instead of taken from
//           the current values.
// Near the recorded state REPLAY is a smooth map whose derivative is what the
// hand-written adjoint (phd_adjoint_step_f64_taped) computes on the branch the run
// took, so central differences through it check the adjoint where the map itself has
// kinks.  Verification only: the product step is phd_step_f64 / phd_step_f32.
//
// Compiled with --fmad=false, like phd_f64.cu.
#include "phd_common.cuh"
#include "phd_physics.cuh"

namespace phd {
namespace {

constexpr int FBLOCK = 128;

// One decision: RECORD takes it from the condition and sets its bit; REPLAY returns the
// recorded bit.  Every face consumes the same sequence of bits whatever the outcome.
template <bool REPLAY>
struct Decide {
    unsigned long long bits;
    int k;
    __device__ __forceinline__ bool operator()(bool c) {
        bool r;
        if (REPLAY) {
            r = (bits >> k) & 1ull;
        } else {
            r = c;
            if (c) bits |= 1ull << k;
        }
        k++;
        return r;
    }
};

// fmin / fmax / fabs as decisions (ties pick either operand: the same value)
template <class D>
__device__ __forceinline__ double dmin(D &dec, double a, double b) { return dec(a <= b) ? a : b; }
template <class D>
__device__ __forceinline__ double dmax(D &dec, double a, double b) { return dec(a >= b) ? a : b; }

// gizmo_pair (phd_physics.cuh; reconstruction.pyx:877-912) with 11 decisions per field.
template <class D>
__device__ __forceinline__ void gizmo_frozen(D &dec, double sl, double sr, double ci, double cj, double sepi_mag,
                                             double sepj_mag, double diff_mag, double &xl, double &xr) {
    const double psi1 = 0.5, psi2 = 0.25;
    const bool lo = dec(sl < sr);                        // |sl - sr|, min and max together
    const double ad = lo ? (sr - sl) : (sl - sr);
    const double delta1 = psi1 * ad, delta2 = psi2 * ad;
    const double phi_min = lo ? sl : sr, phi_max = lo ? sr : sl;
    const double phibar_l = sl + ((sepi_mag / diff_mag) * (sr - sl));
    const double phibar_r = sr + ((sepj_mag / diff_mag) * (sl - sr));
    const bool plus_reg = dec(((phi_max + delta1) * phi_max) >= 0.);
    const double amax = dec(phi_max >= 0.) ? phi_max : -phi_max;
    const bool minus_reg = dec(((phi_min - delta1) * phi_min) >= 0.);
    const double amin = dec(phi_min >= 0.) ? phi_min : -phi_min;
    const double phi_plus = plus_reg ? phi_max + delta1 : phi_max / (1. + (delta1 / amax));
    const double phi_minus = minus_reg ? phi_min - delta1 : phi_min / (1. + (delta1 / amin));
    const bool lt = dec(ci < cj), gt = dec(ci > cj);
    if (lt) {
        xl = dmax(dec, phi_minus, dmin(dec, phibar_l + delta2, xl));
        xr = dmin(dec, phi_plus, dmax(dec, phibar_r - delta2, xr));
    } else if (gt) {
        xl = dmin(dec, phi_plus, dmax(dec, phibar_l - delta2, xl));
        xr = dmax(dec, phi_minus, dmin(dec, phibar_r + delta2, xr));
    } else {
        dec.k += 4;                                      // the clamps' bits stay unused
        xl = sl;
        xr = sr;
    }
}

// get_waves (phd_physics.cuh; riemann.pyx:375-504) with 7 decisions.
template <class D>
__device__ __forceinline__ void waves_frozen(D &dec, double dl, double ul, double pl, double dr, double ur, double pr,
                                             double gamma, double &sl, double &sc, double &sr) {
    const double Q = 2., c_floor = 1.0E-10;
    const double clr = sqrt((gamma * pl) / dl), crr = sqrt((gamma * pr) / dr);
    const double cl = dec(clr >= c_floor) ? clr : c_floor;
    const double cr = dec(crr >= c_floor) ? crr : c_floor;
    const double d_avg = .5 * (dl + dr);
    const double c_avg = .5 * (cl + cr);
    const double pv = (.5 * (pl + pr)) + (((.5 * (ul - ur)) * d_avg) * c_avg);
    double p_star = dec(pv >= 0.) ? pv : 0.;
    const double p_min = fmin(pl, pr), p_max = fmax(pl, pr);
    const bool pvrs = dec(((p_max / p_min) < Q) && ((p_min < p_star) && (p_star < p_max)));
    const bool trrs = dec(p_star <= p_min);
    if (pvrs) {
    } else if (trrs) {
        const double z = (gamma - 1.) / (2. * gamma);
        const double plr = pow(pl / pr, z);
        const double u_star = ((((plr * ul) / cl) + (ur / cr)) + ((2. * (plr - 1.)) / (gamma - 1.))) /
                              ((plr / cl) + (1. / cr));
        p_star = (.5 * pl) * pow((1. + (((gamma - 1.) * (ul - u_star)) / (2. * cl))), (1. / z));
        p_star = p_star + ((.5 * pr) * pow((1. + (((gamma - 1.) * (u_star - ur)) / (2. * cr))), (1. / z)));
    } else {
        const double Al = 2. / ((gamma + 1.) * dl), Ar = 2. / ((gamma + 1.) * dr);
        const double Bl = pl * ((gamma - 1.) / (gamma + 1.)), Br = pr * ((gamma - 1.) / (gamma + 1.));
        const double gl = sqrt(Al / (p_star + Bl)), gr = sqrt(Ar / (p_star + Br));
        p_star = (((gl * pl) + (gr * pr)) - (ur - ul)) / (gl + gr);
    }
    const double k = (gamma + 1.) / (2. * gamma);
    sl = dec(p_star <= pl) ? ul - cl : ul - (cl * sqrt((1. + (k * ((p_star / pl) - 1.)))));
    sr = dec(p_star <= pr) ? ur + cr : ur + (cr * sqrt((1. + (k * ((p_star / pr) - 1.)))));
    sc = (((pr - pl) + ((dl * ul) * (sl - ul))) - ((dr * ur) * (sr - ur))) / ((dl * (sl - ul)) - (dr * (sr - ur)));
}

// hll_family (phd_physics.cuh; riemann.pyx:243-373, 521-682) with 3 region decisions.
template <class D>
__device__ __forceinline__ void hll_frozen(D &dec, bool hllc, const double *L, const double *R, const double *n,
                                           const double *w, double gamma, bool boost, double *f) {
    const double _dl = L[0], _pl = L[3], _dr = R[0], _pr = R[3];
    double Vnl = 0., Vnr = 0., vl_sq = 0., vr_sq = 0., wn = 0.;
    for (int k = 0; k < 2; k++) {
        vl_sq = vl_sq + L[1 + k] * L[1 + k];
        vr_sq = vr_sq + R[1 + k] * R[1 + k];
        Vnl = Vnl + L[1 + k] * n[k];
        Vnr = Vnr + R[1 + k] * n[k];
        wn = wn + w[k] * n[k];
    }
    if (boost) wn = 0.;
    double sl, sc, sr;
    waves_frozen(dec, _dl, Vnl, _pl, _dr, Vnr, _pr, gamma, sl, sc, sr);
    const bool left_data = dec(wn <= sl);
    const bool star = dec((sl < wn) && (wn <= sr));
    const bool left_star = dec(wn <= sc);
    if (left_data) {
        f[0] = _dl * (Vnl - wn);
        f[3] = ((((0.5 * _dl) * vl_sq) + (_pl / (gamma - 1.0))) * (Vnl - wn)) + (_pl * Vnl);
        for (int k = 0; k < 2; k++) f[1 + k] = ((_dl * L[1 + k]) * (Vnl - wn)) + (_pl * n[k]);
    } else if (star) {
        if (!hllc) {
            const double fac1 = sr - wn, fac2 = sl - wn, fac3 = sr - sl;
            f[0] = (((((_dl * Vnl) * fac1) - ((_dr * Vnr) * fac2)) - ((sl * _dl) * fac1)) + ((sr * _dr) * fac2)) / fac3;
            for (int k = 0; k < 2; k++) {
                const double vl = L[1 + k], vr = R[1 + k];
                f[1 + k] = ((((((((_dl * vl) * Vnl) + (_pl * n[k])) * fac1) -
                               ((((_dr * vr) * Vnr) + (_pr * n[k])) * fac2)) -
                              ((sl * (_dl * vl)) * fac1)) + ((sr * (_dr * vr)) * fac2))) / fac3;
            }
            const double el = ((0.5 * _dl) * vl_sq) + (_pl / (gamma - 1.0));
            const double er = ((0.5 * _dr) * vr_sq) + (_pr / (gamma - 1.0));
            f[3] = ((((((el + _pl) * Vnl) * fac1) - (((er + _pr) * Vnr) * fac2)) - ((sl * el) * fac1)) +
                    ((sr * er) * fac2)) / fac3;
        } else {
            const double d = left_star ? _dl : _dr, p = left_star ? _pl : _pr, Vn = left_star ? Vnl : Vnr;
            const double s = left_star ? sl : sr, vsq = left_star ? vl_sq : vr_sq;
            const double *S = left_star ? L : R;
            const double factor_1 = (d * (s - Vn)) / (s - sc);
            const double factor_2 = ((factor_1 * (s - wn)) * (sc - Vn)) + p;
            const double frho = (d * (Vn - s)) + (factor_1 * (s - wn));
            const double e = ((0.5 * d) * vsq) + (p / (gamma - 1.0));
            f[0] = frho;
            f[3] = (((e + p) * Vn) - (s * e)) + (((s - wn) * factor_1) * ((e / d) + ((sc - Vn) * (sc + (p / (d * (s - Vn)))))));
            for (int k = 0; k < 2; k++) f[1 + k] = (frho * S[1 + k]) + (factor_2 * n[k]);
        }
    } else {
        f[0] = _dr * (Vnr - wn);
        f[3] = ((((0.5 * _dr) * vr_sq) + (_pr / (gamma - 1.0))) * (Vnr - wn)) + (_pr * Vnr);
        for (int k = 0; k < 2; k++) f[1 + k] = ((_dr * R[1 + k]) * (Vnr - wn)) + (_pr * n[k]);
    }
    if (boost) deboost<double, 2>(w, f);
}

// Per face: add_spatial with GIZMO (reconstruction.pyx:832-921; 44 + 2 decisions),
// add_temporal (:923-1072; 2 decisions), HLL / HLLC and deboost (10 decisions): at
// most 58 bits.
template <bool REPLAY>
__global__ void __launch_bounds__(FBLOCK) k_face_frozen(phd_mesh M, phd_params P, double dt_half,
                                                        const double *__restrict__ prim,
                                                        const double *__restrict__ grad,
                                                        const double *__restrict__ face_w,
                                                        double *__restrict__ flux,
                                                        unsigned long long *__restrict__ face_bits, phd_clock *clk) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= M.n_faces) return;
    const int n = M.n_cells, F = M.n_faces;
    const int i = M.pair_i[m], j = M.pair_j[m];
    if (i < 0 || i >= n || j < 0 || j >= n) {
        if (clk) atomicOr(&clk->status, PHD_STATUS_BAD_INDEX);
        return;
    }
    Decide<REPLAY> dec{REPLAY ? face_bits[m] : 0ull, 0};
    const bool boost = P.boost != 0, linear = P.reconstruction == PHD_LINEAR, gizmo = P.gizmo != 0;
    double pi[4], pj[4], gi[8], gj[8], w[2], L[4], R[4], nrm[2], f[4];
    for (int q = 0; q < 4; q++) { pi[q] = prim[(size_t)q * n + i]; pj[q] = prim[(size_t)q * n + j]; }
    if (linear)
        for (int r = 0; r < 8; r++) { gi[r] = grad[(size_t)r * n + i]; gj[r] = grad[(size_t)r * n + j]; }
    for (int k = 0; k < 2; k++) {
        w[k] = face_w ? face_w[(size_t)k * F + m] : 0.0;
        nrm[k] = M.normal[(size_t)k * F + m];
    }
    for (int q = 0; q < 4; q++) { L[q] = pi[q]; R[q] = pj[q]; }
    if (boost)
        for (int k = 0; k < 2; k++) { L[1 + k] = pi[1 + k] - w[k]; R[1 + k] = pj[1 + k] - w[k]; }
    if (linear) {
        // add_spatial (face_spatial_f64 of phd_ref.cuh)
        double sl[4], sr[4];
        for (int q = 0; q < 4; q++) { sl[q] = L[q]; sr[q] = R[q]; }
        double diff_mag = 0.0, sepi_mag = 0.0, sepj_mag = 0.0;
        for (int k = 0; k < 2; k++) {
            const double fc = M.com[(size_t)k * F + m];
            const double xik = M.x[(size_t)k * n + i], xjk = M.x[(size_t)k * n + j];
            const double sepi = fc - (xik + M.dcom[(size_t)k * n + i]);
            const double sepj = fc - (xjk + M.dcom[(size_t)k * n + j]);
            sepi_mag = sepi_mag + sepi * sepi;
            sepj_mag = sepj_mag + sepj * sepj;
            diff_mag = diff_mag + t_sq(xjk - xik);
            for (int q = 0; q < 4; q++) {
                L[q] = L[q] + gi[q * 2 + k] * sepi;
                R[q] = R[q] + gj[q * 2 + k] * sepj;
            }
        }
        sepi_mag = sqrt(sepi_mag);
        sepj_mag = sqrt(sepj_mag);
        diff_mag = sqrt(diff_mag);
        if (gizmo) {
            for (int q = 0; q < 4; q++) gizmo_frozen(dec, sl[q], sr[q], pi[q], pj[q], sepi_mag, sepj_mag, diff_mag, L[q], R[q]);
            if (dec(L[0] < 0.0 || L[3] < 0.0))
                for (int q = 0; q < 4; q++) L[q] = sl[q];
            if (dec(R[0] < 0.0 || R[3] < 0.0))
                for (int q = 0; q < 4; q++) R[q] = sr[q];
        }
        // add_temporal (temporal of phd_physics.cuh) with its reverts as decisions
        double tl[4], tr[4], vi[2], vj[2];
        for (int q = 0; q < 4; q++) { tl[q] = L[q]; tr[q] = R[q]; }
        for (int k = 0; k < 2; k++) {
            if (boost) { vi[k] = pi[1 + k] - w[k]; vj[k] = pj[1 + k] - w[k]; }
            else { vi[k] = pi[1 + k]; vj[k] = pj[1 + k]; }
            L[1 + k] = L[1 + k] - ((dt_half * gi[3 * 2 + k]) / pi[0]);
            R[1 + k] = R[1 + k] - ((dt_half * gj[3 * 2 + k]) / pj[0]);
        }
        for (int k = 0; k < 2; k++) {
            const double divi = gi[2 + 3 * k], divj = gj[2 + 3 * k];
            L[0] = L[0] - (dt_half * ((pi[0] * divi) + (vi[k] * gi[k])));
            R[0] = R[0] - (dt_half * ((pj[0] * divj) + (vj[k] * gj[k])));
            L[3] = L[3] - (dt_half * (((P.gamma * pi[3]) * divi) + (vi[k] * gi[3 * 2 + k])));
            R[3] = R[3] - (dt_half * (((P.gamma * pj[3]) * divj) + (vj[k] * gj[3 * 2 + k])));
            for (int c = 0; c < 2; c++) {
                L[1 + c] = L[1 + c] - ((dt_half * vi[k]) * gi[2 + c * 2 + k]);
                R[1 + c] = R[1 + c] - ((dt_half * vj[k]) * gj[2 + c * 2 + k]);
            }
        }
        if (dec(L[0] < 0.0 || L[3] < 0.0))
            for (int q = 0; q < 4; q++) L[q] = tl[q];
        if (dec(R[0] < 0.0 || R[3] < 0.0))
            for (int q = 0; q < 4; q++) R[q] = tr[q];
    }
    hll_frozen(dec, P.solver == PHD_HLLC, L, R, nrm, w, P.gamma, boost, f);
    for (int q = 0; q < 4; q++) flux[(size_t)q * F + m] = f[q];
    if (!REPLAY) face_bits[m] = dec.bits;
}

// Gradient with the limiter's selections replayed from the record phd_gradients_f64_taped
// wrote (rows: per field the active entry -- -1 none, -2 a clamp at zero --, the
// entries of the neighbour maximum and minimum, -1 the cell itself): the unlimited
// estimate of cell_gradient_f64 (reconstruction.pyx:620-681) at the current values,
// alpha = 1, 0, or (phi_ext - phi_i) / dphi at the recorded face with the recorded
// extreme neighbour (:683-703).  Ghost rows: the image's gradient with the reflective
// flip (domain_manager.pyx:819-835).
__global__ void __launch_bounds__(FBLOCK) k_grad_frozen(phd_mesh M, const double *__restrict__ prim,
                                                        const int32_t *__restrict__ tape_i32,
                                                        double *__restrict__ grad, phd_clock *clk) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= M.n_cells) return;
    const int n = M.n_cells, F = M.n_faces;
    int c = i;
    if (M.tag[i] != PHD_REAL_TAG) {
        c = M.map[i];
        if (c < 0 || c >= n) {
            if (clk) atomicOr(&clk->status, PHD_STATUS_BAD_INDEX);
            return;
        }
    }
    double xi[2], cx[2], pc[4], df[8];
    for (int k = 0; k < 2; k++) {
        xi[k] = M.x[(size_t)k * n + c];
        cx[k] = xi[k] + M.dcom[(size_t)k * n + c];
    }
    const double vol = M.vol[c];
    for (int f = 0; f < 4; f++) {
        pc[f] = prim[(size_t)f * n + c];
        df[2 * f] = df[2 * f + 1] = 0;
    }
    const int m0 = M.nbr_ptr[c], m1 = M.nbr_ptr[c + 1];
    for (int m = m0; m < m1; m++) {
        const int fid = M.nbr_idx[m];
        if (fid < 0 || fid >= F) continue;
        const int a = M.pair_i[fid], b = M.pair_j[fid];
        const int j = (c == a) ? b : a;
        if (j < 0 || j >= n) continue;
        const double area = M.area[fid];
        double cfx[2], dr[2], r = 0.0;
        for (int k = 0; k < 2; k++) {
            const double xj = M.x[(size_t)k * n + j];
            cfx[k] = M.com[(size_t)k * F + fid] - 0.5 * (xi[k] + xj);
            dr[k] = xi[k] - xj;
            r = r + t_sq(dr[k]);
        }
        r = sqrt(r);
        for (int f = 0; f < 4; f++) {
            const double pj = prim[(size_t)f * n + j];
            const double d_dif = pj - pc[f];
            const double d_sum = pj + pc[f];
            for (int k = 0; k < 2; k++)
                df[2 * f + k] = df[2 * f + k] + (area * ((d_dif * cfx[k]) - ((0.5 * d_sum) * dr[k]))) / (r * vol);
        }
    }
    for (int f = 0; f < 4; f++) {
        const int act = tape_i32[(size_t)f * n + c];
        double alpha = 1.0;
        if (act == -2) {
            alpha = 0.0;
        } else if (act >= m0 && act < m1) {
            const int fid = M.nbr_idx[act];
            double dphi = 0.0;
            for (int k = 0; k < 2; k++) dphi = dphi + df[2 * f + k] * (M.com[(size_t)k * F + fid] - cx[k]);
            const int ext = tape_i32[(size_t)((dphi > 0 ? 4 : 8) + f) * n + c];
            double phi_ext = pc[f];
            if (ext >= m0 && ext < m1) {
                const int ef = M.nbr_idx[ext];
                const int ea = M.pair_i[ef], eb = M.pair_j[ef];
                const int j = (c == ea) ? eb : ea;
                if (j >= 0 && j < n) phi_ext = prim[(size_t)f * n + j];
            }
            alpha = (phi_ext - pc[f]) / dphi;
        }
        df[2 * f] = alpha * df[2 * f];
        df[2 * f + 1] = alpha * df[2 * f + 1];
    }
    const int fl = M.flip ? M.flip[i] : 0;
    for (int k = 0; k < 2; k++)
        if (fl & (1 << k)) df[2 * (1 + k) + k] *= -1;
    for (int r = 0; r < 8; r++) grad[(size_t)r * n + i] = df[r];
}

inline int grid_n(int n, int b) { return n > 0 ? (n + b - 1) / b : 1; }

}  // namespace
}  // namespace phd

using namespace phd;

extern "C" {

int phd_step_f64_frozen(const phd_mesh *mesh, const phd_params *par, int32_t mode, double dt, double *prim,
                        const double *cons, double *cons_next, double *grad, const double *face_w, double *flux,
                        double *tape_f64, int32_t *tape_i32, uint64_t *face_bits, phd_clock *clk,
                        cudaStream_t stream) {
    phd::NvtxRange nvtx_range("phd_step_f64_frozen");
    if (!mesh || mesh->dim != 2 || mesh->n_cells <= 0 || mesh->n_faces < 0 || !par || !prim || !cons ||
        !cons_next || !flux || !clk || (mesh->n_faces && (!mesh->normal || !face_bits)))
        return PHD_ERR_ARG;
    if (mode != PHD_FROZEN_RECORD && mode != PHD_FROZEN_REPLAY) return PHD_ERR_ARG;
    if (par->solver != PHD_HLL && par->solver != PHD_HLLC) return PHD_ERR_UNSUPPORTED;
    const bool linear = par->reconstruction == PHD_LINEAR;
    if (linear && par->limiter != PHD_LIMITER_AREPO) return PHD_ERR_UNSUPPORTED;
    if (linear && (!grad || !tape_i32 || (mode == PHD_FROZEN_RECORD && !tape_f64))) return PHD_ERR_ARG;
    const int n = mesh->n_cells, F = mesh->n_faces;
    int rc = PHD_OK;
    if (linear) {
        if (mode == PHD_FROZEN_RECORD)
            rc = phd_gradients_f64_taped(mesh, prim, par->limiter, grad, tape_f64, tape_i32, clk, stream);
        else
            k_grad_frozen<<<grid_n(n, FBLOCK), FBLOCK, 0, stream>>>(*mesh, prim, tape_i32, grad, clk);
        if (rc != PHD_OK) return rc;
    }
    if (F) {
        const auto bits = reinterpret_cast<unsigned long long *>(face_bits);
        if (mode == PHD_FROZEN_RECORD)
            k_face_frozen<false><<<grid_n(F, FBLOCK), FBLOCK, 0, stream>>>(*mesh, *par, 0.5 * dt, prim, grad, face_w,
                                                                            flux, bits, clk);
        else
            k_face_frozen<true><<<grid_n(F, FBLOCK), FBLOCK, 0, stream>>>(*mesh, *par, 0.5 * dt, prim, grad, face_w,
                                                                           flux, bits, clk);
    }
    // Mesh.update_from_fluxes, ghost refresh and primitive recovery (the dt is fixed)
    if (cudaMemcpyAsync(cons_next, cons, (size_t)4 * n * sizeof(double), cudaMemcpyDeviceToDevice, stream) !=
        cudaSuccess)
        return PHD_ERR_LAUNCH;
    if ((rc = phd_update_from_fluxes_f64(mesh, flux, dt, cons_next, clk, stream)) != PHD_OK) return rc;
    if ((rc = phd_ghost_cons_f64(mesh, cons_next, stream)) != PHD_OK) return rc;
    if ((rc = phd_prim_from_cons_f64(2, n, par->gamma, mesh->vol, cons_next, prim, stream)) != PHD_OK) return rc;
    return cudaPeekAtLastError() == cudaSuccess ? PHD_OK : PHD_ERR_LAUNCH;
}

}  // extern "C"
