// phd_adj.cu -- hand-written adjoint of one FP64 step (mesh, face velocities, dt fixed).
//
// Forward step (real-cell conserved totals U -> U'):
//   ghost refresh -> primitives -> limited gradients -> face states (spatial +
//   GIZMO + MUSCL-Hancock half step) -> HLL/HLLC flux + deboost -> segmented update.
// Reverse, five deterministic kernels (no atomics; every sum is a per-thread loop):
//   k_adj_face     per face: flux adjoint dt*A*(lam'_j - lam'_i) through Riemann,
//                  temporal and spatial stages -> 24 per-face adjoint values
//   k_adj_gather   per cell: sum its faces' contributions -> lam_prim, lam_grad (own row)
//   k_adj_grad     per real cell: fold ghost rows into lam_grad, reverse the limited
//                  gradient -> per-entry neighbour adjoints and the cell's own adjoint
//   k_adj_gather2  per cell: own + partner-entry contributions -> lam_prim
//   k_adj_final    per real cell: fold ghost rows, reverse the primitive recovery,
//                  lam = lam' + J^T lam_prim

#include "phd_common.cuh"
#include "phd_physics.cuh"
#include "phd_adjoint.cuh"
#include "phd_ref.cuh"

namespace phd {

constexpr int BA = 256;
constexpr int FACE_ADJ = 24;   // api[4] apj[4] agi[8] agj[8]

// add_spatial (reference geometry) for one face, split into a forward pass that keeps
// what the reverse needs (the "tape") and the reverse itself, so the adjoint kernel
// evaluates the forward once.  The forward is face_spatial_f64's arithmetic in the
// same order (so the same branches): boosted cell states, extrapolation along the
// centroid separations, GIZMO pair limiter, revert where density or pressure < 0.
struct SpatialTape {
    double sl[4], sr[4], L0[4], R0[4], sepi[2], sepj[2], sepi_mag, sepj_mag, diff_mag;
    bool revL, revR;
};

__device__ __forceinline__ void spatial_fwd_f64(const phd_mesh &M, int m, int i, int j, const double *pi,
                                                const double *pj, const double *gi, const double *gj,
                                                const double *w, bool boost, bool gizmo, SpatialTape &t,
                                                double *Ls, double *Rs) {
    const int n = M.n_cells, F = M.n_faces;
    for (int f = 0; f < 4; f++) { t.sl[f] = pi[f]; t.sr[f] = pj[f]; }
    if (boost)
        for (int k = 0; k < 2; k++) { t.sl[1 + k] = pi[1 + k] - w[k]; t.sr[1 + k] = pj[1 + k] - w[k]; }
    for (int f = 0; f < 4; f++) { t.L0[f] = t.sl[f]; t.R0[f] = t.sr[f]; }
    double diff_mag = 0.0, sepi_mag = 0.0, sepj_mag = 0.0;
    for (int k = 0; k < 2; k++) {
        const double fc = M.com[(size_t)k * F + m];
        const double xik = M.x[(size_t)k * n + i], xjk = M.x[(size_t)k * n + j];
        t.sepi[k] = fc - (xik + M.dcom[(size_t)k * n + i]);
        t.sepj[k] = fc - (xjk + M.dcom[(size_t)k * n + j]);
        sepi_mag = sepi_mag + t.sepi[k] * t.sepi[k];
        sepj_mag = sepj_mag + t.sepj[k] * t.sepj[k];
        diff_mag = diff_mag + t_sq(xjk - xik);
        for (int f = 0; f < 4; f++) {
            t.L0[f] = t.L0[f] + gi[f * 2 + k] * t.sepi[k];
            t.R0[f] = t.R0[f] + gj[f * 2 + k] * t.sepj[k];
        }
    }
    t.sepi_mag = sqrt(sepi_mag);
    t.sepj_mag = sqrt(sepj_mag);
    t.diff_mag = sqrt(diff_mag);
    t.revL = t.revR = false;
    for (int f = 0; f < 4; f++) { Ls[f] = t.L0[f]; Rs[f] = t.R0[f]; }
    if (gizmo) {
        for (int f = 0; f < 4; f++)
            gizmo_pair<double>(t.sl[f], t.sr[f], pi[f], pj[f], t.sepi_mag, t.sepj_mag, t.diff_mag, Ls[f], Rs[f]);
        t.revL = (Ls[0] < 0.0 || Ls[3] < 0.0);
        t.revR = (Rs[0] < 0.0 || Rs[3] < 0.0);
        for (int f = 0; f < 4; f++) {
            if (t.revL) Ls[f] = t.sl[f];
            if (t.revR) Rs[f] = t.sr[f];
        }
    }
}

__device__ __forceinline__ void spatial_rev_f64(const SpatialTape &t, const double *pi, const double *pj,
                                                bool gizmo, const double *aL, const double *aR, double *api,
                                                double *apj, double *agi, double *agj) {
    double asl[4] = {0, 0, 0, 0}, asr[4] = {0, 0, 0, 0}, aL0[4] = {0, 0, 0, 0}, aR0[4] = {0, 0, 0, 0};
    if (gizmo) {
        double aL1[4], aR1[4];
        for (int f = 0; f < 4; f++) {
            aL1[f] = t.revL ? 0.0 : aL[f];
            aR1[f] = t.revR ? 0.0 : aR[f];
            if (t.revL) asl[f] += aL[f];
            if (t.revR) asr[f] += aR[f];
        }
        const double si = t.sepi_mag / t.diff_mag, sj = t.sepj_mag / t.diff_mag;
        for (int f = 0; f < 4; f++)
            gizmo_pair_adj_q<double>(t.sl[f], t.sr[f], pi[f], pj[f], si, sj, t.L0[f], t.R0[f], aL1[f], aR1[f],
                                     asl[f], asr[f], aL0[f], aR0[f]);
    } else {
        for (int f = 0; f < 4; f++) { aL0[f] = aL[f]; aR0[f] = aR[f]; }
    }
    for (int f = 0; f < 4; f++) {
        asl[f] += aL0[f];
        asr[f] += aR0[f];
        for (int k = 0; k < 2; k++) {
            agi[f * 2 + k] += aL0[f] * t.sepi[k];
            agj[f * 2 + k] += aR0[f] * t.sepj[k];
        }
        api[f] += asl[f];
        apj[f] += asr[f];
    }
}

// EXACT: the exact solver's reverse (exact_flux_adj); otherwise HLL / HLLC -- separate
// instantiations, so the HLL-family kernel carries none of the exact solver's registers.
template <bool EXACT>
__global__ void __launch_bounds__(BA) k_adj_face(phd_mesh M, phd_params P, double dt, const double *__restrict__ prim,
                                                 const double *__restrict__ grad, const double *__restrict__ face_w,
                                                 const double *__restrict__ lam_next, double *__restrict__ out) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= M.n_faces) return;
    const int n = M.n_cells, F = M.n_faces;
    const int i = M.pair_i[m], j = M.pair_j[m];
    double res[FACE_ADJ];
    for (int q = 0; q < FACE_ADJ; q++) res[q] = 0.0;
    if (i >= 0 && i < n && j >= 0 && j < n) {
        const bool boost = (P.boost != 0);
        const bool linear = P.reconstruction == PHD_LINEAR;
        double pi[4], pj[4], gi[8], gj[8], w[2], nrm[2];
        for (int f = 0; f < 4; f++) { pi[f] = prim[(size_t)f * n + i]; pj[f] = prim[(size_t)f * n + j]; }
        for (int r = 0; r < 8; r++) {
            gi[r] = linear ? grad[(size_t)r * n + i] : 0.0;
            gj[r] = linear ? grad[(size_t)r * n + j] : 0.0;
        }
        for (int k = 0; k < 2; k++) {
            w[k] = face_w ? face_w[(size_t)k * F + m] : 0.0;
            nrm[k] = M.normal[(size_t)k * F + m];
        }
        // flux adjoint from the update U_i -= dt a F, U_j += dt a F (j real)
        const double da = dt * M.area[m];
        const bool jr = M.tag[j] == PHD_REAL_TAG;
        double aF[4];
        for (int q = 0; q < 4; q++)
            aF[q] = da * ((jr ? lam_next[(size_t)q * n + j] : 0.0) - lam_next[(size_t)q * n + i]);
        // forward states (the spatial stage once, its tape kept for the reverse)
        double Ls[4], Rs[4], L[4], R[4];
        SpatialTape tape;
        if (linear) {
            spatial_fwd_f64(M, m, i, j, pi, pj, gi, gj, w, boost, P.gizmo != 0, tape, Ls, Rs);
            for (int f = 0; f < 4; f++) { L[f] = Ls[f]; R[f] = Rs[f]; }
            temporal<double, 2>(L, R, pi, pj, gi, gj, w, P.gamma, 0.5 * dt, boost);
        } else {
            for (int f = 0; f < 4; f++) { L[f] = pi[f]; R[f] = pj[f]; }
            if (boost) for (int k = 0; k < 2; k++) { L[1 + k] -= w[k]; R[1 + k] -= w[k]; }
        }
        double aL[4] = {0, 0, 0, 0}, aR[4] = {0, 0, 0, 0};
        if (EXACT) exact_flux_adj(L, R, nrm, w, P.gamma, P.exact_max_iter, aF, aL, aR);
        else hll_family_adj<double>(P.solver == PHD_HLLC, L, R, nrm, w, P.gamma, boost, aF, aL, aR);
        double *api = res, *apj = res + 4, *agi = res + 8, *agj = res + 16;
        if (linear) {
            double aLs[4] = {0, 0, 0, 0}, aRs[4] = {0, 0, 0, 0};
            temporal_adj<double>(Ls, Rs, pi, pj, gi, gj, w, P.gamma, 0.5 * dt, boost, aL, aR, aLs, aRs, api, apj,
                                 agi, agj);
            spatial_rev_f64(tape, pi, pj, P.gizmo != 0, aLs, aRs, api, apj, agi, agj);
        } else {
            for (int f = 0; f < 4; f++) { api[f] += aL[f]; apj[f] += aR[f]; }
        }
    }
    for (int q = 0; q < FACE_ADJ; q++) out[(size_t)q * F + m] = res[q];
}

// per cell: sum of its faces' contributions (own row, ghosts included)
__global__ void __launch_bounds__(BA) k_adj_gather(phd_mesh M, const double *__restrict__ face_adj,
                                                   double *__restrict__ cell_adj /* [12][n] */) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= M.n_cells) return;
    const int n = M.n_cells, F = M.n_faces;
    double s[12];
    for (int q = 0; q < 12; q++) s[q] = 0.0;
    for (int e = M.nbr_ptr[x]; e < M.nbr_ptr[x + 1]; e++) {
        const int f = M.nbr_idx[e];
        if (f < 0 || f >= F) continue;
        const bool as_i = M.pair_i[f] == x;
        const int pbase = as_i ? 0 : 4, gbase = as_i ? 8 : 16;
        for (int q = 0; q < 4; q++) s[q] += face_adj[(size_t)(pbase + q) * F + f];
        for (int q = 0; q < 8; q++) s[4 + q] += face_adj[(size_t)(gbase + q) * F + f];
    }
    for (int q = 0; q < 12; q++) cell_adj[(size_t)q * n + x] = s[q];
}

// per real cell: reverse of the limited gradient (cell_gradient_f64).
// TAPED: the forward selections (unlimited estimate, limiter values, active entries,
// neighbour extrema) come from the limiter record of a taped forward step instead of
// being recomputed.
template <bool TAPED>
__global__ void __launch_bounds__(BA) k_adj_grad(phd_mesh M, phd_adj_index A, int limiter,
                                                 const double *__restrict__ prim, const double *__restrict__ cell_adj,
                                                 double *__restrict__ entry_adj /* [4][2F] */,
                                                 double *__restrict__ self_adj /* [4][n] */,
                                                 const double *__restrict__ tape_f64,
                                                 const int32_t *__restrict__ tape_i32) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= M.n_cells || M.tag[c] != PHD_REAL_TAG) return;
    const int n = M.n_cells, F = M.n_faces;
    const int E2 = 2 * F;
    // lam_grad of this cell = own row + its ghost rows (reflective diagonal flip)
    double ag[8];
    for (int q = 0; q < 8; q++) ag[q] = cell_adj[(size_t)(4 + q) * n + c];
    for (int t = A.ghost_ptr[c]; t < A.ghost_ptr[c + 1]; t++) {
        const int g = A.ghost_idx[t];
        const int fl = M.flip ? M.flip[g] : 0;
        for (int q = 0; q < 8; q++) {
            double v = cell_adj[(size_t)(4 + q) * n + g];
            if ((q == 2 && (fl & 1)) || (q == 5 && (fl & 2))) v = -v;
            ag[q] += v;
        }
    }
    // forward recompute (cell_gradient_f64 with selections)
    double xi[2], cx[2], pc[4], df[8], phi_max[4], phi_min[4];
    int arg_max[4], arg_min[4];
    for (int k = 0; k < 2; k++) {
        xi[k] = M.x[(size_t)k * n + c];
        cx[k] = xi[k] + M.dcom[(size_t)k * n + c];
    }
    const double vol = M.vol[c];
    for (int f = 0; f < 4; f++) {
        pc[f] = prim[(size_t)f * n + c];
        phi_max[f] = phi_min[f] = pc[f];
        arg_max[f] = arg_min[f] = -1;
        df[2 * f] = df[2 * f + 1] = 0.0;
    }
    const int m0 = M.nbr_ptr[c], m1 = M.nbr_ptr[c + 1];
    double alpha[4] = {1.0, 1.0, 1.0, 1.0};
    int act[4] = {-1, -1, -1, -1};     // entry whose psi is the active limit
    int act_f0 = -1;                   // TESS: field of the active psi
    if (TAPED) {
        for (int r = 0; r < 8; r++) df[r] = tape_f64[(size_t)r * n + c];
        for (int f = 0; f < 4; f++) {
            alpha[f] = tape_f64[(size_t)(8 + f) * n + c];
            act[f] = tape_i32[(size_t)f * n + c];
            arg_max[f] = tape_i32[(size_t)(4 + f) * n + c];
            arg_min[f] = tape_i32[(size_t)(8 + f) * n + c];
        }
        act_f0 = tape_i32[(size_t)12 * n + c];
    }
    for (int e = m0; e < (TAPED ? m0 : m1); e++) {
        const int fid = M.nbr_idx[e];
        const int j = (M.pair_i[fid] == c) ? M.pair_j[fid] : M.pair_i[fid];
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
            if (pj > phi_max[f]) { phi_max[f] = pj; arg_max[f] = e; }
            if (pj < phi_min[f]) { phi_min[f] = pj; arg_min[f] = e; }
            const double d_dif = pj - pc[f], d_sum = pj + pc[f];
            for (int k = 0; k < 2; k++)
                df[2 * f + k] = df[2 * f + k] + (area * ((d_dif * cfx[k]) - ((0.5 * d_sum) * dr[k]))) / (r * vol);
        }
    }
    for (int e = m0; e < (TAPED ? m0 : m1); e++) {
        const int fid = M.nbr_idx[e];
        const int j = (M.pair_i[fid] == c) ? M.pair_j[fid] : M.pair_i[fid];
        double sep[2];
        for (int k = 0; k < 2; k++) sep[k] = M.com[(size_t)k * F + fid] - cx[k];
        for (int f = 0; f < 4; f++) {
            double dphi = 0.0, psi;
            for (int k = 0; k < 2; k++) dphi = dphi + df[2 * f + k] * sep[k];
            if (limiter == PHD_LIMITER_AREPO) {
                if (dphi > 0) psi = (phi_max[f] - pc[f]) / dphi;
                else if (dphi < 0) psi = (phi_min[f] - pc[f]) / dphi;
                else psi = 1.0;
                const double cand = fmax(psi, 0.);
                if (cand < alpha[f]) { alpha[f] = cand; act[f] = (psi > 0.0 && dphi != 0.0) ? e : -2; }
            } else {
                if (dphi > 0.0 || dphi < 0.0) {
                    const double t = (prim[(size_t)f * n + j] - pc[f]) / dphi;
                    psi = (0. > t) ? 0. : t;
                } else psi = 1.0;
                const double cand = fmax(psi, 0.);
                if (cand < alpha[0]) { alpha[0] = cand; act[0] = (psi > 0.0 && dphi != 0.0) ? e : -2; act_f0 = f; }
            }
        }
    }
    // reverse: grad = alpha * df
    double adf[8], aself[4] = {0, 0, 0, 0}, aalpha[4];
    for (int f = 0; f < 4; f++) {
        aalpha[f] = 0.0;
        for (int k = 0; k < 2; k++) {
            adf[2 * f + k] = alpha[f] * ag[2 * f + k];
            aalpha[f] += df[2 * f + k] * ag[2 * f + k];
        }
    }
    // limiter: active psi -> (extreme value, own value, df)
    double aext[4] = {0, 0, 0, 0};       // AREPO: adjoint of phi_max / phi_min of field f
    int ext_arg[4] = {-1, -1, -1, -1};
    int tess_e = -1, tess_f = -1;
    double tess_aj = 0.0;
    for (int f = 0; f < 4; f++) {
        const int e = act[f];
        if (e < 0) continue;
        if (limiter == PHD_LIMITER_TESS && f != 0) continue;
        const int ff = (limiter == PHD_LIMITER_TESS) ? act_f0 : f;
        const int fid = M.nbr_idx[e];
        double sep[2];
        for (int k = 0; k < 2; k++) sep[k] = M.com[(size_t)k * F + fid] - cx[k];
        double dphi = 0.0;
        for (int k = 0; k < 2; k++) dphi = dphi + df[2 * ff + k] * sep[k];
        const double apsi = aalpha[f];
        const double psi = alpha[f];
        const double adphi = -apsi * psi / dphi;
        for (int k = 0; k < 2; k++) adf[2 * ff + k] += adphi * sep[k];
        aself[ff] -= apsi / dphi;
        if (limiter == PHD_LIMITER_AREPO) {
            aext[ff] += apsi / dphi;
            ext_arg[ff] = dphi > 0 ? arg_max[ff] : arg_min[ff];
        } else {
            tess_e = e;
            tess_f = ff;
            tess_aj = apsi / dphi;
        }
    }
    for (int f = 0; f < 4; f++)
        if (limiter == PHD_LIMITER_AREPO && aext[f] != 0.0 && ext_arg[f] < 0) aself[f] += aext[f];
    // df = sum_e area (d_dif cfx - d_sum dr / 2) / (r vol)
    for (int e = m0; e < m1; e++) {
        const int fid = M.nbr_idx[e];
        const int j = (M.pair_i[fid] == c) ? M.pair_j[fid] : M.pair_i[fid];
        const double area = M.area[fid];
        double cfx[2], dr[2], r = 0.0;
        for (int k = 0; k < 2; k++) {
            const double xj = M.x[(size_t)k * n + j];
            cfx[k] = M.com[(size_t)k * F + fid] - 0.5 * (xi[k] + xj);
            dr[k] = xi[k] - xj;
            r = r + t_sq(dr[k]);
        }
        r = sqrt(r);
        const double coef = area / (r * vol);
        double aj[4];
        for (int f = 0; f < 4; f++) {
            double sj = 0.0, sc = 0.0;
            for (int k = 0; k < 2; k++) {
                sj += adf[2 * f + k] * (cfx[k] - 0.5 * dr[k]);
                sc += adf[2 * f + k] * (-cfx[k] - 0.5 * dr[k]);
            }
            aj[f] = sj * coef;
            aself[f] += sc * coef;
            if (limiter == PHD_LIMITER_AREPO && ext_arg[f] == e) aj[f] += aext[f];
            if (limiter == PHD_LIMITER_TESS && tess_e == e && tess_f == f) aj[f] += tess_aj;
        }
        for (int f = 0; f < 4; f++) entry_adj[(size_t)f * E2 + e] = aj[f];
    }
    for (int f = 0; f < 4; f++) self_adj[(size_t)f * n + c] = aself[f];
}

// per cell: primitive adjoint = face part + own gradient part + neighbours' gradient parts
__global__ void __launch_bounds__(BA) k_adj_gather2(phd_mesh M, phd_adj_index A, const double *__restrict__ cell_adj,
                                                    const double *__restrict__ entry_adj,
                                                    const double *__restrict__ self_adj,
                                                    double *__restrict__ prim_adj /* [4][n] */) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    if (x >= M.n_cells) return;
    const int n = M.n_cells, E2 = 2 * M.n_faces;
    const bool real = M.tag[x] == PHD_REAL_TAG;
    double s[4];
    for (int f = 0; f < 4; f++) s[f] = cell_adj[(size_t)f * n + x] + (real ? self_adj[(size_t)f * n + x] : 0.0);
    for (int e = M.nbr_ptr[x]; e < M.nbr_ptr[x + 1]; e++) {
        const int pe = A.partner[e];
        if (pe < 0 || pe >= E2) continue;
        for (int f = 0; f < 4; f++) s[f] += entry_adj[(size_t)f * E2 + pe];
    }
    for (int f = 0; f < 4; f++) prim_adj[(size_t)f * n + x] = s[f];
}

// per real cell: fold ghosts, reverse primitive recovery, add the identity of the update
__global__ void __launch_bounds__(BA) k_adj_final(phd_mesh M, phd_adj_index A, double gamma,
                                                  const double *__restrict__ cons, const double *__restrict__ prim_adj,
                                                  const double *__restrict__ lam_next, double *__restrict__ lam) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= M.n_cells) return;
    const int n = M.n_cells;
    if (M.tag[c] != PHD_REAL_TAG) {
        for (int q = 0; q < 4; q++) lam[(size_t)q * n + c] = 0.0;
        return;
    }
    double ap[4];
    for (int f = 0; f < 4; f++) ap[f] = prim_adj[(size_t)f * n + c];
    for (int t = A.ghost_ptr[c]; t < A.ghost_ptr[c + 1]; t++) {
        const int g = A.ghost_idx[t];
        const int fl = M.flip ? M.flip[g] : 0;
        for (int f = 0; f < 4; f++) {
            double v = prim_adj[(size_t)f * n + g];
            if ((f == 1 && (fl & 1)) || (f == 2 && (fl & 2))) v = -v;
            ap[f] += v;
        }
    }
    const double m = cons[c], mx = cons[(size_t)n + c], my = cons[2 * (size_t)n + c];
    const double vol = M.vol[c];
    const double rho = m / vol, vx = mx / m, vy = my / m;
    const double g1 = gamma - 1.0;
    // p = (E/V - rho v^2 / 2)(gamma - 1)
    const double arho = ap[0] - ap[3] * 0.5 * (vx * vx + vy * vy) * g1;
    const double avx = ap[1] - ap[3] * rho * vx * g1;
    const double avy = ap[2] - ap[3] * rho * vy * g1;
    const double aE = ap[3] * g1 / vol;
    const double am = arho / vol - avx * vx / m - avy * vy / m;
    lam[c] = lam_next[c] + am;
    lam[(size_t)n + c] = lam_next[(size_t)n + c] + avx / m;
    lam[2 * (size_t)n + c] = lam_next[2 * (size_t)n + c] + avy / m;
    lam[3 * (size_t)n + c] = lam_next[3 * (size_t)n + c] + aE;
}

inline int ba(int n) { return block_for(n, BA); }
inline int ga(int n) { return grid_for_block(n, ba(n)); }

}  // namespace phd

using namespace phd;

extern "C" {

static int adjoint_step(const phd_mesh *mesh, const phd_adj_index *index, const phd_params *par, double dt,
                        const double *cons, const double *prim, const double *grad, const double *face_w,
                        const double *lam_next, double *lam, double *work, const double *tape_f64,
                        const int32_t *tape_i32, cudaStream_t stream);

int phd_adjoint_step_f64(const phd_mesh *mesh, const phd_adj_index *index, const phd_params *par, double dt,
                         const double *cons, const double *prim, const double *grad, const double *face_w,
                         const double *lam_next, double *lam, double *work, cudaStream_t stream) {
    phd::NvtxRange nvtx_range("phd_adjoint_step_f64");
    return adjoint_step(mesh, index, par, dt, cons, prim, grad, face_w, lam_next, lam, work, nullptr, nullptr,
                        stream);
}

int phd_adjoint_step_f64_taped(const phd_mesh *mesh, const phd_adj_index *index, const phd_params *par,
                               double dt, const double *cons, const double *prim, const double *grad,
                               const double *face_w, const double *lam_next, double *lam, double *work,
                               const double *tape_f64, const int32_t *tape_i32, cudaStream_t stream) {
    phd::NvtxRange nvtx_range("phd_adjoint_step_f64_taped");
    if (!tape_f64 || !tape_i32) return PHD_ERR_ARG;
    return adjoint_step(mesh, index, par, dt, cons, prim, grad, face_w, lam_next, lam, work, tape_f64, tape_i32,
                        stream);
}

static int adjoint_step(const phd_mesh *mesh, const phd_adj_index *index, const phd_params *par, double dt,
                        const double *cons, const double *prim, const double *grad, const double *face_w,
                        const double *lam_next, double *lam, double *work, const double *tape_f64,
                        const int32_t *tape_i32, cudaStream_t stream) {
    if (!mesh || mesh->dim != 2 || !index || !par || !cons || !prim || !lam_next || !lam || !work)
        return PHD_ERR_ARG;
    if (mesh->n_faces && !mesh->normal) return PHD_ERR_ARG;
    if (par->solver < PHD_HLL || par->solver > PHD_EXACT) return PHD_ERR_ARG;
    if (par->reconstruction == PHD_LINEAR && !grad) return PHD_ERR_ARG;
    const phd_mesh &M = *mesh;
    const size_t n = M.n_cells, F = M.n_faces;
    double *face_adj = work;                       // [24][F]
    double *cell_adj = face_adj + 24 * F;          // [12][n]
    double *entry_adj = cell_adj + 12 * n;         // [4][2F]
    double *self_adj = entry_adj + 8 * F;          // [4][n]
    double *prim_adj = self_adj + 4 * n;           // [4][n]
    cudaMemsetAsync(entry_adj, 0, sizeof(double) * 8 * F, stream);
    cudaMemsetAsync(self_adj, 0, sizeof(double) * 4 * n, stream);
    if (F && par->solver == PHD_EXACT)
        k_adj_face<true><<<ga((int)F), ba((int)F), 0, stream>>>(M, *par, dt, prim, grad, face_w, lam_next, face_adj);
    else if (F)
        k_adj_face<false><<<ga((int)F), ba((int)F), 0, stream>>>(M, *par, dt, prim, grad, face_w, lam_next, face_adj);
    k_adj_gather<<<ga((int)n), ba((int)n), 0, stream>>>(M, face_adj, cell_adj);
    if (par->reconstruction == PHD_LINEAR)
    {
        if (tape_f64)
            k_adj_grad<true><<<ga((int)n), ba((int)n), 0, stream>>>(M, *index, par->limiter, prim, cell_adj,
                                                                  entry_adj, self_adj, tape_f64, tape_i32);
        else
            k_adj_grad<false><<<ga((int)n), ba((int)n), 0, stream>>>(M, *index, par->limiter, prim, cell_adj,
                                                                   entry_adj, self_adj, nullptr, nullptr);
    }
    k_adj_gather2<<<ga((int)n), ba((int)n), 0, stream>>>(M, *index, cell_adj, entry_adj, self_adj, prim_adj);
    k_adj_final<<<ga((int)n), ba((int)n), 0, stream>>>(M, *index, par->gamma, cons, prim_adj, lam_next, lam);
    return cudaPeekAtLastError() == cudaSuccess ? PHD_OK : PHD_ERR_LAUNCH;
}

size_t phd_adjoint_work_doubles(int32_t n_cells, int32_t n_faces) {
    return (size_t)24 * n_faces + 12 * (size_t)n_cells + 8 * (size_t)n_faces + 8 * (size_t)n_cells;
}

}  // extern "C"

// ---- adjoint step that allocates nothing --------------------------------------------
// Work space for phd_adjoint_step_f64_noalloc: a fixed array in the library's device
// image, created on every GPU where the library is loaded and kept until the process
// exits.  Its size is the limit of that entry point (PHD_ADJ_NOALLOC_MAX_DOUBLES).
static __device__ __align__(256) double g_adj_scratch[PHD_ADJ_NOALLOC_MAX_DOUBLES];

namespace {

// Device address of g_adj_scratch in the current device's current context.  In host
// code the symbol name is only a host-side stand-in, so the address is asked from the
// runtime on every call (cheap once the library's device code is loaded there): a
// cached address would go stale after cudaDeviceReset, or point into the wrong module
// when the caller switches contexts.
double *adj_scratch_on_current_device(int *rc) {
    void *p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_adj_scratch);
    if (e != cudaSuccess || !p) {
        *rc = PHD_ERR_LAUNCH;
        return nullptr;
    }
    return static_cast<double *>(p);
}

}  // namespace

extern "C" {

int phd_adjoint_step_f64_noalloc(const phd_mesh *mesh, const phd_adj_index *index, const phd_params *par,
                                 double dt, const double *cons, const double *prim, const double *grad,
                                 const double *face_w, const double *lam_next, double *lam, cudaStream_t stream) {
    phd::NvtxRange nvtx_range("phd_adjoint_step_f64_noalloc");
    if (!mesh || mesh->n_cells < 0 || mesh->n_faces < 0) return PHD_ERR_ARG;
    if (phd_adjoint_work_doubles(mesh->n_cells, mesh->n_faces) > (size_t)PHD_ADJ_NOALLOC_MAX_DOUBLES)
        return PHD_ERR_SCRATCH_TOO_SMALL;
    int rc = PHD_OK;
    double *work = adj_scratch_on_current_device(&rc);
    if (!work) return rc;
    return phd_adjoint_step_f64(mesh, index, par, dt, cons, prim, grad, face_w, lam_next, lam, work, stream);
}

}  // extern "C"
