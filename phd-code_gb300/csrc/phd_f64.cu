// phd_f64.cu -- FP64 kernels: one per reference plugin stage, plus the fused step.
//
// Compiled with --fmad=false: every product and sum rounds separately, as in the
// reference's Cython build, so results match the reference to the last few ulps
// (only CUDA's pow/sqrt library rounding can differ from libm's).
#include "phd_common.cuh"
#include "phd_physics.cuh"
#include "phd_ref.cuh"

namespace phd {

constexpr int BLOCK = 256;

__device__ __forceinline__ void set_status(phd_clock *clk, int bits) {
    if (bits && clk) atomicOr(&clk->status, bits);
}

// ---- gradients ------------------------------------------------------------------
// Limiter record of one cell's gradient, kept by a taped forward step for the adjoint:
// f64 [12][n]: the unlimited estimate (8 rows) and the limiter values (4 rows);
// i32 [13][n]: per field the CSR entry of the active limit (-1: none, -2: a clamp at
// zero or a flat field), the entries of the neighbour maximum and minimum (-1: the
// cell itself), and (TESS) the field of the active limit.
struct GradTape {
    double *f64;
    int32_t *i32;
};

// PieceWiseLinear.compute_gradients reconstruction.pyx:620-736 for cell c, result in
// df (limited).  Returns status bits.  TAPE: also records the limiter's selections
// (same arithmetic; only bookkeeping is added) when `record`.
template <int DIM, bool TAPE = false>
__device__ int cell_gradient_f64(const phd_mesh &M, const double *__restrict__ prim, int limiter,
                                 int c, double *df, GradTape tape = GradTape{nullptr, nullptr},
                                 bool record = false) {
    constexpr int NF = DIM + 2;
    const int n = M.n_cells, F = M.n_faces;
    double phi_max[NF], phi_min[NF], alpha[NF], xi[DIM], cx[DIM], pc[NF];
    int arg_max[NF], arg_min[NF], act[NF], act_f0 = -1;
    int status = 0;
#pragma unroll
    for (int k = 0; k < DIM; k++) {
        xi[k] = M.x[(size_t)k * n + c];
        cx[k] = xi[k] + M.dcom[(size_t)k * n + c];
    }
    const double vol = M.vol[c];
#pragma unroll
    for (int f = 0; f < NF; f++) {
        pc[f] = prim[(size_t)f * n + c];
        phi_max[f] = phi_min[f] = pc[f];
        alpha[f] = 1.0;
        arg_max[f] = arg_min[f] = act[f] = -1;
#pragma unroll
        for (int k = 0; k < DIM; k++) df[DIM * f + k] = 0;
    }
    const int m0 = M.nbr_ptr[c], m1 = M.nbr_ptr[c + 1];
    for (int m = m0; m < m1; m++) {
        const int fid = M.nbr_idx[m];
        if (fid < 0 || fid >= F) { status |= PHD_STATUS_BAD_INDEX; continue; }
        const double area = M.area[fid];
        int j;
        const int a = M.pair_i[fid], b = M.pair_j[fid];
        if (c == a) j = b;
        else if (c == b) j = a;
        else { status |= PHD_STATUS_BAD_INDEX; continue; }
        if (j < 0 || j >= n) { status |= PHD_STATUS_BAD_INDEX; continue; }
        double cfx[DIM], dr[DIM], r = 0.0;
#pragma unroll
        for (int k = 0; k < DIM; k++) {
            const double xj = M.x[(size_t)k * n + j];
            cfx[k] = M.com[(size_t)k * F + fid] - 0.5 * (xi[k] + xj);
            dr[k] = xi[k] - xj;
            r = r + t_sq(dr[k]);
        }
        r = sqrt(r);
#pragma unroll
        for (int f = 0; f < NF; f++) {
            const double pj = prim[(size_t)f * n + j];
            if (TAPE) {
                if (pj > phi_max[f]) arg_max[f] = m;
                if (pj < phi_min[f]) arg_min[f] = m;
            }
            phi_max[f] = fmax(phi_max[f], pj);
            phi_min[f] = fmin(phi_min[f], pj);
            const double d_dif = pj - pc[f];
            const double d_sum = pj + pc[f];
#pragma unroll
            for (int k = 0; k < DIM; k++)
                df[DIM * f + k] = df[DIM * f + k] + (area * ((d_dif * cfx[k]) - ((0.5 * d_sum) * dr[k]))) / (r * vol);
        }
    }
    if (limiter == PHD_LIMITER_AREPO) {
        for (int m = m0; m < m1; m++) {
            const int fid = M.nbr_idx[m];
            if (fid < 0 || fid >= F) continue;
            double sep[DIM];
#pragma unroll
            for (int k = 0; k < DIM; k++) sep[k] = M.com[(size_t)k * F + fid] - cx[k];
#pragma unroll
            for (int f = 0; f < NF; f++) {
                double dphi = 0.0, psi;
#pragma unroll
                for (int k = 0; k < DIM; k++) dphi = dphi + df[DIM * f + k] * sep[k];
                if (dphi > 0) psi = (phi_max[f] - pc[f]) / dphi;
                else if (dphi < 0) psi = (phi_min[f] - pc[f]) / dphi;
                else psi = 1.0;
                if (TAPE && fmax(psi, 0.) < alpha[f]) act[f] = (psi > 0.0 && dphi != 0.0) ? m : -2;
                alpha[f] = fmin(alpha[f], fmax(psi, 0.));
            }
        }
    } else if (limiter == PHD_LIMITER_TESS) {
        for (int m = m0; m < m1; m++) {
            const int fid = M.nbr_idx[m];
            if (fid < 0 || fid >= F) continue;
            const int a = M.pair_i[fid], b = M.pair_j[fid];
            const int j = (c == a) ? b : a;
            if (j < 0 || j >= n) continue;
            double sep[DIM];
#pragma unroll
            for (int k = 0; k < DIM; k++) sep[k] = M.com[(size_t)k * F + fid] - cx[k];
#pragma unroll
            for (int f = 0; f < NF; f++) {
                double dphi = 0.0, psi;
#pragma unroll
                for (int k = 0; k < DIM; k++) dphi = dphi + df[DIM * f + k] * sep[k];
                if (dphi > 0.0 || dphi < 0.0) {
                    const double t = (prim[(size_t)f * n + j] - pc[f]) / dphi;
                    psi = (0. > t) ? 0. : t;
                } else psi = 1.0;
                if (TAPE && fmax(psi, 0.) < alpha[0]) {
                    act[0] = (psi > 0.0 && dphi != 0.0) ? m : -2;
                    act_f0 = f;
                }
                alpha[0] = fmin(alpha[0], fmax(psi, 0.));     // only alpha[0]: :731
            }
        }
    }
    if (TAPE && record) {
#pragma unroll
        for (int r = 0; r < NF * DIM; r++) tape.f64[(size_t)r * n + c] = df[r];
#pragma unroll
        for (int f = 0; f < NF; f++) {
            tape.f64[(size_t)(NF * DIM + f) * n + c] = alpha[f];
            tape.i32[(size_t)f * n + c] = act[f];
            tape.i32[(size_t)(NF + f) * n + c] = arg_max[f];
            tape.i32[(size_t)(2 * NF + f) * n + c] = arg_min[f];
        }
        tape.i32[(size_t)(3 * NF) * n + c] = act_f0;
    }
#pragma unroll
    for (int f = 0; f < NF; f++)
#pragma unroll
        for (int k = 0; k < DIM; k++) df[DIM * f + k] = alpha[f] * df[DIM * f + k];
    return status;
}

// Real rows: own gradient.  Ghost rows: the image's gradient (computed again from the
// image's faces, bit-identical), with the reflective diagonal flip of grad v
// (domain_manager.pyx:819-835, boundary.pyx:287-307).
template <int DIM, bool TAPE = false>
__global__ void __launch_bounds__(BLOCK) k_gradients(phd_mesh M, const double *__restrict__ prim,
                                                      int limiter, double *__restrict__ grad,
                                                      phd_clock *clk, GradTape tape = GradTape{nullptr, nullptr}) {
    constexpr int NF = DIM + 2;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= M.n_cells) return;
    int c = i;
    if (M.tag[i] != PHD_REAL_TAG) {
        c = M.map[i];
        if (c < 0 || c >= M.n_cells) { set_status(clk, PHD_STATUS_BAD_INDEX); return; }
    }
    double df[NF * DIM];
    const int st = cell_gradient_f64<DIM, TAPE>(M, prim, limiter, c, df, tape, i == c);
    set_status(clk, st);
    const int fl = M.flip ? M.flip[i] : 0;
#pragma unroll
    for (int kk = 0; kk < DIM; kk++)
        if (fl & (1 << kk)) df[DIM * (1 + kk) + kk] *= -1;
#pragma unroll
    for (int r = 0; r < NF * DIM; r++) grad[(size_t)r * M.n_cells + i] = df[r];
}

template <int DIM>
__device__ __forceinline__ void load_face_inputs(const phd_mesh &M, const double *__restrict__ prim,
                                                 const double *__restrict__ grad, const double *__restrict__ face_w,
                                                 int m, int i, int j, bool linear, double *pi, double *pj,
                                                 double *gi, double *gj, double *w) {
    constexpr int NF = DIM + 2;
    const int n = M.n_cells, F = M.n_faces;
#pragma unroll
    for (int f = 0; f < NF; f++) { pi[f] = prim[(size_t)f * n + i]; pj[f] = prim[(size_t)f * n + j]; }
    if (linear) {
#pragma unroll
        for (int r = 0; r < NF * DIM; r++) { gi[r] = grad[(size_t)r * n + i]; gj[r] = grad[(size_t)r * n + j]; }
    }
#pragma unroll
    for (int k = 0; k < DIM; k++) w[k] = face_w ? face_w[(size_t)k * F + m] : 0.0;
}

template <int DIM>
__device__ __forceinline__ void face_states_f64(const phd_mesh &M, int m, int i, int j, const double *pi,
                                                const double *pj, const double *gi, const double *gj,
                                                const double *w, double gamma, double dt_half, bool boost,
                                                bool linear, bool gizmo, double *L, double *R) {
    constexpr int NF = DIM + 2;
    if (linear) {
        face_spatial_f64<DIM>(M, m, i, j, pi, pj, gi, gj, w, boost, gizmo, L, R);
        temporal<double, DIM>(L, R, pi, pj, gi, gj, w, gamma, dt_half, boost);
    } else {                                   // PieceWiseConstant :323-352
#pragma unroll
        for (int f = 0; f < NF; f++) { L[f] = pi[f]; R[f] = pj[f]; }
        if (boost) {
#pragma unroll
            for (int k = 0; k < DIM; k++) { L[1 + k] = pi[1 + k] - w[k]; R[1 + k] = pj[1 + k] - w[k]; }
        }
    }
}

template <int DIM>
__global__ void __launch_bounds__(BLOCK) k_states(phd_mesh M, const double *__restrict__ prim,
                                                   const double *__restrict__ grad, const double *__restrict__ face_w,
                                                   double gamma, double dt_half, int boost, int linear, int gizmo,
                                                   int stages, double *__restrict__ left,
                                                   double *__restrict__ right) {
    constexpr int NF = DIM + 2;
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= M.n_faces) return;
    const int i = M.pair_i[m], j = M.pair_j[m];
    if (i < 0 || i >= M.n_cells || j < 0 || j >= M.n_cells) return;
    double pi[NF], pj[NF], gi[NF * DIM], gj[NF * DIM], w[DIM], L[NF], R[NF];
    load_face_inputs<DIM>(M, prim, grad, face_w, m, i, j, linear, pi, pj, gi, gj, w);
    if (!linear || stages == (PHD_STAGE_SPATIAL | PHD_STAGE_TEMPORAL)) {
        face_states_f64<DIM>(M, m, i, j, pi, pj, gi, gj, w, gamma, dt_half, boost, linear, gizmo, L, R);
    } else if (stages == PHD_STAGE_SPATIAL) {
        face_spatial_f64<DIM>(M, m, i, j, pi, pj, gi, gj, w, boost, gizmo, L, R);
    } else {
#pragma unroll
        for (int f = 0; f < NF; f++) {
            L[f] = left[(size_t)f * M.n_faces + m];
            R[f] = right[(size_t)f * M.n_faces + m];
        }
        temporal<double, DIM>(L, R, pi, pj, gi, gj, w, gamma, dt_half, boost);
    }
#pragma unroll
    for (int f = 0; f < NF; f++) {
        left[(size_t)f * M.n_faces + m] = L[f];
        right[(size_t)f * M.n_faces + m] = R[f];
    }
}

template <int DIM>
__global__ void __launch_bounds__(BLOCK) k_riemann(phd_mesh M, int solver, double gamma, int boost,
                                                    int max_iter, const double *__restrict__ left,
                                                    const double *__restrict__ right,
                                                    const double *__restrict__ face_w,
                                                    double *__restrict__ flux, phd_clock *clk) {
    constexpr int NF = DIM + 2;
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= M.n_faces) return;
    const int F = M.n_faces;
    double L[NF], R[NF], nrm[DIM], w[DIM], f[NF];
#pragma unroll
    for (int q = 0; q < NF; q++) { L[q] = left[(size_t)q * F + m]; R[q] = right[(size_t)q * F + m]; }
#pragma unroll
    for (int k = 0; k < DIM; k++) {
        nrm[k] = M.normal[(size_t)k * F + m];
        w[k] = face_w ? face_w[(size_t)k * F + m] : 0.0;
    }
    bool failed = false;
    riemann_flux<double, DIM>(solver, L, R, nrm, w, gamma, boost != 0, max_iter, f, &failed);
    if (failed) set_status(clk, PHD_STATUS_RIEMANN_NONCONVERGED);
#pragma unroll
    for (int q = 0; q < NF; q++) flux[(size_t)q * F + m] = f[q];
}

// Fused: states + Riemann + deboost per face; the states never reach memory.
template <int DIM>
__global__ void __launch_bounds__(BLOCK) k_face_flux(phd_mesh M, phd_params P, const double *__restrict__ prim,
                                                      const double *__restrict__ grad,
                                                      const double *__restrict__ face_w,
                                                      double *__restrict__ flux, phd_clock *clk) {
    constexpr int NF = DIM + 2;
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= M.n_faces) return;
    const int F = M.n_faces;
    const int i = M.pair_i[m], j = M.pair_j[m];
    if (i < 0 || i >= M.n_cells || j < 0 || j >= M.n_cells) { set_status(clk, PHD_STATUS_BAD_INDEX); return; }
    const bool boost = (P.solver == PHD_EXACT) ? true : (P.boost != 0);
    const bool linear = P.reconstruction == PHD_LINEAR;
    const double dt_half = 0.5 * clk->dt;
    double pi[NF], pj[NF], gi[NF * DIM], gj[NF * DIM], w[DIM], L[NF], R[NF], nrm[DIM], f[NF];
    load_face_inputs<DIM>(M, prim, grad, face_w, m, i, j, linear, pi, pj, gi, gj, w);
    face_states_f64<DIM>(M, m, i, j, pi, pj, gi, gj, w, P.gamma, dt_half, boost, linear, P.gizmo != 0, L, R);
#pragma unroll
    for (int k = 0; k < DIM; k++) nrm[k] = M.normal[(size_t)k * F + m];
    bool failed = false;
    riemann_flux<double, DIM>(P.solver, L, R, nrm, w, P.gamma, boost, P.exact_max_iter, f, &failed);
    if (failed) set_status(clk, PHD_STATUS_RIEMANN_NONCONVERGED);
#pragma unroll
    for (int q = 0; q < NF; q++) flux[(size_t)q * F + m] = f[q];
}

// ---- conserved update -----------------------------------------------------------
// Mesh.update_from_fluxes mesh.pyx:519-551 for cell c as a segmented sum over its
// faces in ascending face id (the order in which the reference's face loop reaches
// it): U -= dt*a*F where c is pair-i, U += dt*a*F where c is pair-j.
template <int DIM>
__device__ __forceinline__ int cell_update_f64(const phd_mesh &M, const double *__restrict__ flux, double dt,
                                               int c, double *U) {
    constexpr int NF = DIM + 2;
    const int F = M.n_faces;
    int status = 0;
    const int m0 = M.nbr_ptr[c], m1 = M.nbr_ptr[c + 1];
    for (int m = m0; m < m1; m++) {
        const int fid = M.nbr_idx[m];
        if (fid < 0 || fid >= F) { status |= PHD_STATUS_BAD_INDEX; continue; }
        const double a = M.area[fid];
        if (M.pair_i[fid] == c) {
#pragma unroll
            for (int q = 0; q < NF; q++) U[q] = U[q] - ((dt * a) * flux[(size_t)q * F + fid]);
        } else {
#pragma unroll
            for (int q = 0; q < NF; q++) U[q] = U[q] + ((dt * a) * flux[(size_t)q * F + fid]);
        }
        if (U[0] <= 0.0) status |= PHD_STATUS_NEG_MASS;
        if (U[DIM + 1] <= 0.0) status |= PHD_STATUS_NEG_ENERGY;
    }
    return status;
}

template <int DIM>
__global__ void __launch_bounds__(BLOCK) k_update(phd_mesh M, const double *__restrict__ flux, double dt,
                                                   double *__restrict__ cons, phd_clock *clk) {
    constexpr int NF = DIM + 2;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= M.n_cells || M.tag[i] != PHD_REAL_TAG) return;
    const int n = M.n_cells;
    double U[NF];
#pragma unroll
    for (int q = 0; q < NF; q++) U[q] = cons[(size_t)q * n + i];
    const int st = cell_update_f64<DIM>(M, flux, dt, i, U);
    set_status(clk, st);
#pragma unroll
    for (int q = 0; q < NF; q++) cons[(size_t)q * n + i] = U[q];
}

template <int DIM>
__global__ void __launch_bounds__(BLOCK) k_ghost_cons(phd_mesh M, double *__restrict__ cons) {
    constexpr int NF = DIM + 2;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= M.n_cells || M.tag[i] == PHD_REAL_TAG) return;
    const int n = M.n_cells, c = M.map[i];
    if (c < 0 || c >= n) return;
    const int fl = M.flip ? M.flip[i] : 0;
#pragma unroll
    for (int q = 0; q < NF; q++) {
        double u = cons[(size_t)q * n + c];
        if (q >= 1 && q <= DIM && (fl & (1 << (q - 1)))) u *= -1;
        cons[(size_t)q * n + i] = u;
    }
}

// IdealGas.primitive_from_conservative equation_state.pyx:106-117 for one cell.
template <int DIM>
__device__ __forceinline__ void prim_of(const double *U, double vol, double gamma, double *p) {
    const double m = U[0];
    const double d = m / vol;
    p[0] = d;
    double v_sq = 0.;
#pragma unroll
    for (int k = 0; k < DIM; k++) {
        const double v = U[1 + k] / m;
        p[1 + k] = v;
        v_sq = v_sq + v * v;
    }
    p[DIM + 1] = ((U[DIM + 1] / vol) - ((.5 * d) * v_sq)) * (gamma - 1.);
}

// CFL candidate of one real cell, RiemannBase.compute_time_step riemann.pyx:170-187.
template <int DIM>
__device__ __forceinline__ double cfl_candidate(const double *p, double vol, double gamma, bool boost) {
    const double c = sqrt((gamma * p[DIM + 1]) / p[0]);
    const double R = (DIM == 2) ? sqrt(vol / 3.141592653589793)
                                : pow((3.0 * vol) / (4.0 * 3.141592653589793), 1.0 / 3.0);
    if (boost) return R / c;
    double vsq = 0.0;
#pragma unroll
    for (int k = 0; k < DIM; k++) vsq = vsq + p[1 + k] * p[1 + k];
    return R / (c + sqrt(vsq));
}

template <int DIM>
__global__ void __launch_bounds__(BLOCK) k_prim_from_cons(int n, double gamma, const double *__restrict__ vol,
                                                           const double *__restrict__ cons, double *__restrict__ prim) {
    constexpr int NF = DIM + 2;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double U[NF], p[NF];
#pragma unroll
    for (int q = 0; q < NF; q++) U[q] = cons[(size_t)q * n + i];
    prim_of<DIM>(U, vol[i], gamma, p);
#pragma unroll
    for (int q = 0; q < NF; q++) prim[(size_t)q * n + i] = p[q];
}

// IdealGas.conservative_from_primitive equation_state.pyx:65-79.
template <int DIM>
__global__ void __launch_bounds__(BLOCK) k_cons_from_prim(int n, double gamma, const double *__restrict__ vol,
                                                           const double *__restrict__ prim, double *__restrict__ cons) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double d = prim[i];
    const double m = d * vol[i];
    cons[i] = m;
    double v_sq = 0.;
#pragma unroll
    for (int k = 0; k < DIM; k++) {
        const double v = prim[(size_t)(1 + k) * n + i];
        cons[(size_t)(1 + k) * n + i] = v * m;
        v_sq = v_sq + v * v;
    }
    cons[(size_t)(DIM + 1) * n + i] = (((.5 * d) * v_sq) + (prim[(size_t)(DIM + 1) * n + i] / (gamma - 1.))) * vol[i];
}

template <int DIM>
__global__ void __launch_bounds__(BLOCK) k_time_step(phd_mesh M, const double *__restrict__ prim, double gamma,
                                                      double cfl, int boost, int advance, phd_clock *clk) {
    constexpr int NF = DIM + 2;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = M.n_cells;
    double cand = INFINITY;
    if (i < n && M.tag[i] == PHD_REAL_TAG) {
        double p[NF];
#pragma unroll
        for (int q = 0; q < NF; q++) p[q] = prim[(size_t)q * n + i];
        cand = cfl_candidate<DIM>(p, M.vol[i], gamma, boost != 0);
    }
    block_min_to(cand, &clk->dtmin_bits);
    finish_cfl(clk, cfl, advance != 0);
}

// Fused end of step: segmented update into cons_next (ghosts redo their image's sum
// and flip the reflective momentum), primitive recovery for every cell and the CFL
// minimum over real cells for the next step.
template <int DIM>
__global__ void __launch_bounds__(BLOCK) k_update_step(phd_mesh M, phd_params P, const double *__restrict__ flux,
                                                        const double *__restrict__ cons,
                                                        double *__restrict__ cons_next,
                                                        double *__restrict__ prim, phd_clock *clk) {
    constexpr int NF = DIM + 2;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = M.n_cells;
    const double dt = clk->dt;
    double cand = INFINITY;
    if (i < n) {
        const bool real = M.tag[i] == PHD_REAL_TAG;
        const int c = real ? i : M.map[i];
        if (c >= 0 && c < n) {
            double U[NF], p[NF];
#pragma unroll
            for (int q = 0; q < NF; q++) U[q] = cons[(size_t)q * n + c];
            set_status(clk, cell_update_f64<DIM>(M, flux, dt, c, U));
            if (!real) {
                const int fl = M.flip ? M.flip[i] : 0;
#pragma unroll
                for (int k = 0; k < DIM; k++)
                    if (fl & (1 << k)) U[1 + k] *= -1;
            }
#pragma unroll
            for (int q = 0; q < NF; q++) cons_next[(size_t)q * n + i] = U[q];
            prim_of<DIM>(U, M.vol[i], P.gamma, p);
#pragma unroll
            for (int q = 0; q < NF; q++) prim[(size_t)q * n + i] = p[q];
            if (real) {
                const bool boost = (P.solver == PHD_EXACT) ? true : (P.boost != 0);
                cand = cfl_candidate<DIM>(p, M.vol[i], P.gamma, boost);
            }
        } else {
            set_status(clk, PHD_STATUS_BAD_INDEX);
        }
    }
    block_min_to(cand, &clk->dtmin_bits);
    finish_cfl(clk, P.cfl, true);
}

// ---- mesh motion ------------------------------------------------------------------
// Mesh.assign_generator_velocities mesh.pyx:397-426 (all cells).
template <int DIM>
__global__ void __launch_bounds__(BLOCK) k_gen_vel(phd_mesh M, const double *__restrict__ prim, double gamma,
                                                    double eta, int regularize, double *__restrict__ w) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int n = M.n_cells;
    if (i >= n) return;
    double wx[DIM];
#pragma unroll
    for (int k = 0; k < DIM; k++) wx[k] = prim[(size_t)(1 + k) * n + i];
    if (regularize) {
        const double c = sqrt((gamma * prim[(size_t)(DIM + 1) * n + i]) / prim[i]);
        double d = 0.0;
#pragma unroll
        for (int k = 0; k < DIM; k++) d = d + t_sq(M.dcom[(size_t)k * n + i]);
        d = sqrt(d);
        const double vol = M.vol[i];
        const double R = (DIM == 2) ? sqrt(vol / 3.141592653589793)
                                    : pow((3.0 * vol) / (4.0 * 3.141592653589793), 1.0 / 3.0);
        if ((0.9 <= (d / (eta * R))) && ((d / (eta * R)) < 1.1)) {
#pragma unroll
            for (int k = 0; k < DIM; k++)
                wx[k] = wx[k] + (((c * M.dcom[(size_t)k * n + i]) * (d - ((0.9 * eta) * R))) / (((d * 0.2) * eta) * R));
        } else if (1.1 <= (d / (eta * R))) {
#pragma unroll
            for (int k = 0; k < DIM; k++) wx[k] = wx[k] + ((c * M.dcom[(size_t)k * n + i]) / d);
        }
    }
#pragma unroll
    for (int k = 0; k < DIM; k++) w[(size_t)k * n + i] = wx[k];
}

// Mesh.assign_face_velocities mesh.pyx:462-477.
template <int DIM>
__global__ void __launch_bounds__(BLOCK) k_face_vel(phd_mesh M, const double *__restrict__ w,
                                                     double *__restrict__ face_w) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= M.n_faces) return;
    const int n = M.n_cells, F = M.n_faces;
    const int i = M.pair_i[m], j = M.pair_j[m];
    if (i < 0 || i >= n || j < 0 || j >= n) return;
    double factor = 0.0, denom = 0.0;
#pragma unroll
    for (int k = 0; k < DIM; k++) {
        const double xi = M.x[(size_t)k * n + i], xj = M.x[(size_t)k * n + j];
        factor = factor + ((w[(size_t)k * n + i] - w[(size_t)k * n + j]) * (M.com[(size_t)k * F + m] - (0.5 * (xi + xj))));
        denom = denom + t_sq(xj - xi);
    }
    factor = factor / denom;
#pragma unroll
    for (int k = 0; k < DIM; k++) {
        const double xi = M.x[(size_t)k * n + i], xj = M.x[(size_t)k * n + j];
        face_w[(size_t)k * F + m] = (0.5 * (w[(size_t)k * n + i] + w[(size_t)k * n + j])) + (factor * (xj - xi));
    }
}

inline int blk_of(int n) { return block_for(n, BLOCK); }
inline int grid_of(int n) { return grid_for_block(n, blk_of(n)); }

inline int launch_status() {
    return cudaPeekAtLastError() == cudaSuccess ? PHD_OK : PHD_ERR_LAUNCH;
}

inline bool mesh_ok(const phd_mesh *M) {
    return M && M->dim == 2 && M->n_cells > 0 && M->n_faces >= 0 && M->n_real <= M->n_cells;
}

}  // namespace phd

using namespace phd;

extern "C" {

int phd_abi_version(void) { return PHDFLUX_ABI_VERSION; }

const char *phd_status_string(int bit) {
    switch (bit) {
        case PHD_STATUS_NEG_MASS: return "Mass less than zero in flux update";
        case PHD_STATUS_NEG_ENERGY: return "Energy less than zero in flux update";
        case PHD_STATUS_RIEMANN_NONCONVERGED: return "No convergence in Exact Riemann Solver";
        case PHD_STATUS_BAD_INDEX: return "ERROR: incorrect neighbors!";
        case PHD_STATUS_LEFT_DOMAIN: return "particle left domain in reflective boundary condition!!";
        case PHD_STATUS_NONFINITE: return "Non-finite primitive state after flux update";
        default: return "unknown status";
    }
}

int phd_gradients_f64(const phd_mesh *mesh, const double *prim, int32_t limiter, double *grad,
                      phd_clock *clk, cudaStream_t stream) {
    if (!mesh_ok(mesh) || !prim || !grad) return PHD_ERR_ARG;
    k_gradients<2><<<grid_of(mesh->n_cells), blk_of(mesh->n_cells), 0, stream>>>(*mesh, prim, limiter, grad, clk);
    return launch_status();
}

int phd_gradients_f64_taped(const phd_mesh *mesh, const double *prim, int32_t limiter, double *grad,
                            double *tape_f64, int32_t *tape_i32, phd_clock *clk, cudaStream_t stream) {
    if (!mesh_ok(mesh) || !prim || !grad || !tape_f64 || !tape_i32) return PHD_ERR_ARG;
    k_gradients<2, true><<<grid_of(mesh->n_cells), blk_of(mesh->n_cells), 0, stream>>>(
        *mesh, prim, limiter, grad, clk, GradTape{tape_f64, tape_i32});
    return launch_status();
}

int phd_states_f64(const phd_mesh *mesh, const double *prim, const double *grad, const double *face_w,
                   double gamma, double dt_half, int32_t boost, int32_t reconstruction, int32_t gizmo,
                   int32_t stages, double *left, double *right, cudaStream_t stream) {
    if (!mesh_ok(mesh) || !prim || !left || !right) return PHD_ERR_ARG;
    if (reconstruction == PHD_LINEAR && !grad) return PHD_ERR_ARG;
    if (stages < 1 || stages > 3) return PHD_ERR_ARG;
    if (mesh->n_faces == 0) return PHD_OK;
    k_states<2><<<grid_of(mesh->n_faces), blk_of(mesh->n_faces), 0, stream>>>(*mesh, prim, grad, face_w, gamma, dt_half, boost,
                                                             reconstruction == PHD_LINEAR, gizmo, stages,
                                                             left, right);
    return launch_status();
}

int phd_riemann_f64(const phd_mesh *mesh, int32_t solver, double gamma, int32_t boost, int32_t exact_max_iter,
                    const double *left, const double *right, const double *face_w, double *flux,
                    phd_clock *clk, cudaStream_t stream) {
    if (!mesh_ok(mesh) || !left || !right || !flux) return PHD_ERR_ARG;
    if (mesh->n_faces && !mesh->normal) return PHD_ERR_ARG;
    if (solver < PHD_HLL || solver > PHD_EXACT) return PHD_ERR_ARG;
    if (mesh->n_faces == 0) return PHD_OK;
    k_riemann<2><<<grid_of(mesh->n_faces), blk_of(mesh->n_faces), 0, stream>>>(*mesh, solver, gamma, boost, exact_max_iter,
                                                              left, right, face_w, flux, clk);
    return launch_status();
}

int phd_update_from_fluxes_f64(const phd_mesh *mesh, const double *flux, double dt, double *cons,
                               phd_clock *clk, cudaStream_t stream) {
    if (!mesh_ok(mesh) || !flux || !cons) return PHD_ERR_ARG;
    k_update<2><<<grid_of(mesh->n_cells), blk_of(mesh->n_cells), 0, stream>>>(*mesh, flux, dt, cons, clk);
    return launch_status();
}

int phd_ghost_cons_f64(const phd_mesh *mesh, double *cons, cudaStream_t stream) {
    if (!mesh_ok(mesh) || !cons) return PHD_ERR_ARG;
    k_ghost_cons<2><<<grid_of(mesh->n_cells), blk_of(mesh->n_cells), 0, stream>>>(*mesh, cons);
    return launch_status();
}

int phd_prim_from_cons_f64(int32_t dim, int32_t n, double gamma, const double *vol, const double *cons,
                           double *prim, cudaStream_t stream) {
    if (dim != 2 || n <= 0 || !vol || !cons || !prim) return PHD_ERR_ARG;
    k_prim_from_cons<2><<<grid_of(n), blk_of(n), 0, stream>>>(n, gamma, vol, cons, prim);
    return launch_status();
}

int phd_cons_from_prim_f64(int32_t dim, int32_t n, double gamma, const double *vol, const double *prim,
                           double *cons, cudaStream_t stream) {
    if (dim != 2 || n <= 0 || !vol || !cons || !prim) return PHD_ERR_ARG;
    k_cons_from_prim<2><<<grid_of(n), blk_of(n), 0, stream>>>(n, gamma, vol, prim, cons);
    return launch_status();
}

int phd_time_step_f64(const phd_mesh *mesh, const double *prim, double gamma, double cfl, int32_t boost,
                      int32_t advance, phd_clock *clk, cudaStream_t stream) {
    if (!mesh_ok(mesh) || !prim || !clk) return PHD_ERR_ARG;
    k_time_step<2><<<grid_of(mesh->n_cells), blk_of(mesh->n_cells), 0, stream>>>(*mesh, prim, gamma, cfl, boost, advance, clk);
    return launch_status();
}

int phd_generator_velocities_f64(const phd_mesh *mesh, const double *prim, double gamma, double eta,
                                 int32_t regularize, double *w, cudaStream_t stream) {
    if (!mesh_ok(mesh) || !prim || !w) return PHD_ERR_ARG;
    k_gen_vel<2><<<grid_of(mesh->n_cells), blk_of(mesh->n_cells), 0, stream>>>(*mesh, prim, gamma, eta, regularize, w);
    return launch_status();
}

int phd_face_velocities_f64(const phd_mesh *mesh, const double *w, double *face_w, cudaStream_t stream) {
    if (!mesh_ok(mesh) || !w || !face_w) return PHD_ERR_ARG;
    if (mesh->n_faces == 0) return PHD_OK;
    k_face_vel<2><<<grid_of(mesh->n_faces), blk_of(mesh->n_faces), 0, stream>>>(*mesh, w, face_w);
    return launch_status();
}

static int step_f64(const phd_mesh *mesh, const phd_params *par, int32_t moving, double *prim, const double *cons,
                    double *cons_next, double *grad, double *w, double *face_w, double *flux, phd_clock *clk,
                    cudaStream_t stream, cudaEvent_t *marks, GradTape tape);

int phd_step_f64_marked(const phd_mesh *mesh, const phd_params *par, int32_t moving, double *prim,
                        const double *cons, double *cons_next, double *grad, double *w, double *face_w,
                        double *flux, phd_clock *clk, cudaStream_t stream, cudaEvent_t *marks) {
    phd::NvtxRange nvtx_range("phd_step_f64");
    return step_f64(mesh, par, moving, prim, cons, cons_next, grad, w, face_w, flux, clk, stream, marks,
                    GradTape{nullptr, nullptr});
}

int phd_step_f64_taped(const phd_mesh *mesh, const phd_params *par, int32_t moving, double *prim,
                       const double *cons, double *cons_next, double *grad, double *w, double *face_w,
                       double *flux, double *tape_f64, int32_t *tape_i32, phd_clock *clk, cudaStream_t stream) {
    phd::NvtxRange nvtx_range("phd_step_f64_taped");
    if (!tape_f64 || !tape_i32) return PHD_ERR_ARG;
    return step_f64(mesh, par, moving, prim, cons, cons_next, grad, w, face_w, flux, clk, stream, nullptr,
                    GradTape{tape_f64, tape_i32});
}

static int step_f64(const phd_mesh *mesh, const phd_params *par, int32_t moving, double *prim, const double *cons,
                    double *cons_next, double *grad, double *w, double *face_w, double *flux, phd_clock *clk,
                    cudaStream_t stream, cudaEvent_t *marks, GradTape tape) {
    if (!mesh_ok(mesh) || !par || !prim || !cons || !cons_next || !flux || !clk) return PHD_ERR_ARG;
    if (mesh->n_faces && !mesh->normal) return PHD_ERR_ARG;
    const bool linear = par->reconstruction == PHD_LINEAR;
    if (linear && !grad) return PHD_ERR_ARG;
    if (moving && (!w || !face_w)) return PHD_ERR_ARG;
    const int gc = grid_of(mesh->n_cells), gf = grid_of(mesh->n_faces);
    const int bc = blk_of(mesh->n_cells), bf = blk_of(mesh->n_faces);
    if (marks) cudaEventRecord(marks[0], stream);
    if (moving) {
        k_gen_vel<2><<<gc, bc, 0, stream>>>(*mesh, prim, par->gamma, par->eta, par->regularize, w);
        if (mesh->n_faces) k_face_vel<2><<<gf, bf, 0, stream>>>(*mesh, w, face_w);
    }
    if (linear) {
        if (tape.f64) k_gradients<2, true><<<gc, bc, 0, stream>>>(*mesh, prim, par->limiter, grad, clk, tape);
        else k_gradients<2><<<gc, bc, 0, stream>>>(*mesh, prim, par->limiter, grad, clk);
    }
    if (marks) cudaEventRecord(marks[1], stream);
    if (mesh->n_faces)
        k_face_flux<2><<<gf, bf, 0, stream>>>(*mesh, *par, prim, grad, face_w, flux, clk);
    if (marks) cudaEventRecord(marks[2], stream);
    k_update_step<2><<<gc, bc, 0, stream>>>(*mesh, *par, flux, cons, cons_next, prim, clk);
    if (marks) cudaEventRecord(marks[3], stream);
    return launch_status();
}

int phd_step_f64(const phd_mesh *mesh, const phd_params *par, int32_t moving, double *prim, const double *cons,
                 double *cons_next, double *grad, double *w, double *face_w, double *flux, phd_clock *clk,
                 cudaStream_t stream) {
    phd::NvtxRange nvtx_range("phd_step_f64");
    return phd_step_f64_marked(mesh, par, moving, prim, cons, cons_next, grad, w, face_w, flux, clk, stream,
                               nullptr);
}

}  // extern "C"
