// phd_ref.cuh -- face extrapolation in the reference's own FP64 geometry (positions).
#pragma once
#include "phd_physics.cuh"

namespace phd {

// add_spatial reconstruction.pyx:832-921 for face m (reference geometry in FP64).
template <int DIM>
__device__ __forceinline__ void face_spatial_f64(const phd_mesh &M, int m, int i, int j, const double *pi,
                                                 const double *pj, const double *gi, const double *gj,
                                                 const double *w, bool boost, bool gizmo, double *L,
                                                 double *R) {
    constexpr int NF = DIM + 2;
    const int n = M.n_cells, F = M.n_faces;
    double sl[NF], sr[NF];
#pragma unroll
    for (int f = 0; f < NF; f++) { L[f] = pi[f]; R[f] = pj[f]; }
    if (boost) {
#pragma unroll
        for (int k = 0; k < DIM; k++) { L[1 + k] = pi[1 + k] - w[k]; R[1 + k] = pj[1 + k] - w[k]; }
    }
#pragma unroll
    for (int f = 0; f < NF; f++) { sl[f] = L[f]; sr[f] = R[f]; }
    double diff_mag = 0.0, sepi_mag = 0.0, sepj_mag = 0.0;
#pragma unroll
    for (int k = 0; k < DIM; k++) {
        const double fc = M.com[(size_t)k * F + m];
        const double xik = M.x[(size_t)k * n + i], xjk = M.x[(size_t)k * n + j];
        const double sepi = fc - (xik + M.dcom[(size_t)k * n + i]);
        const double sepj = fc - (xjk + M.dcom[(size_t)k * n + j]);
        sepi_mag = sepi_mag + sepi * sepi;
        sepj_mag = sepj_mag + sepj * sepj;
        diff_mag = diff_mag + t_sq(xjk - xik);
#pragma unroll
        for (int f = 0; f < NF; f++) {
            L[f] = L[f] + gi[f * DIM + k] * sepi;
            R[f] = R[f] + gj[f * DIM + k] * sepj;
        }
    }
    sepi_mag = sqrt(sepi_mag);
    sepj_mag = sqrt(sepj_mag);
    diff_mag = sqrt(diff_mag);
    if (gizmo) {
#pragma unroll
        for (int f = 0; f < NF; f++)
            gizmo_pair<double>(sl[f], sr[f], pi[f], pj[f], sepi_mag, sepj_mag, diff_mag, L[f], R[f]);
        if (L[0] < 0.0 || L[DIM + 1] < 0.0) {
#pragma unroll
            for (int f = 0; f < NF; f++) L[f] = sl[f];
        }
        if (R[0] < 0.0 || R[DIM + 1] < 0.0) {
#pragma unroll
            for (int f = 0; f < NF; f++) R[f] = sr[f];
        }
    }
}

}  // namespace phd
