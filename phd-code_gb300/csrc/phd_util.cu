// phd_util.cu -- mesh-preparation kernels: reflective flip bits and Hilbert keys.
#include "phd_common.cuh"

namespace phd {

constexpr int UBLOCK = 256;

// Reflective.update_gradients / update_fields (boundary.pyx:287-348) flip the normal
// velocity components of Exterior ghosts lying outside the box; precompute the bits.
__global__ void k_flip_mask(int dim, int n, const int8_t *__restrict__ type, const double *__restrict__ x,
                            double x0, double x1, double x2, double y0, double y1, double y2,
                            int reflective, int8_t *__restrict__ flip) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    int bits = 0;
    if (reflective && type[i] == PHD_EXTERIOR_TYPE) {
        const double lo[3] = {x0, x1, x2}, hi[3] = {y0, y1, y2};
        for (int k = 0; k < dim; k++) {
            const double v = x[(size_t)k * n + i];
            // two independent tests as in the reference: a ghost outside on both
            // sides of one axis cannot exist, so each axis flips at most once
            if (v < lo[k]) bits ^= (1 << k);
            if (v > hi[k]) bits ^= (1 << k);
        }
    }
    flip[i] = static_cast<int8_t>(bits);
}

// hilbert_key_2d hilbert.pyx:9-23 on xh = int32((x - corner) * fac)
// (LoadBalance.compute_hilbert_keys load_balance.pyx:212-215).
__global__ void k_hilbert_2d(int n, const double *__restrict__ x, double cx, double cy, double fac, int order,
                             int64_t *__restrict__ keys) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= n) return;
    int32_t xh = static_cast<int32_t>((x[p] - cx) * fac);
    int32_t yh = static_cast<int32_t>((x[(size_t)n + p] - cy) * fac);
    int64_t key = 0;
    for (int i = order - 1; i >= 0; i--) {
        const int xbit = (xh & (1 << i)) ? 1 : 0;
        const int ybit = (yh & (1 << i)) ? 1 : 0;
        if (xbit == 0 && ybit == 0) { const int32_t t = xh; xh = yh; yh = t; }
        else if (xbit == 1 && ybit == 0) { const int32_t t = xh; xh = ~yh; yh = ~t; }
        const int q = (xbit << 1) + ybit;
        const int idx = (q == 0) ? 0 : (q == 1) ? 1 : (q == 2) ? 3 : 2;     // key_index_2d
        key = (key << 2) + idx;
    }
    keys[p] = key;
}

}  // namespace phd

extern "C" {

int phd_flip_mask(int32_t dim, int32_t n, const int8_t *type, const double *x, const double *xmin,
                  const double *xmax, int32_t reflective, int8_t *flip, cudaStream_t stream) {
    if (dim < 2 || dim > 3 || n <= 0 || !type || !x || !xmin || !xmax || !flip) return PHD_ERR_ARG;
    double lo[3] = {0, 0, 0}, hi[3] = {0, 0, 0};
    for (int k = 0; k < dim; k++) { lo[k] = xmin[k]; hi[k] = xmax[k]; }
    phd::k_flip_mask<<<(n + phd::UBLOCK - 1) / phd::UBLOCK, phd::UBLOCK, 0, stream>>>(
        dim, n, type, x, lo[0], lo[1], lo[2], hi[0], hi[1], hi[2], reflective, flip);
    return cudaPeekAtLastError() == cudaSuccess ? PHD_OK : PHD_ERR_LAUNCH;
}

int phd_hilbert_keys_2d(int32_t n, const double *x, double corner_x, double corner_y, double fac, int32_t order,
                        int64_t *keys, cudaStream_t stream) {
    if (n <= 0 || !x || !keys || order < 1 || order > 31) return PHD_ERR_ARG;
    phd::k_hilbert_2d<<<(n + phd::UBLOCK - 1) / phd::UBLOCK, phd::UBLOCK, 0, stream>>>(n, x, corner_x, corner_y,
                                                                                     fac, order, keys);
    return cudaPeekAtLastError() == cudaSuccess ? PHD_OK : PHD_ERR_LAUNCH;
}

}  // extern "C"
