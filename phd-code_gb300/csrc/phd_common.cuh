// phd_common.cuh -- shared constants, math overloads and small device helpers.
#pragma once
#include <atomic>
#include <cstdint>
#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>
#include "../../include/phdflux.h"

#define PHD_REAL_TAG 0
#define PHD_EXTERIOR_TYPE 2

#ifndef PHD_HD
#define PHD_HD __host__ __device__
#endif

namespace phd {

// A named NVTX range over the launches one entry point issues (Nsight tools can select
// kernels by it, e.g. ncu --nvtx --nvtx-include "phd_step_f32/"); header-only NVTX costs
// nothing when no tool is attached.
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
    NvtxRange(const NvtxRange &) = delete;
    NvtxRange &operator=(const NvtxRange &) = delete;
};

// Programmatic dependent launch (sm_90 and later).  pdl_launch_dependents lets the
// runtime schedule the next kernel of the stream (launched with programmatic stream
// serialization) into SM slots this grid frees; pdl_wait blocks until every
// prerequisite grid has completed and its memory operations are visible.  A kernel
// reads only data that no earlier kernel of the step writes (the mesh) before pdl_wait.
// Launched without the attribute, both are no-ops in effect.
__device__ __forceinline__ void pdl_launch_dependents() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }

// Threads per block for a launch over n items with at most max_block threads: halved
// (down to one warp) while the grid would not cover every SM twice, so small meshes
// (16k cells) still spread FP64-bound work over the whole GPU.
inline int sm_count_current() {
    static std::atomic<int> cached[64];
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return 152;
    int v = cached[dev].load(std::memory_order_relaxed);
    if (v <= 0) {
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || v <= 0) v = 152;
        cached[dev].store(v, std::memory_order_relaxed);
    }
    return v;
}

inline int block_for(int n, int max_block) {
    int b = max_block;
    const long long want = 2LL * sm_count_current();
    while (b > 32 && ((long long)n + b - 1) / b < want) b >>= 1;
    return b;
}

inline int grid_for_block(int n, int b) { return n > 0 ? (n + b - 1) / b : 1; }

// Type-generic math so one template body serves the FP64 and FP32 builds.
PHD_HD __forceinline__ double t_sqrt(double a) { return sqrt(a); }
PHD_HD __forceinline__ float t_sqrt(float a) { return sqrtf(a); }
PHD_HD __forceinline__ double t_pow(double a, double b) { return pow(a, b); }
PHD_HD __forceinline__ float t_pow(float a, float b) { return powf(a, b); }
PHD_HD __forceinline__ double t_fmax(double a, double b) { return fmax(a, b); }
PHD_HD __forceinline__ float t_fmax(float a, float b) { return fmaxf(a, b); }
PHD_HD __forceinline__ double t_fmin(double a, double b) { return fmin(a, b); }
PHD_HD __forceinline__ float t_fmin(float a, float b) { return fminf(a, b); }
PHD_HD __forceinline__ double t_fabs(double a) { return fabs(a); }
PHD_HD __forceinline__ float t_fabs(float a) { return fabsf(a); }
// x**2 in the reference lowers to libm pow(x, 2.0).  Neither CUDA's pow nor the
// product reproduces every glibc result bit for bit (each is within an ulp of it); the
// product is the exactly rounded square and costs one FP64 multiply instead of a pow.
PHD_HD __forceinline__ double t_sq(double a) { return a * a; }
PHD_HD __forceinline__ float t_sq(float a) { return a * a; }

// Positive doubles order like their bit patterns: min-reduce them as integers.
__device__ __forceinline__ unsigned long long dbits(double v) {
    return static_cast<unsigned long long>(__double_as_longlong(v));
}

__device__ __forceinline__ double warp_min(double v) {
    for (int o = 16; o > 0; o >>= 1) v = fmin(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Block-wide min of positive doubles into *slot (bit-pattern atomicMin).  Every
// thread of the block must call it.
__device__ __forceinline__ void block_min_to(double v, unsigned long long *slot) {
    __shared__ double s_min[32];
    v = warp_min(v);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) s_min[wid] = v;
    __syncthreads();
    if (wid == 0) {
        const int nw = (blockDim.x + 31) >> 5;
        double u = (lane < nw) ? s_min[lane] : INFINITY;
        u = warp_min(u);
        if (lane == 0 && u < INFINITY) atomicMin(slot, dbits(u));
    }
}

// FP32 <-> FP64 conversions done with integer operations, for kernels whose FP64
// pipe is the bottleneck (GB300 issues FP64 at a small fraction of the FP32 rate).
// Zero / denormal inputs map to signed zero; infinities stay infinite and NaN stays NaN.
__device__ __forceinline__ double widen_f32(float f) {
    const unsigned u = __float_as_uint(f);
    const unsigned ex = (u >> 23) & 0xffu;
    const unsigned e64 = (ex == 0xffu) ? 0x7ffu : ex + 896u;
    const unsigned hi = (u & 0x80000000u) | (e64 << 20) | ((u & 0x7fffffu) >> 3);
    const unsigned lo = u << 29;
    return __hiloint2double((int)(ex ? hi : (u & 0x80000000u)), (int)(ex ? lo : 0u));
}

// The same for finite inputs only (an infinity or NaN comes out as a finite value of
// magnitude >= 2^128): the hot update path, which range-checks its FP64 results instead
// (fp64_beyond_f32).
__device__ __forceinline__ double widen_f32_finite(float f) {
    const unsigned u = __float_as_uint(f);
    const unsigned ex = (u >> 23) & 0xffu;
    const unsigned hi = (u & 0x80000000u) | ((ex + 896u) << 20) | ((u & 0x7fffffu) >> 3);
    const unsigned lo = u << 29;
    return __hiloint2double((int)(ex ? hi : (u & 0x80000000u)), (int)(ex ? lo : 0u));
}

// Round-to-nearest-even FP64 -> FP32 for magnitudes below 2^128 (smaller magnitudes
// than the FP32 normal range flush to signed zero): the hot update path, after
// fp64_beyond_f32 has ruled out everything else.
__device__ __forceinline__ float narrow_f64_finite(double d) {
    const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(d));
    const unsigned sign = static_cast<unsigned>(b >> 32) & 0x80000000u;
    const int ex = static_cast<int>((b >> 52) & 0x7ffull) - 896;
    const unsigned m23 = static_cast<unsigned>((b >> 29) & 0x7fffffull);
    const unsigned rem = static_cast<unsigned>(b & 0x1fffffffull);
    const unsigned up = (rem > 0x10000000u) || (rem == 0x10000000u && (m23 & 1u));
    const unsigned mag = ((static_cast<unsigned>(ex) << 23) | m23) + up;
    return __uint_as_float(ex > 0 ? (sign | mag) : sign);
}

// True when |d| >= 2^127 (so it may round beyond FLT_MAX), or d is infinite or NaN:
// one look at the exponent field.
__device__ __forceinline__ bool fp64_beyond_f32(double d) {
    return (static_cast<unsigned>(__double2hiint(d)) & 0x7ff00000u) >= ((1023u + 127u) << 20);
}

// Round-to-nearest-even FP64 -> FP32.  Magnitudes below the FP32 normal range flush
// to signed zero; magnitudes that round above FLT_MAX, and infinities, give signed
// infinity; NaN gives NaN -- so a blown-up FP64 total never turns into a plausible
// finite float.
__device__ __forceinline__ float narrow_f64(double d) {
    const unsigned long long b = static_cast<unsigned long long>(__double_as_longlong(d));
    const unsigned sign = static_cast<unsigned>(b >> 32) & 0x80000000u;
    const int ex = static_cast<int>((b >> 52) & 0x7ffull) - 896;
    const unsigned m23 = static_cast<unsigned>((b >> 29) & 0x7fffffull);
    const unsigned rem = static_cast<unsigned>(b & 0x1fffffffull);
    const unsigned up = (rem > 0x10000000u) || (rem == 0x10000000u && (m23 & 1u));
    // exponents 1..254: a carry out of the mantissa lands on the next binade, and out
    // of binade 254 on the infinity pattern 0x7f800000
    const unsigned mag = ((static_cast<unsigned>(ex) << 23) | m23) + up;
    const bool nan = (b & 0x7fffffffffffffffull) > 0x7ff0000000000000ull;
    const unsigned big = nan ? 0x7fc00000u : (sign | 0x7f800000u);
    return __uint_as_float(ex >= 255 ? big : (ex > 0 ? (sign | mag) : sign));
}

__device__ __forceinline__ float warp_min_f(float v) {
    for (int o = 16; o > 0; o >>= 1) v = fminf(v, __shfl_xor_sync(0xffffffffu, v, o));
    return v;
}

// Block-wide min of positive floats, merged into the double accumulator *slot.
__device__ __forceinline__ void block_min_to_f(float v, unsigned long long *slot) {
    __shared__ float s_minf[32];
    v = warp_min_f(v);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) s_minf[wid] = v;
    __syncthreads();
    if (wid == 0) {
        const int nw = (blockDim.x + 31) >> 5;
        float u = (lane < nw) ? s_minf[lane] : INFINITY;
        u = warp_min_f(u);
        if (lane == 0 && u < INFINITY) atomicMin(slot, dbits((double)u));
    }
}

// Turn one run's CFL minimum into its next time step (cfl * min, clipped to land on
// t_end) and re-arm its accumulator; with `advance` the clock first moves past the
// step just taken (t += dt, step += 1).
__device__ __forceinline__ void finalize_clock(phd_clock *clk, double cfl, bool advance) {
    const unsigned long long bits = atomicAdd(&clk->dtmin_bits, 0ull);
    const double mn = __longlong_as_double(static_cast<long long>(bits));
    if (advance) {
        clk->t = clk->t + clk->dt;
        clk->dt_last = clk->dt;
        clk->step = clk->step + 1;
    }
    double dt = cfl * mn;
    clk->dt_hydro = dt;
    // Time.modify_timestep + Simulation.compute_time_step (simulation_finish.py:82-88,
    // simulation.py:201-212): land exactly on t_end.
    if (clk->t_end > 0.0 && clk->t + dt >= clk->t_end) dt = fmin(clk->t_end - clk->t, dt);
    clk->dt = dt;
    clk->dtmin_bits = dbits(INFINITY);
}

// Finish a grid-wide CFL reduction over n_runs clocks: the last block to arrive
// finalises every run.  No block waits on another: every block reads the clocks'
// dt before its arrival is counted (clocks[0].arrive), and only the last arrival
// writes them.  The block's minimum reached L2 through an atomic issued by thread 0
// (block_min_to / block_min_to_f); thread 0 alone fences before counting the arrival
// (release), so the block's other threads never wait for their own outstanding stores.
// Per-run minima issued by other threads (the batched path) are fenced where they are
// issued (atomic_min_fenced).
__device__ __forceinline__ void finish_cfl_multi(phd_clock *clocks, int n_runs, double cfl, bool advance) {
    __shared__ bool s_last;
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        const unsigned int prev = atomicAdd(&clocks[0].arrive, 1u);
        s_last = (prev == gridDim.x - 1);
    }
    __syncthreads();
    if (s_last) {
        __threadfence();
        for (int r = threadIdx.x; r < n_runs; r += blockDim.x) finalize_clock(clocks + r, cfl, advance);
        __syncthreads();
        if (threadIdx.x == 0) clocks[0].arrive = 0u;
        __threadfence();
    }
}

// A per-run CFL candidate merged by a thread other than the block's thread 0: the
// fence orders it before the block's arrival (finish_cfl_multi).
__device__ __forceinline__ void atomic_min_fenced(unsigned long long *slot, unsigned long long v) {
    atomicMin(slot, v);
    __threadfence();
}

__device__ __forceinline__ void finish_cfl(phd_clock *clk, double cfl, bool advance) {
    finish_cfl_multi(clk, 1, cfl, advance);
}

// The compact FP32 face geometry from one interleaved (area, offset) array [F][2]
// (defined with the FP32 kernels).
int prepare_faces32_interleaved(const phd_mesh *mesh, const float *face32, phd_geom32_out *out, cudaStream_t stream);
// The tail of an FP32 mesh hand-over in one kernel (defined with the FP32 kernels):
// cell geometry from the prepared faces and lists, ghost totals from their images,
// primitives and the next dt.
int cells_prim_f32(const phd_mesh *mesh, const phd_params *par, const phd_geom32_out *out, double *cons,
                   float *prim4, phd_clock *clk, cudaStream_t stream);

// FP32 list codes of cell c's list entries [e0, e1) (face ids in idx, ascending): the
// face id where c is pair-i, ~face id where it is pair-j, and the other cell.  Where a
// twin table is given (periodic faces the reference computes twice, once from each
// side), the entry of a dropped twin points at the kept face from the other side.
// Invalid face ids give (0, c); an out-of-range other cell gives c.  Each chunk's
// gathers are issued together.
__device__ __forceinline__ void emit_list_codes(int c, int e0, int e1, int n, int F, const int32_t *idx,
                                                const int32_t *__restrict__ pair_i,
                                                const int32_t *__restrict__ pair_j,
                                                const int32_t *__restrict__ twin, int32_t *__restrict__ csr_face,
                                                int32_t *__restrict__ csr_nbr) {
    constexpr int CH = 4;
    for (int eb = e0; eb < e1; eb += CH) {
        int fid[CH], a[CH], b[CH], t[CH];
#pragma unroll
        for (int k = 0; k < CH; k++) fid[k] = idx[(eb + k < e1) ? eb + k : e0];
#pragma unroll
        for (int k = 0; k < CH; k++) {
            const bool ok = fid[k] >= 0 && fid[k] < F;
            a[k] = ok ? pair_i[fid[k]] : -1;
            b[k] = ok ? pair_j[fid[k]] : -1;
            t[k] = (ok && twin) ? twin[fid[k]] : -1;
        }
#pragma unroll
        for (int k = 0; k < CH; k++) {
            const int e = eb + k;
            if (e >= e1) break;
            if (fid[k] < 0 || fid[k] >= F) { csr_face[e] = 0; csr_nbr[e] = c; continue; }
            const bool as_i = (a[k] == c);
            int other = as_i ? b[k] : a[k];
            int code = as_i ? fid[k] : ~fid[k];
            if (as_i && t[k] >= 0 && t[k] < F) {   // this face is dropped: use the twin from the j side
                code = ~t[k];
                other = pair_i[t[k]];
            }
            if (other < 0 || other >= n) other = c;
            csr_face[e] = code;
            csr_nbr[e] = other;
        }
    }
}

}  // namespace phd
