// phd_util.cu -- mesh-preparation kernels: reflective flip bits, Hilbert keys, and the
// quantities of an uploaded face list that the device derives instead of receiving them
// (face normals, neighbour lists).
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


// Face normal n = (x_j - x_i) / |x_j - x_i| as the tessellation forms it
// (tess.cpp:320-327, 367-369): h = sqrt(xr*xr + yr*yr), n = (xr/h, yr/h).  Explicit
// round-to-nearest operations keep the products and the sum unfused, so the result is
// the same double a host computes with IEEE arithmetic.
__global__ void k_face_normals(int n, int F, const int32_t *__restrict__ pair_i, const int32_t *__restrict__ pair_j,
                               const double *__restrict__ x, double *__restrict__ normal,
                               int32_t *__restrict__ bad) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= F) return;
    const int i = pair_i[m], j = pair_j[m];
    double nx = 0.0, ny = 0.0;
    if (i >= 0 && i < n && j >= 0 && j < n) {
        const double xr = __dsub_rn(x[j], x[i]);
        const double yr = __dsub_rn(x[(size_t)n + j], x[(size_t)n + i]);
        const double h = __dsqrt_rn(__dadd_rn(__dmul_rn(xr, xr), __dmul_rn(yr, yr)));
        nx = __ddiv_rn(xr, h);
        ny = __ddiv_rn(yr, h);
    } else if (bad) {
        atomicAdd(bad, 1);
    }
    normal[m] = nx;
    normal[(size_t)F + m] = ny;
}

// ---- neighbour lists from the face pairs -----------------------------------------
// The tessellation appends every face id to the lists of both its cells in creation
// order (tess.cpp:378-379), so each cell's list is its face ids in ascending order.
// Built here as: count per cell, exclusive scan to offsets, scatter with a per-cell
// cursor, then sort each cell's short list -- the scatter order does not matter, the
// result is deterministic.
constexpr int SCAN_THREADS = 1024, SCAN_ITEMS = 4, SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

__global__ void k_csr_count(int n, int F, const int32_t *__restrict__ pair_i, const int32_t *__restrict__ pair_j,
                            int32_t *__restrict__ cnt, int32_t *__restrict__ bad) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= F) return;
    const int i = pair_i[m], j = pair_j[m];
    if (i >= 0 && i < n && j >= 0 && j < n && i != j) {
        atomicAdd(&cnt[i], 1);
        atomicAdd(&cnt[j], 1);
    } else if (bad) {
        atomicAdd(bad, 1);
    }
}

// Exclusive prefix sum of one block's SCAN_TILE items (returns this thread's four
// exclusive prefixes and the tile total).
__device__ __forceinline__ void tile_scan(const int32_t v[SCAN_ITEMS], int32_t ex[SCAN_ITEMS], int32_t &total) {
    __shared__ int32_t s_warp[SCAN_THREADS / 32];
    int32_t run = 0;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) { ex[k] = run; run += v[k]; }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int32_t inc = run;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int32_t t = __shfl_up_sync(0xffffffffu, inc, o);
        if (lane >= o) inc += t;
    }
    if (lane == 31) s_warp[wid] = inc;
    __syncthreads();
    if (wid == 0) {
        int32_t w = s_warp[lane];
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int32_t t = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += t;
        }
        s_warp[lane] = w;                       // inclusive over warps
    }
    __syncthreads();
    const int32_t before = (wid ? s_warp[wid - 1] : 0) + inc - run;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) ex[k] += before;
    total = s_warp[SCAN_THREADS / 32 - 1];
    __syncthreads();
}

template <typename T>
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_tiles(int n, const T *__restrict__ cnt,
                                                             int32_t *__restrict__ tile_sum) {
    const int base = blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_ITEMS;
    int32_t v[SCAN_ITEMS], ex[SCAN_ITEMS], total;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) v[k] = (base + k < n) ? int32_t(cnt[base + k]) : 0;
    tile_scan(v, ex, total);
    if (threadIdx.x == 0) tile_sum[blockIdx.x] = total;
}

// one block: exclusive scan of the tile sums in place
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_tile_sums(int n_tiles, int32_t *__restrict__ tile_sum) {
    int32_t carry = 0;
    for (int b0 = 0; b0 < n_tiles; b0 += SCAN_TILE) {
        const int base = b0 + threadIdx.x * SCAN_ITEMS;
        int32_t v[SCAN_ITEMS], ex[SCAN_ITEMS], total;
#pragma unroll
        for (int k = 0; k < SCAN_ITEMS; k++) v[k] = (base + k < n_tiles) ? tile_sum[base + k] : 0;
        tile_scan(v, ex, total);
#pragma unroll
        for (int k = 0; k < SCAN_ITEMS; k++)
            if (base + k < n_tiles) tile_sum[base + k] = carry + ex[k];
        carry += total;
    }
}

// cap: offsets are clamped to it (list lengths from the host are not trusted to add
// up to the entries' storage; with them clamped every list stays inside it)
template <typename T>
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_offsets(int n, const T *__restrict__ cnt,
                                                               const int32_t *__restrict__ tile_sum,
                                                               int32_t *__restrict__ ptr, int cap) {
    const int base = blockIdx.x * SCAN_TILE + threadIdx.x * SCAN_ITEMS;
    int32_t v[SCAN_ITEMS], ex[SCAN_ITEMS], total;
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) v[k] = (base + k < n) ? int32_t(cnt[base + k]) : 0;
    tile_scan(v, ex, total);
    const int32_t off = tile_sum[blockIdx.x];
#pragma unroll
    for (int k = 0; k < SCAN_ITEMS; k++) {
        if (base + k < n) ptr[base + k] = min(off + ex[k], cap);
        if (base + k == n - 1) ptr[n] = min(off + ex[k] + v[k], cap);
    }
}

__global__ void k_csr_scatter(int n, int F, const int32_t *__restrict__ pair_i, const int32_t *__restrict__ pair_j,
                              const int32_t *__restrict__ ptr, int32_t *__restrict__ cursor,
                              int32_t *__restrict__ idx) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= F) return;
    const int i = pair_i[m], j = pair_j[m];
    if (i >= 0 && i < n && j >= 0 && j < n && i != j) {
        idx[ptr[i] + atomicAdd(&cursor[i], 1)] = m;
        idx[ptr[j] + atomicAdd(&cursor[j], 1)] = m;
    }
}

// Sort each cell's list.  Lists of up to 16 entries (every cell of a 2D Voronoi mesh
// but rare outliers) are sorted in registers with an odd-even transposition network of
// 8 or 16 lanes; longer lists fall back to an insertion sort in place.
template <int N>
__device__ __forceinline__ void sort_list_regs(int32_t *__restrict__ idx, int e0, int d) {
    int32_t v[N];
#pragma unroll
    for (int k = 0; k < N; k++) v[k] = (k < d) ? idx[e0 + k] : INT32_MAX;
#pragma unroll
    for (int r = 0; r < N; r++) {
#pragma unroll
        for (int k = (r & 1); k + 1 < N; k += 2) {
            const int32_t a = v[k], b = v[k + 1];
            v[k] = min(a, b);
            v[k + 1] = max(a, b);
        }
    }
#pragma unroll
    for (int k = 0; k < N; k++)
        if (k < d) idx[e0 + k] = v[k];
}

__device__ __forceinline__ void sort_list(int32_t *__restrict__ idx, int e0, int e1) {
    const int d = e1 - e0;
    if (d <= 1) return;
    if (d <= 8) { sort_list_regs<8>(idx, e0, d); return; }
    if (d <= 16) { sort_list_regs<16>(idx, e0, d); return; }
    for (int e = e0 + 1; e < e1; e++) {
        const int32_t v = idx[e];
        int k = e - 1;
        while (k >= e0 && idx[k] > v) {
            idx[k + 1] = idx[k];
            k--;
        }
        idx[k + 1] = v;
    }
}

__global__ void k_csr_sort(int n, const int32_t *__restrict__ ptr, int32_t *__restrict__ idx) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n) return;
    sort_list(idx, ptr[c], ptr[c + 1]);
}

// The FP32 list codes of cell c's sorted list entries [e0, e1) of src (face ids), for a
// hand-over whose faces come in per-real-cell ranges ([f0, f1) the cell's own, empty
// for a ghost), written at the same positions of code / nbr: an entry is pair-i side
// exactly when its face lies in the cell's own range (pair-i was written from the
// ranges), so one gather per entry gives the other cell -- pair-j of an own face, pair-i
// of another -- and only own faces to a ghost look up the twin table (the table built
// from the ranges holds twins of such faces only).  The codes equal emit_list_codes'
// (the PHD_PREP_LISTS kernel) on any hand-over whose ranges tile the face list.
__device__ __forceinline__ void range_list_codes(const phd_mesh &M, int c, int f0, int f1,
                                                 const int32_t *__restrict__ twin, const int32_t *src, int e0,
                                                 int e1, int32_t *code_out, int32_t *nbr_out) {
    const int n = M.n_cells, nr = M.n_real, F = M.n_faces;
    constexpr int CH = 4;
    for (int eb = e0; eb < e1; eb += CH) {
        int fid[CH], o[CH];
#pragma unroll
        for (int k = 0; k < CH; k++) fid[k] = src[(eb + k < e1) ? eb + k : e0];
#pragma unroll
        for (int k = 0; k < CH; k++) {
            const bool ok = fid[k] >= 0 && fid[k] < F;
            const bool own = fid[k] >= f0 && fid[k] < f1;
            o[k] = ok ? (own ? M.pair_j[fid[k]] : M.pair_i[fid[k]]) : -1;
        }
#pragma unroll
        for (int k = 0; k < CH; k++) {
            const int e = eb + k;
            if (e >= e1) break;
            if (fid[k] < 0 || fid[k] >= F) { code_out[e] = 0; nbr_out[e] = c; continue; }
            const bool own = fid[k] >= f0 && fid[k] < f1;
            int other = o[k];
            int code = own ? fid[k] : ~fid[k];
            if (own && other >= nr && twin) {
                const int t = twin[fid[k]];
                if (t >= 0 && t < F) {          // this face is dropped: use the twin from the j side
                    code = ~t;
                    other = M.pair_i[t];
                }
            }
            if (other < 0 || other >= n) other = c;
            code_out[e] = code;
            nbr_out[e] = other;
        }
    }
}

// k_csr_sort followed by the FP32 list codes (range_list_codes), one pass.  Each warp
// takes 32 consecutive cells, whose lists are one contiguous span of entries: the span
// is loaded into shared memory with coalesced loads, each thread sorts and codes its
// own cell's list there, and the sorted ids and codes go back with coalesced stores.
// A span longer than SC_CAP entries (cells with unusually many faces) is done by each
// thread in global memory instead.
constexpr int SC_WARPS = UBLOCK / 32, SC_CAP = 320;

// cursor (with list lengths from the host): each list's pair-j entries as scattered,
// checked against its length less its own range (a mismatch adds to *bad).
__global__ void __launch_bounds__(UBLOCK) k_csr_sort_codes_ranges(phd_mesh M, const int32_t *__restrict__ face_ptr,
                                                                  const int32_t *__restrict__ twin, int32_t *idx,
                                                                  int32_t *__restrict__ csr_face,
                                                                  int32_t *__restrict__ csr_nbr,
                                                                  const int32_t *__restrict__ cursor,
                                                                  int32_t *__restrict__ bad) {
    __shared__ int32_t s_idx[SC_WARPS][SC_CAP], s_code[SC_WARPS][SC_CAP], s_nbr[SC_WARPS][SC_CAP];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int n = M.n_cells, nr = M.n_real;
    const int c0 = blockIdx.x * blockDim.x + w * 32;
    if (c0 >= n) return;                                      // the whole warp
    const int c = c0 + lane;
    const bool live = c < n;
    const int e0 = live ? M.nbr_ptr[c] : 0, e1 = live ? M.nbr_ptr[c + 1] : 0;
    const int f0 = (live && c < nr) ? face_ptr[c] : 0, f1 = (live && c < nr) ? face_ptr[c + 1] : 0;
    if (cursor && live && cursor[c] != (e1 - e0) - (f1 - f0)) atomicAdd(bad, 1);
    const int last = min(31, n - 1 - c0);
    const int E0 = __shfl_sync(0xffffffffu, e0, 0), E1 = __shfl_sync(0xffffffffu, e1, last);
    const bool fits = !live || (e0 >= E0 && e0 <= e1 && e1 <= E1);
    if (!__all_sync(0xffffffffu, fits) || E1 - E0 > SC_CAP) {
        if (live) {
            sort_list(idx, e0, e1);
            range_list_codes(M, c, f0, f1, twin, idx, e0, e1, csr_face, csr_nbr);
        }
        return;
    }
    const int span = E1 - E0;
    for (int k = lane; k < span; k += 32) s_idx[w][k] = idx[E0 + k];
    __syncwarp();
    if (live) {
        sort_list(&s_idx[w][0], e0 - E0, e1 - E0);
        range_list_codes(M, c, f0, f1, twin, &s_idx[w][0], e0 - E0, e1 - E0, &s_code[w][0], &s_nbr[w][0]);
    }
    __syncwarp();
    for (int k = lane; k < span; k += 32) {
        idx[E0 + k] = s_idx[w][k];
        csr_face[E0 + k] = s_code[w][k];
        csr_nbr[E0 + k] = s_nbr[w][k];
    }
}

// rint(d / L) for the offsets of periodic images (|d| < 1.5 L), by comparison
__device__ __forceinline__ int shift_of(double d, double L) {
    const double h = 0.5 * L;
    return d > h ? 1 : (d < -h ? -1 : 0);
}

__global__ void k_periodic_twins(phd_mesh M, int periodic, double Lx, double Ly, int32_t *__restrict__ twin) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= M.n_faces) return;
    const int n = M.n_cells, nr = M.n_real;
    int32_t out = -1;
    const int i = M.pair_i[a], g = M.pair_j[a];
    if (periodic && i >= 0 && i < nr && g >= nr && g < n) {
        const int k = M.map[g];
        if (k >= 0 && k < nr && k != i) {
            const int sx = shift_of(M.x[g] - M.x[k], Lx);
            const int sy = shift_of(M.x[(size_t)n + g] - M.x[(size_t)n + k], Ly);
            for (int e = M.nbr_ptr[k]; e < M.nbr_ptr[k + 1]; e++) {
                const int b = M.nbr_idx[e];
                if (b < 0 || b >= M.n_faces || b == a || M.pair_i[b] != k) continue;
                const int g2 = M.pair_j[b];
                if (g2 < nr || g2 >= n || M.map[g2] != i) continue;
                const int tx = shift_of(M.x[g2] - M.x[i], Lx);
                const int ty = shift_of(M.x[(size_t)n + g2] - M.x[(size_t)n + i], Ly);
                if (tx == -sx && ty == -sy) {
                    if (b < a) out = b;
                    break;
                }
            }
        }
    }
    twin[a] = out;
}


// k_periodic_twins for a hand-over whose faces come in per-real-cell ranges: the
// candidates of image cell k are its own faces [face_ptr[k], face_ptr[k+1]) -- in
// ascending order, as they stand in k's sorted neighbour list, so the table is the same
// -- and the neighbour lists are not needed.
__global__ void k_periodic_twins_ranges(phd_mesh M, const int32_t *__restrict__ face_ptr, double Lx, double Ly,
                                        int32_t *__restrict__ twin) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= M.n_faces) return;
    const int n = M.n_cells, nr = M.n_real, F = M.n_faces;
    int32_t out = -1;
    const int i = M.pair_i[a], g = M.pair_j[a];
    if (i >= 0 && i < nr && g >= nr && g < n) {
        const int k = M.map[g];
        if (k >= 0 && k < nr && k != i) {
            const int sx = shift_of(M.x[g] - M.x[k], Lx);
            const int sy = shift_of(M.x[(size_t)n + g] - M.x[(size_t)n + k], Ly);
            const int b0 = max(face_ptr[k], 0), b1 = min(face_ptr[k + 1], F);
            for (int b = b0; b < b1; b++) {
                if (b == a || M.pair_i[b] != k) continue;
                const int g2 = M.pair_j[b];
                if (g2 < nr || g2 >= n || M.map[g2] != i) continue;
                const int tx = shift_of(M.x[g2] - M.x[i], Lx);
                const int ty = shift_of(M.x[(size_t)n + g2] - M.x[(size_t)n + i], Ly);
                if (tx == -sx && ty == -sy) {
                    if (b < a) out = b;
                    break;
                }
            }
        }
    }
    twin[a] = out;
}

// DomainManager.move_generators (domain_manager.pyx:566-590) and the boundary
// conditions' migrate_particles (boundary.pyx:236-263 reflective, 502-538 periodic) for
// the real cells, after a step, with the step's own dt (clk->dt_last).  The product and
// the sum are rounded separately (no contraction), as in the reference.
__global__ void k_move_generators(int n_real, int n, const double *__restrict__ x, const float2 *__restrict__ w2,
                                  const double *__restrict__ w, const phd_clock *clk, int periodic, double lo0,
                                  double lo1, double hi0, double hi1, double *__restrict__ x_out, int *status) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n_real) return;
    const double dt = clk->dt_last;
    double wx, wy;
    if (w2) {
        const float2 v = w2[i];
        wx = v.x;
        wy = v.y;
    } else {
        wx = w[i];
        wy = w[(size_t)n + i];
    }
    double xs[2] = {__dadd_rn(x[i], __dmul_rn(dt, wx)), __dadd_rn(x[(size_t)n + i], __dmul_rn(dt, wy))};
    const double lo[2] = {lo0, lo1}, hi[2] = {hi0, hi1};
    const bool inside = !(xs[0] < lo[0] || xs[0] > hi[0] || xs[1] < lo[1] || xs[1] > hi[1]);   // intersect_bounds
    double xo[2] = {xs[0], xs[1]};
    if (!inside) {
        if (periodic) {
            for (int k = 0; k < 2; k++) {
                const double L = __dsub_rn(hi[k], lo[k]);            // domain_manager.translate
                if (xs[k] <= lo[k]) xo[k] = __dadd_rn(xo[k], L);
                if (xs[k] >= hi[k]) xo[k] = __dsub_rn(xo[k], L);
            }
        } else {
            atomicOr(status, PHD_STATUS_LEFT_DOMAIN);
        }
    }
    x_out[i] = xo[0];
    x_out[(size_t)n_real + i] = xo[1];
}


// Ghost positions from the real cells' (domain_manager.pyx:712-774 ghost copies;
// boundary.pyx:66-130 mirror images, 351-400 periodic copies), with the host
// tessellation's arithmetic: x + s L for a periodic copy, x - 2 (x - wall) across a
// mirror.  code (per ghost): 1 + 3 (sx + 1) + (sy + 1) periodic, 16 + 2 k + h mirror.
// Rows of x: the real rows copied from src (rows of stride src_stride) when copy_real,
// and every ghost row from its image's row of src by its code.  src may be x itself
// (stride n, copy_real = 0).
__global__ void k_positions(int n_real, int n, int copy_real, const int32_t *__restrict__ map,
                            const int8_t *__restrict__ code, double lo0, double lo1, double hi0, double hi1,
                            const double *src, size_t src_stride, double *x, int *bad) {
    const int g = (copy_real ? 0 : n_real) + blockIdx.x * blockDim.x + threadIdx.x;
    if (g >= n) return;
    if (g < n_real) {
        x[g] = src[g];
        x[(size_t)n + g] = src[src_stride + g];
        return;
    }
    const int img = map[g];
    const int c = code[g - n_real];
    if (img < 0 || img >= n_real) { atomicAdd(bad, 1); return; }
    double px = src[img], py = src[src_stride + img];
    if (c >= 1 && c <= 9 && c != 5) {
        const int sx = (c - 1) / 3 - 1, sy = (c - 1) % 3 - 1;
        px = __dadd_rn(px, __dmul_rn(double(sx), __dsub_rn(hi0, lo0)));
        py = __dadd_rn(py, __dmul_rn(double(sy), __dsub_rn(hi1, lo1)));
    } else if (c >= 16 && c <= 19) {
        const int k = (c - 16) >> 1, high = (c - 16) & 1;
        if (k == 0) {
            const double wall = high ? hi0 : lo0;
            px = __dsub_rn(px, __dmul_rn(2.0, __dsub_rn(px, wall)));
        } else {
            const double wall = high ? hi1 : lo1;
            py = __dsub_rn(py, __dmul_rn(2.0, __dsub_rn(py, wall)));
        }
    } else {
        atomicAdd(bad, 1);
        return;
    }
    x[g] = px;
    x[(size_t)n + g] = py;
}

// Neighbour lists of a hand-over whose faces come grouped by pair-i in per-real-cell
// ranges [face_ptr[c], face_ptr[c+1]) (the compact format): pair-i is written from the
// ranges, a cell's count is its own range plus the faces naming it as pair-j, and its
// own range goes to the tail of its list without atomics; the pair-j side is scattered
// with a cursor, and k_csr_sort orders every list.  A broken range (face_ptr not
// starting at 0, decreasing, or not ending at n_faces) and faces with out-of-range or
// equal cells add to *bad, as phd_pair_i_from_face_ptr and phd_build_csr count them.
__device__ __forceinline__ bool range_ok(int c, int n_real, int F, int a, int b) {
    return !(a < 0 || b < a || b > F || (c == 0 && a != 0) || (c == n_real - 1 && b != F));
}

// Host-to-device copies issued in order, each merged into the one before when both its
// source and its destination continue that copy's exactly.
struct CopyRun {
    static constexpr int N = 8;
    void *dst[N];
    const void *src[N];
    size_t bytes[N];
    int k = 0;
    cudaError_t err = cudaSuccess;
    void add(void *d, const void *s, size_t b) {
        if (b == 0) return;
        if (k > 0 && static_cast<const char *>(src[k - 1]) + bytes[k - 1] == s &&
            static_cast<char *>(dst[k - 1]) + bytes[k - 1] == d) {
            bytes[k - 1] += b;
            return;
        }
        if (k == N) {
            err = cudaErrorInvalidValue;
            return;
        }
        dst[k] = d;
        src[k] = s;
        bytes[k] = b;
        k++;
    }
    cudaError_t issue(cudaStream_t stream) {
        cudaError_t e = err;
        for (int q = 0; q < k && e == cudaSuccess; q++)
            e = cudaMemcpyAsync(dst[q], src[q], bytes[q], cudaMemcpyHostToDevice, stream);
        k = 0;
        err = cudaSuccess;
        return e;
    }
};

// The escaped faces of a packed pair-j hand-over: pair_j[fid] from the (face id, pair-j)
// list px[K], and the face's packed entry (the device staging copy) turned from
// PHD_PAIR16_ESCAPE into PAIR16_LISTED, so k_faces_from_ranges can tell a listed face
// from one marked escaped but missing from the list (an error).  A listed face that is
// not marked escaped, or out of range, adds to *bad.
constexpr uint16_t PAIR16_LISTED = 0xffff;

__global__ void k_pair_escapes(int K, int F, const int32_t *__restrict__ px, uint16_t *__restrict__ dj,
                               int32_t *__restrict__ pair_j, int32_t *__restrict__ bad) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= K) return;
    const int fid = px[2 * k];
    if (fid < 0 || fid >= F || (dj[fid] != PHD_PAIR16_ESCAPE && dj[fid] != PAIR16_LISTED)) {
        atomicAdd(bad, 1);
        return;
    }
    pair_j[fid] = px[2 * k + 1];
    dj[fid] = PAIR16_LISTED;
}

// pair-i (and pair-j, when packed) of every face from the per-real-cell face ranges,
// one thread per face: a block takes UBLOCK consecutive real cells, stages their range
// bounds in shared memory, and each thread finds its face's owner there by bisection,
// so every face array is read and written coalesced.  dj (optional): pair-j packed as
// the difference to the owner (PAIR16_LISTED: k_pair_escapes has written it;
// PHD_PAIR16_ESCAPE: escaped but not listed, an error).  COUNT: the list lengths counted
// with atomics into cnt; otherwise they came from the host.  A block holding a broken
// range (face_ptr not starting at 0, decreasing, or not ending at n_faces) adds 1 to
// *bad per broken cell and writes nothing; faces with out-of-range or equal cells add 1.
template <bool COUNT>
__global__ void __launch_bounds__(UBLOCK) k_faces_from_ranges(int n_real, int n, int F,
                                                              const int32_t *__restrict__ face_ptr,
                                                              int32_t *__restrict__ pair_j, const uint16_t *dj,
                                                              int32_t *__restrict__ pair_i,
                                                              int32_t *__restrict__ cnt, int32_t *__restrict__ bad) {
    __shared__ int32_t s_fp[UBLOCK + 1];
    __shared__ int s_broken;
    const int c0 = blockIdx.x * UBLOCK;
    const int nc = min(UBLOCK, n_real - c0);
    if (nc <= 0) return;
    if (threadIdx.x == 0) s_broken = 0;
    for (int k = threadIdx.x; k <= nc; k += blockDim.x) s_fp[k] = face_ptr[c0 + k];
    __syncthreads();
    if (threadIdx.x < nc && !range_ok(c0 + threadIdx.x, n_real, F, s_fp[threadIdx.x], s_fp[threadIdx.x + 1])) {
        atomicAdd(bad, 1);
        s_broken = 1;
    }
    __syncthreads();
    if (s_broken) return;
    const int m1 = s_fp[nc];
    for (int m = s_fp[0] + threadIdx.x; m < m1; m += blockDim.x) {
        int lo = 0, hi = nc;                       // s_fp[lo] <= m < s_fp[hi]
        while (hi - lo > 1) {
            const int mid = (lo + hi) >> 1;
            if (s_fp[mid] <= m)
                lo = mid;
            else
                hi = mid;
        }
        const int c = c0 + lo;
        pair_i[m] = c;
        int j;
        const int d = dj ? dj[m] : PAIR16_LISTED;
        if (d == PAIR16_LISTED) {
            j = pair_j[m];
        } else {
            j = d != PHD_PAIR16_ESCAPE ? c + d : -1;
            pair_j[m] = j;
        }
        if (j >= 0 && j < n && j != c) {
            if (COUNT) {
                atomicAdd(&cnt[j], 1);
                atomicAdd(&cnt[c], 1);
            }
        } else {
            atomicAdd(bad, 1);
        }
    }
}

// The faces into the neighbour lists, one thread per face: the owner's entry at the
// tail of its list in face order (its own range, so the list ends with it sorted), the
// other cell's through its cursor.  Faces with bad cells (counted by
// k_faces_from_ranges) are skipped.  Every write lands inside idx[0, cap): with list
// lengths from the host, a face set that does not match them adds to *bad here (a
// write outside) or in the sort (a list not filled exactly), and never writes out of
// bounds.
__global__ void k_csr_scatter_faces(int n_real, int n, int F, const int32_t *__restrict__ face_ptr,
                                    const int32_t *__restrict__ pair_i, const int32_t *__restrict__ pair_j,
                                    const int32_t *__restrict__ ptr, int32_t *__restrict__ cursor,
                                    int32_t *__restrict__ idx, int cap, int32_t *__restrict__ bad) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= F) return;
    const int i = pair_i[m], j = pair_j[m];
    if (i < 0 || i >= n_real || j < 0 || j >= n || j == i) return;
    const int own = ptr[i + 1] - (face_ptr[i + 1] - m);
    const int q = ptr[j] + atomicAdd(&cursor[j], 1);
    if (own >= 0 && own < cap && q >= 0 && q < cap) {
        idx[own] = m;
        idx[q] = m;
    } else {
        atomicAdd(bad, 1);
    }
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


int phd_face_normals_f64(const phd_mesh *mesh, double *normal, int32_t *bad, cudaStream_t stream) {
    if (!mesh || mesh->dim != 2 || mesh->n_cells < 0 || mesh->n_faces < 0 || !normal) return PHD_ERR_ARG;
    if (mesh->n_faces && (!mesh->pair_i || !mesh->pair_j || !mesh->x)) return PHD_ERR_ARG;
    if (!mesh->n_faces) return PHD_OK;
    phd::k_face_normals<<<(mesh->n_faces + phd::UBLOCK - 1) / phd::UBLOCK, phd::UBLOCK, 0, stream>>>(
        mesh->n_cells, mesh->n_faces, mesh->pair_i, mesh->pair_j, mesh->x, normal, bad);
    return cudaPeekAtLastError() == cudaSuccess ? PHD_OK : PHD_ERR_LAUNCH;
}

size_t phd_csr_work_ints(int32_t n_cells) {
    const size_t n = n_cells > 0 ? (size_t)n_cells : 0;
    return 2 * n + (n + phd::SCAN_TILE - 1) / phd::SCAN_TILE;
}

int phd_build_csr(const phd_mesh *mesh, int32_t *nbr_ptr, int32_t *nbr_idx, int32_t *work, int32_t *bad,
                  cudaStream_t stream) {
    phd::NvtxRange nvtx_range("phd_build_csr");
    if (!mesh || mesh->n_cells <= 0 || mesh->n_faces < 0 || !nbr_ptr || !work) return PHD_ERR_ARG;
    if (mesh->n_faces && (!mesh->pair_i || !mesh->pair_j || !nbr_idx)) return PHD_ERR_ARG;
    const int n = mesh->n_cells, F = mesh->n_faces;
    const int n_tiles = (n + phd::SCAN_TILE - 1) / phd::SCAN_TILE;
    int32_t *cnt = work, *cursor = work + n, *tile_sum = work + 2 * (size_t)n;
    cudaMemsetAsync(work, 0, sizeof(int32_t) * phd_csr_work_ints(n), stream);
    const int gf = F ? (F + phd::UBLOCK - 1) / phd::UBLOCK : 1;
    if (F) phd::k_csr_count<<<gf, phd::UBLOCK, 0, stream>>>(n, F, mesh->pair_i, mesh->pair_j, cnt, bad);
    phd::k_scan_tiles<<<n_tiles, phd::SCAN_THREADS, 0, stream>>>(n, cnt, tile_sum);
    phd::k_scan_tile_sums<<<1, phd::SCAN_THREADS, 0, stream>>>(n_tiles, tile_sum);
    phd::k_scan_offsets<<<n_tiles, phd::SCAN_THREADS, 0, stream>>>(n, cnt, tile_sum, nbr_ptr, INT32_MAX);
    if (F) {
        phd::k_csr_scatter<<<gf, phd::UBLOCK, 0, stream>>>(n, F, mesh->pair_i, mesh->pair_j, nbr_ptr, cursor,
                                                            nbr_idx);
        phd::k_csr_sort<<<(n + phd::UBLOCK - 1) / phd::UBLOCK, phd::UBLOCK, 0, stream>>>(n, nbr_ptr, nbr_idx);
    }
    return cudaPeekAtLastError() == cudaSuccess ? PHD_OK : PHD_ERR_LAUNCH;
}

int phd_periodic_twins(const phd_mesh *mesh, int32_t periodic, double box_x, double box_y, int32_t *twin,
                       cudaStream_t stream) {
    if (!mesh || mesh->dim != 2 || mesh->n_cells <= 0 || mesh->n_faces < 0 || !twin) return PHD_ERR_ARG;
    if (periodic && (!(box_x > 0.0) || !(box_y > 0.0))) return PHD_ERR_ARG;
    if (!mesh->n_faces) return PHD_OK;
    if (!mesh->pair_i || !mesh->pair_j || !mesh->map || !mesh->x || !mesh->nbr_ptr || !mesh->nbr_idx)
        return PHD_ERR_ARG;
    phd::k_periodic_twins<<<(mesh->n_faces + phd::UBLOCK - 1) / phd::UBLOCK, phd::UBLOCK, 0, stream>>>(
        *mesh, periodic != 0, box_x, box_y, twin);
    return cudaPeekAtLastError() == cudaSuccess ? PHD_OK : PHD_ERR_LAUNCH;
}

int phd_move_generators(const phd_mesh *mesh, const float *w2, const double *w, phd_clock *clk, int32_t periodic,
                        double xmin0, double xmin1, double xmax0, double xmax1, double *x_out, cudaStream_t stream) {
    phd::NvtxRange nvtx_range("phd_move_generators");
    if (!mesh || mesh->dim != 2 || !mesh->x || !clk || !x_out || (!w2) == (!w) || mesh->n_real < 0 ||
        mesh->n_real > mesh->n_cells || !(xmax0 > xmin0) || !(xmax1 > xmin1))
        return PHD_ERR_ARG;
    if (mesh->n_real == 0) return PHD_OK;
    phd::k_move_generators<<<(mesh->n_real + phd::UBLOCK - 1) / phd::UBLOCK, phd::UBLOCK, 0, stream>>>(
        mesh->n_real, mesh->n_cells, mesh->x, reinterpret_cast<const float2 *>(w2), w, clk, periodic, xmin0, xmin1,
        xmax0, xmax1, x_out, &clk->status);
    return cudaPeekAtLastError() == cudaSuccess ? PHD_OK : PHD_ERR_LAUNCH;
}


int phd_ghost_positions(const phd_mesh *mesh, const int8_t *ghost_code, double xmin0, double xmin1, double xmax0,
                        double xmax1, int32_t *bad, cudaStream_t stream) {
    phd::NvtxRange nvtx_range("phd_ghost_positions");
    if (!mesh || mesh->dim != 2 || !mesh->x || !mesh->map || !bad || mesh->n_real < 0 ||
        mesh->n_real > mesh->n_cells || !(xmax0 > xmin0) || !(xmax1 > xmin1))
        return PHD_ERR_ARG;
    const int ng = mesh->n_cells - mesh->n_real;
    if (ng == 0) return PHD_OK;
    if (!ghost_code) return PHD_ERR_ARG;
    phd::k_positions<<<(ng + phd::UBLOCK - 1) / phd::UBLOCK, phd::UBLOCK, 0, stream>>>(
        mesh->n_real, mesh->n_cells, 0, mesh->map, ghost_code, xmin0, xmin1, xmax0, xmax1, mesh->x,
        (size_t)mesh->n_cells, const_cast<double *>(mesh->x), bad);
    return cudaPeekAtLastError() == cudaSuccess ? PHD_OK : PHD_ERR_LAUNCH;
}


int phd_load_mesh_f32(const phd_mesh *mesh, const phd_handover32 *h, const phd_params *par, phd_geom32_out *out,
                      double *cons, float *prim4, phd_clock *clk, cudaStream_t stream, const cudaStream_t *side,
                      cudaEvent_t *events) {
    phd::NvtxRange nvtx_range("phd_load_mesh_f32");
    if (!mesh || !h || !par || !out || !cons || !prim4 || !clk || !side || !events || mesh->dim != 2 ||
        mesh->normal || mesh->n_cells <= 0 || mesh->n_real < 0 || mesh->n_real > mesh->n_cells ||
        mesh->n_faces < 0)
        return PHD_ERR_ARG;
    if (!mesh->pair_i || !mesh->pair_j || !mesh->map || !mesh->x || !mesh->flip || !mesh->nbr_ptr || !mesh->nbr_idx)
        return PHD_ERR_ARG;
    const bool interleaved = h->face32 != nullptr;    // one (area, offset) array
    if (!h->face_ptr || !h->d_face_ptr || (interleaved ? !h->d_face32 : (!h->area32 || !h->ct32 || !h->d_area32 ||
                                                                          !h->d_ct32)) ||
        !h->type || !h->twin || !h->csr_work || !h->bad || !(h->xmax[0] > h->xmin[0]) || !(h->xmax[1] > h->xmin[1]))
        return PHD_ERR_ARG;
    const int n = mesh->n_cells, nr = mesh->n_real, F = mesh->n_faces, ng = n - nr;
    if (!out->csr_face || !out->csr_nbr) return PHD_ERR_ARG;
    const bool packed = h->pair_j == nullptr;      // pair-j as 16-bit differences + escapes
    if (packed && (!h->pair_dj || !h->d_pair_dj || h->n_pair_x < 0 || h->n_pair_x > F ||
                   (h->n_pair_x > 0 && (!h->pair_x || !h->d_pair_x))))
        return PHD_ERR_ARG;
    if (!h->x && ng > 0 && (!h->ghost_code || !h->d_ghost_code)) return PHD_ERR_ARG;
    const bool host_len = h->list_len != nullptr;  // list lengths from the host: no atomic count
    if (host_len && !h->d_list_len) return PHD_ERR_ARG;
    int32_t *pair_i = const_cast<int32_t *>(mesh->pair_i);
    int32_t *pair_j = const_cast<int32_t *>(mesh->pair_j);
    double *x = const_cast<double *>(mesh->x);
    const cudaStream_t lists = side[0], geom = side[1];
    int rc = PHD_OK;
#define PHD_TRY(call)                                                      \
    do {                                                                   \
        if ((rc = (call)) != PHD_OK) return rc;                            \
    } while (0)
#define PHD_TRY_CUDA(call)                                                 \
    do {                                                                   \
        if ((call) != cudaSuccess) return PHD_ERR_LAUNCH;                  \
    } while (0)
    // stream: the face ranges, pair-j, the list lengths and ghost codes, then the ghost
    // map (and positions), then the large FP32 face records; each group's event releases
    // the work that needs it.  Arrays adjacent both on the host and in the staging are
    // copied as one (each copy costs a few microseconds on top of its bytes).
    PHD_TRY_CUDA(cudaMemsetAsync(h->bad, 0, sizeof(int32_t), stream));
    phd::CopyRun run;
    if (packed && h->n_pair_x > 0) run.add(h->d_pair_x, h->pair_x, (size_t)2 * h->n_pair_x * sizeof(int32_t));
    run.add(h->d_face_ptr, h->face_ptr, (size_t)(nr + 1) * sizeof(int32_t));
    if (!packed)
        run.add(pair_j, h->pair_j, (size_t)F * sizeof(int32_t));
    else
        run.add(h->d_pair_dj, h->pair_dj, (size_t)F * sizeof(uint16_t));
    if (host_len) run.add(h->d_list_len, h->list_len, (size_t)n);
    if (!h->x && ng > 0) run.add(h->d_ghost_code, h->ghost_code, (size_t)ng);
    PHD_TRY_CUDA(run.issue(stream));
    PHD_TRY_CUDA(cudaEventRecord(events[0], stream));
    if (h->ghost_map && ng > 0)
        run.add(const_cast<int32_t *>(mesh->map) + nr, h->ghost_map, (size_t)ng * sizeof(int32_t));
    if (h->x) run.add(x, h->x, (size_t)2 * n * sizeof(double));
    PHD_TRY_CUDA(run.issue(stream));
    PHD_TRY_CUDA(cudaEventRecord(events[1], stream));
    // the face records in two parts, three quarters and the rest: the first part's
    // geometry is formed while the rest is in flight, so only a quarter of it is left
    // once the copies end
    const int F0 = (int)(((int64_t)F * 3) / 4);
    if (interleaved) {
        run.add(h->d_face32, h->face32, (size_t)2 * F0 * sizeof(float));
    } else {
        run.add(h->d_area32, h->area32, (size_t)F0 * sizeof(float));
        run.add(h->d_ct32, h->ct32, (size_t)F0 * sizeof(float));
    }
    PHD_TRY_CUDA(run.issue(stream));
    PHD_TRY_CUDA(cudaEventRecord(events[7], stream));
    if (interleaved) {
        run.add(h->d_face32 + 2 * (size_t)F0, h->face32 + 2 * (size_t)F0, (size_t)2 * (F - F0) * sizeof(float));
    } else {
        run.add(h->d_area32 + F0, h->area32 + F0, (size_t)(F - F0) * sizeof(float));
        run.add(h->d_ct32 + F0, h->ct32 + F0, (size_t)(F - F0) * sizeof(float));
    }
    PHD_TRY_CUDA(run.issue(stream));
    PHD_TRY_CUDA(cudaEventRecord(events[2], stream));

    // lists stream, while the face records are in flight: pair-i with the list counts,
    // every position, the neighbour lists
    const int32_t *nbr_ptr = mesh->nbr_ptr;
    int32_t *cnt = h->csr_work, *cursor = h->csr_work + n, *tile_sum = h->csr_work + 2 * (size_t)n;
    const int n_tiles = (n + phd::SCAN_TILE - 1) / phd::SCAN_TILE;
    const int gr = nr > 0 ? (nr + phd::UBLOCK - 1) / phd::UBLOCK : 1;
    PHD_TRY_CUDA(cudaStreamWaitEvent(lists, events[0], 0));
    if (host_len)                                      // the cursors only
        PHD_TRY_CUDA(cudaMemsetAsync(cursor, 0, sizeof(int32_t) * (size_t)n, lists));
    else
        PHD_TRY_CUDA(cudaMemsetAsync(h->csr_work, 0, sizeof(int32_t) * phd_csr_work_ints(n), lists));
    if (packed && h->n_pair_x > 0)        // the escaped faces first
        phd::k_pair_escapes<<<(h->n_pair_x + phd::UBLOCK - 1) / phd::UBLOCK, phd::UBLOCK, 0, lists>>>(
            h->n_pair_x, F, h->d_pair_x, h->d_pair_dj, pair_j, h->bad);
    if (nr > 0) {
        const uint16_t *dj = packed ? h->d_pair_dj : nullptr;
        if (host_len)
            phd::k_faces_from_ranges<false><<<gr, phd::UBLOCK, 0, lists>>>(nr, n, F, h->d_face_ptr, pair_j, dj,
                                                                           pair_i, cnt, h->bad);
        else
            phd::k_faces_from_ranges<true><<<gr, phd::UBLOCK, 0, lists>>>(nr, n, F, h->d_face_ptr, pair_j, dj,
                                                                          pair_i, cnt, h->bad);
    }
    PHD_TRY_CUDA(cudaEventRecord(events[3], lists));
    if (host_len) {
        phd::k_scan_tiles<<<n_tiles, phd::SCAN_THREADS, 0, lists>>>(n, h->d_list_len, tile_sum);
        phd::k_scan_tile_sums<<<1, phd::SCAN_THREADS, 0, lists>>>(n_tiles, tile_sum);
        phd::k_scan_offsets<<<n_tiles, phd::SCAN_THREADS, 0, lists>>>(n, h->d_list_len, tile_sum,
                                                                      const_cast<int32_t *>(nbr_ptr), 2 * F);
    } else {
        phd::k_scan_tiles<<<n_tiles, phd::SCAN_THREADS, 0, lists>>>(n, cnt, tile_sum);
        phd::k_scan_tile_sums<<<1, phd::SCAN_THREADS, 0, lists>>>(n_tiles, tile_sum);
        phd::k_scan_offsets<<<n_tiles, phd::SCAN_THREADS, 0, lists>>>(n, cnt, tile_sum,
                                                                      const_cast<int32_t *>(nbr_ptr), INT32_MAX);
    }
    if (nr > 0 && F > 0) {
        phd::k_csr_scatter_faces<<<(F + phd::UBLOCK - 1) / phd::UBLOCK, phd::UBLOCK, 0, lists>>>(
            nr, n, F, h->d_face_ptr, pair_i, pair_j, nbr_ptr, cursor, const_cast<int32_t *>(mesh->nbr_idx), 2 * F,
            h->bad);
    }
    PHD_TRY_CUDA(cudaPeekAtLastError());

    // geometry stream, beside the lists: the flip bits and periodic twins once the
    // positions are there, the FP32 face geometry once the face records are too
    const double lo[3] = {h->xmin[0], h->xmin[1], 0.}, hi[3] = {h->xmax[0], h->xmax[1], 0.};
    // every position first (the ghosts' from their codes), beside the list counts
    PHD_TRY_CUDA(cudaStreamWaitEvent(geom, events[1], 0));
    if (!h->x && n > 0) {
        const bool copy_real = h->x_real != nullptr;
        const int first = copy_real ? 0 : nr;
        if (n > first)
            phd::k_positions<<<(n - first + phd::UBLOCK - 1) / phd::UBLOCK, phd::UBLOCK, 0, geom>>>(
                nr, n, copy_real, mesh->map, h->d_ghost_code, h->xmin[0], h->xmin[1], h->xmax[0], h->xmax[1],
                copy_real ? h->x_real : x, copy_real ? (size_t)nr : (size_t)n, x, h->bad);
    }
    PHD_TRY(phd_flip_mask(2, n, h->type, x, lo, hi, !h->periodic, const_cast<int8_t *>(mesh->flip), geom));
    PHD_TRY_CUDA(cudaStreamWaitEvent(geom, events[3], 0));      // pair-i and pair-j
    if (F > 0) {
        if (h->periodic && h->dedup_periodic)
            phd::k_periodic_twins_ranges<<<(F + phd::UBLOCK - 1) / phd::UBLOCK, phd::UBLOCK, 0, geom>>>(
                *mesh, h->d_face_ptr, h->xmax[0] - h->xmin[0], h->xmax[1] - h->xmin[1], h->twin);
        else
            PHD_TRY_CUDA(cudaMemsetAsync(h->twin, 0xff, (size_t)F * sizeof(int32_t), geom));
    }
    PHD_TRY_CUDA(cudaEventRecord(events[6], geom));
    for (int half = 0; half < 2; half++) {        // faces [0, F0), then [F0, F)
        const int m0 = half ? F0 : 0, cnt = half ? F - F0 : F0;
        phd_mesh part = *mesh;
        part.pair_i += m0;
        part.pair_j += m0;
        part.n_faces = cnt;
        phd_geom32_out po = *out;
        po.face_geo += 4 * (size_t)m0;
        po.face_ar += 2 * (size_t)m0;
        PHD_TRY_CUDA(cudaStreamWaitEvent(geom, events[half ? 2 : 7], 0));
        if (cnt > 0 && interleaved)
            PHD_TRY(phd::prepare_faces32_interleaved(&part, h->d_face32 + 2 * (size_t)m0, &po, geom));
        else if (cnt > 0)
            PHD_TRY(phd_prepare_f32_faces_compact(&part, h->d_area32 + m0, h->d_ct32 + m0, &po, geom));
    }
    PHD_TRY_CUDA(cudaEventRecord(events[4], geom));

    // lists stream, once the twins are there: each list sorted and its FP32 codes formed
    // in one pass (k_csr_sort + PHD_PREP_LISTS)
    PHD_TRY_CUDA(cudaStreamWaitEvent(lists, events[6], 0));
    if (n > 0)
        phd::k_csr_sort_codes_ranges<<<(n + phd::UBLOCK - 1) / phd::UBLOCK, phd::UBLOCK, 0, lists>>>(
            *mesh, h->d_face_ptr, h->twin, const_cast<int32_t *>(mesh->nbr_idx), out->csr_face, out->csr_nbr,
            host_len ? cursor : nullptr, h->bad);
    PHD_TRY_CUDA(cudaPeekAtLastError());
    PHD_TRY_CUDA(cudaEventRecord(events[5], lists));

    // stream, once the lists and the faces are in: cell geometry, ghost totals from
    // their images, primitives and the next dt in one pass
    PHD_TRY_CUDA(cudaStreamWaitEvent(stream, events[5], 0));
    PHD_TRY_CUDA(cudaStreamWaitEvent(stream, events[4], 0));
    PHD_TRY(phd::cells_prim_f32(mesh, par, out, cons, prim4, clk, stream));
#undef PHD_TRY
#undef PHD_TRY_CUDA
    return PHD_OK;
}

}  // extern "C"
