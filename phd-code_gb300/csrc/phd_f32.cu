// phd_f32.cu -- FP32 reconstruction / Riemann with FP64 conserved-state accumulation.
//
// Precision split: every geometric quantity that would cancel catastrophically in
// FP32 (face centroid minus generator midpoint, generator separation) is formed in
// FP64 once per mesh (k_prepare32) and stored relative; cell primitives and gradients
// are FP32; each face flux is FP32; the per-face conserved increment is formed once in
// FP32 and both cells of the face add exactly that value, so mass, momentum and energy
// are exchanged exactly; the sum over a cell's faces is compensated (two-sum) and added
// to the FP64 conserved totals.  The exact solver keeps its Newton pressure iteration in
// FP64 (phd_physics.cuh).
//
// Layout (device):
//   face_geo  float4 [F]  (n_x, n_y, c_x, c_y)  c = face centroid - (x_i + x_j)/2
//   face_ar   float2 [F]  (area, r = |x_j - x_i|)
//   csr_face  int32 [2F]  face id where the cell is pair-i, ~face id where it is pair-j
//   csr_nbr   int32 [2F]  the other cell of that face
//   entry_rec float4 [2F] per list entry, sigma = +1 (pair-i) / -1 (pair-j):
//                         (w_x, w_y, t_x, t_y), w = (A/r) c + sigma (A/2) n (the
//                         gradient weight), t = c + sigma (r/2) n (face centroid minus
//                         the generator): the gradient kernel reads its geometry in list
//                         order instead of gathering two face records per entry
//   cell_geo  float4 [n]  (dcom_x, dcom_y, 1/vol, R = sqrt(vol/pi))
//   prim4     float4 [n]  (rho, v_x, v_y, p)
//   cellrec   float4 [4n] what the face kernel needs of a cell, 64 B (two 256-bit
//                         loads): prim4 | d/dx, d/dy of rho, v_x | of v_y, p |
//                         (dcom_x, dcom_y, w_x, w_y); written by the gradient kernel
//   w2        float2 [n]  generator velocity (the host re-mesh reads it)
//   flux4     float4 [F]  dt*A*F: the face's conserved increment (mass, mom_x, mom_y, energy)
#include <cmath>
#include <utility>
#include "phd_common.cuh"
#include "phd_physics.cuh"

namespace phd {

constexpr int B32 = 256;

// d > 0.0 for an FP64 value, by one integer comparison of its bits (positive normal,
// subnormal and +inf; not +-0, negatives or NaN): the update kernel's FP64 pipe, at a
// small fraction of the FP32 rate on GB300, then carries only the additions.
__device__ __forceinline__ bool fp64_positive(double d) {
    const long long b = __double_as_longlong(d);
    return b > 0 && b <= 0x7ff0000000000000ll;
}

__device__ __forceinline__ void set_status32(phd_clock *clk, int bits) {
    if (bits) atomicOr(&clk->status, bits);
}

// ---- mesh preparation (once per uploaded mesh) ----------------------------------
// The differences that cancel (x_j - x_i, face centroid minus generator midpoint) are
// taken in FP64 and rounded once to FP32; everything formed from them afterwards
// (separation length, normal when the mesh carries none, 1/V, R) is FP32.  The
// FP64 -> FP32 roundings use integer arithmetic (narrow_f64), off the FP64 pipe.
// Separation length and unit normal from the FP32-rounded separation, with the IEEE
// operations spelled out (fast-math would let each kernel pick its own sqrt /
// reciprocal sequence): every kernel that forms them gets the same bits.
__device__ __forceinline__ void face_normal32(float fx, float fy, float &r, float &nx, float &ny) {
    r = __fsqrt_rn(__fmaf_rn(fx, fx, __fmul_rn(fy, fy)));
    const float inv = r > 0.f ? __frcp_rn(r) : 0.f;
    nx = __fmul_rn(fx, inv);
    ny = __fmul_rn(fy, inv);
}

// The face centroid's offset from the generator midpoint, c = com - (x_i + x_j)/2,
// lies along the face (a Voronoi face is on the perpendicular bisector of x_i x_j), so
// one number carries it: s = c . t, t = (-n_y, n_x), formed in FP64 with every
// rounding spelled out --
//   dx = x_j - x_i, r = sqrt(dx.dx), s = (c_x (-dy) + c_y dx) / r --
// exactly as the host forms it for the compact hand-over, and rounded once to FP32.
// The FP32 offset is then s t with t from the FP32 normal of the rounded separation,
// in both hand-overs, so their FP32 geometry is the same bit for bit.
__device__ __forceinline__ double face_offset_f64(double xi, double yi, double xj, double yj, double comx,
                                                  double comy) {
    const double dx = __dsub_rn(xj, xi), dy = __dsub_rn(yj, yi);
    const double cx = __dsub_rn(comx, __dmul_rn(0.5, __dadd_rn(xi, xj)));
    const double cy = __dsub_rn(comy, __dmul_rn(0.5, __dadd_rn(yi, yj)));
    const double r = __dsqrt_rn(__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)));
    return r > 0.0 ? __ddiv_rn(__dadd_rn(__dmul_rn(cx, -dy), __dmul_rn(cy, dx)), r) : 0.0;
}

__device__ __forceinline__ float2 face_offset32(float s, float nx, float ny) {
    return make_float2(__fmul_rn(s, -ny), __fmul_rn(s, nx));
}

__global__ void k_prepare_faces32(phd_mesh M, float4 *__restrict__ face_geo, float2 *__restrict__ face_ar) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= M.n_faces) return;
    const int n = M.n_cells, F = M.n_faces;
    const int i = M.pair_i[m], j = M.pair_j[m];
    double dx = 0, dy = 0, sc = 0;
    if (i >= 0 && i < n && j >= 0 && j < n) {
        const double xi = M.x[i], yi = M.x[(size_t)n + i], xj = M.x[j], yj = M.x[(size_t)n + j];
        dx = xj - xi;
        dy = yj - yi;
        sc = face_offset_f64(xi, yi, xj, yj, M.com[m], M.com[(size_t)F + m]);
    }
    const float fx = narrow_f64(dx), fy = narrow_f64(dy);
    float r, nx, ny;                // n = (x_j - x_i)/|x_j - x_i| (tess.cpp:367-369)
    face_normal32(fx, fy, r, nx, ny);
    const float2 c = face_offset32(narrow_f64(sc), nx, ny);
    if (M.normal) {
        nx = narrow_f64(M.normal[m]);
        ny = narrow_f64(M.normal[(size_t)F + m]);
    }
    face_geo[m] = make_float4(nx, ny, c.x, c.y);
    face_ar[m] = make_float2(narrow_f64(M.area[m]), r);
}

// The same face geometry from the compact FP32 hand-over: the host rounds the area and
// the centroid offset along the face (face_offset_f64) once to FP32, so the face
// record crosses the link in 12 bytes (pair-j, area, offset) instead of 32;
// separations and normals still come from the FP64 positions.
// stride: 1 for separate area / offset arrays, 2 for one interleaved (area, offset) array
__global__ void k_prepare_faces32_compact(phd_mesh M, const float *__restrict__ area32,
                                          const float *__restrict__ ct32, int stride, float4 *__restrict__ face_geo,
                                          float2 *__restrict__ face_ar) {
    const int m = blockIdx.x * blockDim.x + threadIdx.x;
    if (m >= M.n_faces) return;
    const int n = M.n_cells;
    const int i = M.pair_i[m], j = M.pair_j[m];
    double dx = 0, dy = 0;
    if (i >= 0 && i < n && j >= 0 && j < n) {
        dx = M.x[j] - M.x[i];
        dy = M.x[(size_t)n + j] - M.x[(size_t)n + i];
    }
    const float fx = narrow_f64(dx), fy = narrow_f64(dy);
    float r, nx, ny;
    face_normal32(fx, fy, r, nx, ny);
    const float2 c = face_offset32(ct32[(size_t)m * stride], nx, ny);
    face_geo[m] = make_float4(nx, ny, c.x, c.y);
    face_ar[m] = make_float2(area32[(size_t)m * stride], r);
}

// pair-i of every face from the per-real-cell face ranges (faces are emitted per real
// cell in ascending cell order, tess.cpp:363): face_ptr[0] = 0, face_ptr[n_real] =
// n_faces, non-decreasing -- then the ranges tile the face list exactly; a range that
// breaks this is counted in *bad and left unwritten.
__global__ void k_pair_i_from_ptr(int n_real, int n_faces, const int32_t *__restrict__ face_ptr,
                                  int32_t *__restrict__ pair_i, int32_t *bad) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= n_real) return;
    const int a = face_ptr[c], b = face_ptr[c + 1];
    if (a < 0 || b < a || b > n_faces || (c == 0 && a != 0) || (c == n_real - 1 && b != n_faces)) {
        atomicAdd(bad, 1);
        return;
    }
    for (int m = a; m < b; m++) pair_i[m] = c;
}

__global__ void k_prepare_cells32(phd_mesh M, float4 *__restrict__ cell_geo) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= M.n_cells) return;
    const int n = M.n_cells;
    const float v = narrow_f64(M.vol[i]);
    cell_geo[i] = make_float4(narrow_f64(M.dcom[i]), narrow_f64(M.dcom[(size_t)n + i]), 1.f / v,
                              sqrtf(v * 0.3183098861837907f));
}

// Cell geometry from the prepared faces, as the tessellation forms it
// (Tess2d::extract_geometry tess.cpp:330-393): each face contributes the triangle
// (generator, face) of area w = A h / 4 (h = |x_j - x_i|) to the volume and w times
// its centroid (2 f + x) / 3 to the centre of mass, so
//   vol = sum w,   dcom = (2/3) sum w (f - x) / vol,
// with f - x = c + r n / 2 from pair-i and c - r n / 2 from pair-j.  Ghost rows take
// their image's values (dcom unflipped, as the ghost copies do).  FP32 throughout: the
// relative vectors have no cancellation left.
// The gradient record of one list entry (see entry_rec): minus = the cell is pair-j.
// The roundings are spelled out (IEEE quotient, explicit FMAs) so every kernel that
// forms a record gets the same bits (the full and compact hand-overs form them in
// different kernels).
__device__ __forceinline__ float4 entry_record(float4 g, float2 ar, bool minus) {
    const float a_r = __fdiv_rn(ar.x, ar.y);
    const float ha = (minus ? -0.5f : 0.5f) * ar.x;
    const float hr = (minus ? -0.5f : 0.5f) * ar.y;
    return make_float4(__fmaf_rn(a_r, g.z, __fmul_rn(ha, g.x)), __fmaf_rn(a_r, g.w, __fmul_rn(ha, g.y)),
                       __fmaf_rn(hr, g.x, g.z), __fmaf_rn(hr, g.y, g.w));
}

// The (t_x, t_y) half of entry_record alone, with the same roundings.
__device__ __forceinline__ float2 entry_t(float4 g, float2 ar, bool minus) {
    const float hr = (minus ? -0.5f : 0.5f) * ar.y;
    return make_float2(__fmaf_rn(hr, g.x, g.z), __fmaf_rn(hr, g.y, g.w));
}

// entry_rec, when given, receives the gradient records of a real cell's list entries
// (a ghost's gradient is its image's, formed from the image's entries).
__device__ __forceinline__ float4 cell_geo_of(const phd_mesh &M, int i, const float4 *__restrict__ face_geo,
                                              const float2 *__restrict__ face_ar,
                                              const int32_t *__restrict__ csr_face,
                                              float4 *__restrict__ entry_rec = nullptr) {
    const bool real = M.tag[i] == PHD_REAL_TAG;
    const int c = real ? i : M.map[i];
    float vol = 0.f, sx = 0.f, sy = 0.f;
    if (c >= 0 && c < M.n_cells) {
        for (int e = M.nbr_ptr[c]; e < M.nbr_ptr[c + 1]; e++) {
            const int code = csr_face[e];
            const int fid = code < 0 ? ~code : code;
            const float4 g = face_geo[fid];
            const float2 ar = face_ar[fid];
            const float hr = (code < 0 ? -0.5f : 0.5f) * ar.y;
            const float w = 0.25f * ar.x * ar.y;
            vol += w;
            sx += w * (g.z + hr * g.x);
            sy += w * (g.w + hr * g.y);
            if (entry_rec && real) entry_rec[e] = entry_record(g, ar, code < 0);
        }
    }
    const float inv = vol > 0.f ? 1.f / vol : 0.f;
    return make_float4((2.f / 3.f) * sx * inv, (2.f / 3.f) * sy * inv, inv, sqrtf(vol * 0.3183098861837907f));
}

// entry_rec of every real cell's list from the prepared faces and list codes (a
// ghost's gradient is its image's, formed from the image's entries).
__global__ void k_entry_rec32(phd_mesh M, const float4 *__restrict__ face_geo, const float2 *__restrict__ face_ar,
                              const int32_t *__restrict__ csr_face, float4 *__restrict__ entry_rec) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= M.n_cells || M.tag[c] != PHD_REAL_TAG) return;
    const int F = M.n_faces;
    for (int e = M.nbr_ptr[c]; e < M.nbr_ptr[c + 1]; e++) {
        const int code = csr_face[e];
        const int fid = code < 0 ? ~code : code;
        if (fid < 0 || fid >= F) { entry_rec[e] = make_float4(0.f, 0.f, 0.f, 0.f); continue; }
        entry_rec[e] = entry_record(face_geo[fid], face_ar[fid], code < 0);
    }
}

__global__ void k_cells_from_faces32(phd_mesh M, const float4 *__restrict__ face_geo,
                                     const float2 *__restrict__ face_ar, const int32_t *__restrict__ csr_face,
                                     float4 *__restrict__ cell_geo) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= M.n_cells) return;
    cell_geo[i] = cell_geo_of(M, i, face_geo, face_ar, csr_face);
}

// CSR entries with the side folded into the face id, plus the neighbour cell.  Where a
// twin table is given (periodic faces computed twice by the reference, once from
// each side), the entry of the dropped twin points at the kept face from the other side.
__global__ void k_prepare_csr32(phd_mesh M, const int32_t *__restrict__ twin, int32_t *__restrict__ csr_face,
                                int32_t *__restrict__ csr_nbr) {
    const int c = blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= M.n_cells) return;
    emit_list_codes(c, M.nbr_ptr[c], M.nbr_ptr[c + 1], M.n_cells, M.n_faces, M.nbr_idx, M.pair_i, M.pair_j, twin,
                    csr_face, csr_nbr);
}

// ---- gradients + generator velocity ----------------------------------------------
// Same estimator and limiter as cell_gradient_f64 (reconstruction.pyx:620-736) in
// the relative geometry: with sigma = +1 for pair-i and -1 for pair-j,
//   d phi/dx_k = 1/V sum_faces [ (A/r) (phi_j - phi_i) c_k + sigma A/2 (phi_j + phi_i) n_k ]
//              = 1/V sum_faces (phi_j - phi_i) w_k + (2 phi_i / V) sum_faces sigma A/2 n_k,
//   w = (A/r) c + sigma (A/2) n,
// and the last sum is the cell's closure sum, zero for a closed Voronoi cell (it is
// FP32 rounding noise of the face geometry here; the FP64 path keeps the reference's
// form), so the FP32 estimate is sum (phi_j - phi_i) w / V: one difference and two
// FMAs per face and field, and no cancellation between the two terms.  The neighbour
// extrema enter the limiter only through phi_max - phi_i and phi_min - phi_i, tracked
// directly as the extrema of the same differences (fl(x - phi_i) is monotonic in x, so
// these are the bits of the reference's max - phi_i).  Limiter separation
//   f - (x + dcom) = t - dcom,  t = c + sigma r/2 n.
// w and t of every list entry come precomputed in list order (entry_rec), so the only
// gather left is the neighbour's primitive row.
// The mesh rows of a cell that no kernel of the step writes (its tag, list bounds and
// cell geometry), issued together at the start of the cell.  (Loading the next cell's
// rows during the current one measured about 1 us slower: more live registers.)
struct GradHead {
    int real, e0, e1;
    float4 gc;
};

__device__ __forceinline__ GradHead grad_head(int i, const phd_mesh &M, const float4 *__restrict__ cell_geo) {
    GradHead h;
    h.real = 0;
    h.e0 = h.e1 = 0;
    h.gc = make_float4(0.f, 0.f, 0.f, 0.f);
    if (i < M.n_cells) {
        h.real = M.tag[i] == PHD_REAL_TAG;
        h.e0 = M.nbr_ptr[i];
        h.e1 = M.nbr_ptr[i + 1];
        h.gc = cell_geo[i];
    }
    return h;
}

// Where the list entries' gradient records come from: REC, the precomputed entry_rec in
// list order; otherwise each entry's record is formed here from its face's records
// (csr_face -> face_geo, face_ar) with entry_record's roundings, the same bits (a mesh
// stepped once does not pay for writing and reading 32 B of records per face).
struct EntrySrc {
    const float4 *__restrict__ entry_rec;
    const int32_t *__restrict__ csr_face;
    const float4 *__restrict__ face_geo;
    const float2 *__restrict__ face_ar;
    int n_faces;
};

// An entry's record with at least its (t_x, t_y) half (.z, .w) filled in.
template <bool REC>
__device__ __forceinline__ float4 entry_t_of(const EntrySrc &S, int e) {
    if (REC) return S.entry_rec[e];
    const int code = S.csr_face[e];
    const int fid = code < 0 ? ~code : code;
    if (fid < 0 || fid >= S.n_faces) return make_float4(0.f, 0.f, 0.f, 0.f);
    const float2 t = entry_t(S.face_geo[fid], S.face_ar[fid], code < 0);
    return make_float4(0.f, 0.f, t.x, t.y);
}

template <int LIMITER, bool REC>
__device__ __forceinline__ void grad32_cell(int i, const GradHead &H, const phd_mesh &M, const phd_params &P,
                                            int moving, const EntrySrc &S,
                                            const int32_t *__restrict__ csr_nbr,
                                            const float4 *__restrict__ cell_geo,
                                            const float4 *__restrict__ prim4, float4 *__restrict__ cellrec,
                                            float2 *__restrict__ w2, phd_clock *clk) {
    // the cell's own rows were loaded before its tag was known: for a real cell they are
    // the rows the gradient needs; a ghost reloads its twin's
    const bool real = H.real;
    float4 pc = prim4[i];
    float4 gc = H.gc;
    int e0 = H.e0, e1 = H.e1;
    int c = i;
    if (!real) {
        c = M.map[i];
        if (c < 0 || c >= M.n_cells) { set_status32(clk, PHD_STATUS_BAD_INDEX); return; }
        pc = prim4[c];
        gc = cell_geo[c];
        e0 = M.nbr_ptr[c];
        e1 = M.nbr_ptr[c + 1];
    }
    const float P0[4] = {pc.x, pc.y, pc.z, pc.w};
    float dmx[4], dmn[4], df[4][2];
#pragma unroll
    for (int f = 0; f < 4; f++) { dmx[f] = dmn[f] = 0.f; df[f][0] = df[f][1] = 0.f; }
    // entries in chunks of CH: all of a chunk's loads are issued before any arithmetic,
    // so their latencies overlap (lanes past the end reload entry e0)
    // (two entries per chunk when the records are formed here: 4 took 84 registers and
    // ran 96 us against 76 at 1M cells)
    constexpr int CH = REC ? 4 : 2;
    for (int eb = e0; eb < e1; eb += CH) {
        int nb[CH];
        float4 rw[CH];
        if (REC) {
#pragma unroll
            for (int k = 0; k < CH; k++) {
                const int e = (eb + k < e1) ? eb + k : e0;
                nb[k] = csr_nbr[e];
                rw[k] = S.entry_rec[e];
            }
        } else {
            int code[CH];
#pragma unroll
            for (int k = 0; k < CH; k++) {
                const int e = (eb + k < e1) ? eb + k : e0;
                nb[k] = csr_nbr[e];
                code[k] = S.csr_face[e];
            }
            float4 g[CH];
            float2 ar[CH];
#pragma unroll
            for (int k = 0; k < CH; k++) {
                const int fid = code[k] < 0 ? ~code[k] : code[k];
                const int f = (fid >= 0 && fid < S.n_faces) ? fid : 0;
                g[k] = S.face_geo[f];
                ar[k] = S.face_ar[f];
            }
#pragma unroll
            for (int k = 0; k < CH; k++) {
                const int fid = code[k] < 0 ? ~code[k] : code[k];
                rw[k] = (fid >= 0 && fid < S.n_faces) ? entry_record(g[k], ar[k], code[k] < 0)
                                                      : make_float4(0.f, 0.f, 0.f, 0.f);
            }
        }
        float4 pj[CH];
#pragma unroll
        for (int k = 0; k < CH; k++) pj[k] = prim4[nb[k]];
#pragma unroll
        for (int k = 0; k < CH; k++) {
            if (eb + k >= e1) break;
            const float Pj[4] = {pj[k].x, pj[k].y, pj[k].z, pj[k].w};
#pragma unroll
            for (int f = 0; f < 4; f++) {
                const float d = Pj[f] - P0[f];
                dmx[f] = fmaxf(dmx[f], d);
                dmn[f] = fminf(dmn[f], d);
                df[f][0] += d * rw[k].x;
                df[f][1] += d * rw[k].y;
            }
        }
    }
    float alpha[4] = {1.f, 1.f, 1.f, 1.f};
#pragma unroll
    for (int f = 0; f < 4; f++) { df[f][0] *= gc.z; df[f][1] *= gc.z; }
    if (LIMITER == PHD_LIMITER_AREPO) {
        // alpha_f = min over faces of max(psi, 0), psi = (phi_max - phi)/dphi for dphi > 0
        // and (phi_min - phi)/dphi for dphi < 0: the numerators do not depend on the
        // face, so the minimum is reached at the largest |dphi| of each sign -- two
        // divisions per field instead of one per face and field.  dphi = grad . t -
        // grad . dcom, the second term once per field.
        float dpos[4], dneg[4], gd[4];
#pragma unroll
        for (int f = 0; f < 4; f++) {
            gd[f] = df[f][0] * gc.x + df[f][1] * gc.y;
            dpos[f] = dneg[f] = gd[f];          // the offset is taken out after the loop
        }
        // the same entries again (L1 hits), each chunk's loads issued together
        for (int eb = e0; eb < e1; eb += CH) {
            float4 rt[CH];
#pragma unroll
            for (int k = 0; k < CH; k++) rt[k] = entry_t_of<REC>(S, (eb + k < e1) ? eb + k : e0);
#pragma unroll
            for (int k = 0; k < CH; k++) {
                if (eb + k >= e1) break;
#pragma unroll
                for (int f = 0; f < 4; f++) {
                    const float dphi = df[f][0] * rt[k].z + df[f][1] * rt[k].w;
                    dpos[f] = fmaxf(dpos[f], dphi);
                    dneg[f] = fminf(dneg[f], dphi);
                }
            }
        }
#pragma unroll
        for (int f = 0; f < 4; f++) {
            const float hi = dpos[f] - gd[f], lo = dneg[f] - gd[f];
            if (hi > 0.f) alpha[f] = fminf(alpha[f], dmx[f] / hi);
            if (lo < 0.f) alpha[f] = fminf(alpha[f], dmn[f] / lo);
        }
    } else {
        for (int e = e0; e < e1; e++) {
            const float4 rt = entry_t_of<REC>(S, e);
            const float sx = rt.z - gc.x, sy = rt.w - gc.y;
            const float4 pj = prim4[csr_nbr[e]];
            const float Pj[4] = {pj.x, pj.y, pj.z, pj.w};
#pragma unroll
            for (int f = 0; f < 4; f++) {
                const float dphi = df[f][0] * sx + df[f][1] * sy;
                float psi = 1.f;
                if (dphi != 0.f) psi = fmaxf((Pj[f] - P0[f]) / dphi, 0.f);
                alpha[0] = fminf(alpha[0], fmaxf(psi, 0.f));     // only alpha[0] (:731)
            }
        }
    }
    float gv[8];
#pragma unroll
    for (int f = 0; f < 4; f++) { gv[2 * f] = alpha[f] * df[f][0]; gv[2 * f + 1] = alpha[f] * df[f][1]; }
    const int fl = M.flip[i];
    if (fl & 1) gv[2] = -gv[2];        // d vx / dx
    if (fl & 2) gv[5] = -gv[5];        // d vy / dy

    // the cell's own row (a ghost's, not its image's) for the face kernel
    const float4 p = (i == c) ? pc : prim4[i];
    const float4 gi = (i == c) ? gc : cell_geo[i];
    float wx = 0.f, wy = 0.f;
    if (moving) {   // Mesh.assign_generator_velocities mesh.pyx:397-426, own (ghost) cell data
        wx = p.y;
        wy = p.z;
        if (P.regularize) {
            const float cs = sqrtf(narrow_f64(P.gamma) * p.w / p.x);
            const float d = sqrtf(gi.x * gi.x + gi.y * gi.y);
            const float eR = narrow_f64(P.eta) * gi.w;
            const float q = d / eR;
            if (q >= 0.9f && q < 1.1f) {
                const float s = cs * (d - 0.9f * eR) / (d * 0.2f * eR);
                wx += s * gi.x;
                wy += s * gi.y;
            } else if (q >= 1.1f) {
                wx += cs * gi.x / d;
                wy += cs * gi.y / d;
            }
        }
        w2[i] = make_float2(wx, wy);
    }
    float4 *rec = cellrec + 4 * (size_t)i;
    rec[0] = p;
    rec[1] = make_float4(gv[0], gv[1], gv[2], gv[3]);
    rec[2] = make_float4(gv[4], gv[5], gv[6], gv[7]);
    rec[3] = make_float4(gi.x, gi.y, wx, wy);
}

// ITEMS cells per thread: a block covers blockDim * ITEMS consecutive cells, thread t
// taking cells t, t + blockDim, ... of each tile (the autotuner picks 1, 2 or 4).
template <int LIMITER, int ITEMS, bool REC>
__global__ void __launch_bounds__(512) k_grad32(phd_mesh M, phd_params P, int moving, EntrySrc S,
                                                const int32_t *__restrict__ csr_nbr,
                                                const float4 *__restrict__ cell_geo,
                                                const float4 *__restrict__ prim4, float4 *__restrict__ cellrec,
                                                float2 *__restrict__ w2, phd_clock *clk) {
    pdl_launch_dependents();
    const int tile = blockDim.x * ITEMS;
    pdl_wait();                                  // prim4: written by the previous step's update
    for (int base = blockIdx.x * tile; base < M.n_cells; base += gridDim.x * tile) {
#pragma unroll
        for (int k = 0; k < ITEMS; k++) {
            const int i = base + k * blockDim.x + threadIdx.x;
            if (i < M.n_cells)
                grad32_cell<LIMITER, REC>(i, grad_head(i, M, cell_geo), M, P, moving, S, csr_nbr, cell_geo, prim4,
                                          cellrec, w2, clk);
        }
    }
}

// ---- FP32 Riemann solver with the gas constants formed once on the host -------------
// HLL.get_waves riemann.pyx:375-504 and HLL/HLLC.riemann_solver riemann.pyx:243-373,
// 521-682 in FP32: the same formulas as hll_family<float> with every quantity that
// depends only on gamma ((g-1)/(2g), 1/(g-1), (g+1)/(2g), ...) precomputed, and the
// HLLC left / right star branches merged into one (selects instead of divergence).
// (A variant sharing one density reciprocal per side between the sound speed, the
// shock speeds and the star flux issued fewer multi-function-unit instructions but
// more instructions in all, and measured no faster: with fast-math a division is
// already one reciprocal and one multiply.)
struct GasC {
    float g, inv_gm1, gp1_2g, one_m_gp1_2g, z, inv_z, gm1_gp1, half_gm1, sq_two_gp1;
    ExGas64 X;                 // the exact solver's FP64 Newton constants
};

inline GasC gas_consts(double gamma) {
    const float g = (float)gamma;
    GasC c;
    c.g = g;
    c.inv_gm1 = 1.f / (g - 1.f);
    c.gp1_2g = (g + 1.f) / (2.f * g);
    c.one_m_gp1_2g = 1.f - c.gp1_2g;
    c.z = (g - 1.f) / (2.f * g);
    c.inv_z = 1.f / c.z;
    c.gm1_gp1 = (g - 1.f) / (g + 1.f);
    c.half_gm1 = 0.5f * (g - 1.f);
    c.sq_two_gp1 = std::sqrt(2.f / (g + 1.f));
    c.X = ex_gas64(gamma);
    return c;
}

// ml = d_l (s_l - u_l) and mr = d_r (s_r - u_r) go back with the wave speeds: the
// contact speed is formed from them, and the HLLC star flux reuses them.
__device__ __forceinline__ void get_waves32(float dl, float ul, float pl, float dr, float ur, float pr,
                                            const GasC &C, float &sl, float &sc, float &sr, float &ml, float &mr) {
    float p_star;
    const float cl = fmaxf(sqrtf((C.g * pl) / dl), 1.0e-10f);
    const float cr = fmaxf(sqrtf((C.g * pr) / dr), 1.0e-10f);
    const float d_avg = 0.5f * (dl + dr);
    const float c_avg = 0.5f * (cl + cr);
    p_star = fmaxf(0.f, ((0.5f * (pl + pr)) + (((0.5f * (ul - ur)) * d_avg) * c_avg)));
    const float p_min = fminf(pl, pr);
    const float p_max = fmaxf(pl, pr);
    if (((p_max / p_min) < 2.f) && ((p_min < p_star) && (p_star < p_max))) {
        // PVRS estimate stands
    } else if (p_star <= p_min) {          // two-rarefaction (TRRS)
        // The reference forms u* from both rarefaction relations and averages the two
        // side pressures they give at u*; both equal the root p*, whose closed form is
        // p*^z = (c_l + c_r - (g-1)/2 (u_r - u_l)) / (c_l / p_l^z + c_r / p_r^z) (Toro,
        // eq. 9.42), here with p_l^z / p_r^z = (p_l/p_r)^z: two powers, one division.
        const float plr = __powf(pl / pr, C.z);
        const float num = (cl + cr) - C.half_gm1 * (ur - ul);
        p_star = pr * __powf((plr * num) / (cl + plr * cr), C.inv_z);
    } else {                               // two-shock (TSRS)
        // g_K = sqrt(A_K / (p + B_K)), A_K = 2 / ((g+1) d_K): sqrt(2/(g+1)) / sqrt(d_K (p + B_K))
        const float gl = C.sq_two_gp1 * rsqrtf(dl * (p_star + pl * C.gm1_gp1));
        const float gr = C.sq_two_gp1 * rsqrtf(dr * (p_star + pr * C.gm1_gp1));
        p_star = (((gl * pl) + (gr * pr)) - (ur - ul)) / (gl + gr);
    }
    // shock factor sqrt(1 + (g+1)/(2g) (p*/p_K - 1)) where p* > p_K, else 1 (rarefaction),
    // chosen by a select: both sides' lanes run one code path
    const float xl = sqrtf(fmaf(C.gp1_2g, p_star / pl, C.one_m_gp1_2g));
    const float xr = sqrtf(fmaf(C.gp1_2g, p_star / pr, C.one_m_gp1_2g));
    sl = ul - cl * (p_star <= pl ? 1.f : xl);
    sr = ur + cr * (p_star <= pr ? 1.f : xr);
    ml = dl * (sl - ul);
    mr = dr * (sr - ur);
    sc = (((pr - pl) + ul * ml) - ur * mr) / (ml - mr);
}

// HLL / HLLC flux in FP32.  BOOST: the states are in the face's frame (w.n = 0 there)
// and the flux is de-boosted; else the face moves at w through the lab-frame states.
template <bool HLLC, bool BOOST>
__device__ __forceinline__ void hll_family32(const float *L, const float *R, const float *n, const float *w,
                                             const GasC &C, float *f) {
    const float _dl = L[0], _pl = L[3], _dr = R[0], _pr = R[3];
    const float vl_sq = L[1] * L[1] + L[2] * L[2], vr_sq = R[1] * R[1] + R[2] * R[2];
    const float Vnl = L[1] * n[0] + L[2] * n[1], Vnr = R[1] * n[0] + R[2] * n[1];
    const float wn = BOOST ? 0.f : (w[0] * n[0] + w[1] * n[1]);
    float sl, sc, sr, ml, mr;
    get_waves32(_dl, Vnl, _pl, _dr, Vnr, _pr, C, sl, sc, sr, ml, mr);
    if (wn <= sl) {
        f[0] = _dl * (Vnl - wn);
        f[3] = ((((0.5f * _dl) * vl_sq) + (_pl * C.inv_gm1)) * (Vnl - wn)) + (_pl * Vnl);
        for (int k = 0; k < 2; k++) f[1 + k] = ((_dl * L[1 + k]) * (Vnl - wn)) + (_pl * n[k]);
    } else if ((sl < wn) && (wn <= sr)) {
        if (!HLLC) {
            const float fac1 = sr - wn, fac2 = sl - wn, inv3 = 1.f / (sr - sl);
            f[0] = (((((_dl * Vnl) * fac1) - ((_dr * Vnr) * fac2)) - ((sl * _dl) * fac1)) + ((sr * _dr) * fac2)) *
                   inv3;
            for (int k = 0; k < 2; k++) {
                const float vl = L[1 + k], vr = R[1 + k];
                f[1 + k] = ((((((((_dl * vl) * Vnl) + (_pl * n[k])) * fac1) -
                               ((((_dr * vr) * Vnr) + (_pr * n[k])) * fac2)) -
                              ((sl * (_dl * vl)) * fac1)) + ((sr * (_dr * vr)) * fac2))) * inv3;
            }
            const float el = ((0.5f * _dl) * vl_sq) + (_pl * C.inv_gm1);
            const float er = ((0.5f * _dr) * vr_sq) + (_pr * C.inv_gm1);
            f[3] = ((((((el + _pl) * Vnl) * fac1) - (((er + _pr) * Vnr) * fac2)) - ((sl * el) * fac1)) +
                    ((sr * er) * fac2)) * inv3;
        } else {                           // star region on the side of the contact
            // with m = d (s - Vn) from the wave speeds: factor_1 = m / (s - sc),
            // p / (d (s - Vn)) = p / m
            const bool left = wn <= sc;
            const float d = left ? _dl : _dr, p = left ? _pl : _pr, Vn = left ? Vnl : Vnr, s = left ? sl : sr;
            const float m = left ? ml : mr;
            const float vsq = left ? vl_sq : vr_sq;
            const float *S = left ? L : R;
            const float sw = s - wn;
            const float factor_1 = m / (s - sc);
            const float factor_2 = ((factor_1 * sw) * (sc - Vn)) + p;
            const float frho = (factor_1 * sw) - m;
            const float e = ((0.5f * d) * vsq) + (p * C.inv_gm1);
            f[0] = frho;
            f[3] = (((e + p) * Vn) - (s * e)) + ((sw * factor_1) * ((e / d) + ((sc - Vn) * (sc + (p / m)))));
            for (int k = 0; k < 2; k++) f[1 + k] = (frho * S[1 + k]) + (factor_2 * n[k]);
        }
    } else {
        f[0] = _dr * (Vnr - wn);
        f[3] = ((((0.5f * _dr) * vr_sq) + (_pr * C.inv_gm1)) * (Vnr - wn)) + (_pr * Vnr);
        for (int k = 0; k < 2; k++) f[1 + k] = ((_dr * R[1 + k]) * (Vnr - wn)) + (_pr * n[k]);
    }
    if (BOOST) deboost<float, 2>(w, f);
}

// ---- fused face kernel ------------------------------------------------------------

// FP32 MUSCL-Hancock half step for one side (add_temporal reconstruction.pyx:923-1072,
// temporal of phd_physics.cuh, 2D): X is the side's limited spatial state, p its cell's
// primitives, g the cell's gradient rows (rho 0 1, v_x 2 3, v_y 4 5, p 6 7), (v0, v1)
// the cell's velocity in the frame the states are in, h the half step.  Each field is
// one chain of fused multiply-adds; the state reverts to X where density or pressure
// would turn negative.
__device__ __forceinline__ void half_step32(float *X, const float *p, const float *g, float v0, float v1,
                                            float gamma, float h) {
    const float a0 = h * v0, a1 = h * v1;
    const float hr = h / p[0];
    const float hdiv = h * (g[2] + g[5]);
    const float x0 = fmaf(-p[0], hdiv, fmaf(-a1, g[1], fmaf(-a0, g[0], X[0])));
    const float x1 = fmaf(-hr, g[6], fmaf(-a1, g[3], fmaf(-a0, g[2], X[1])));
    const float x2 = fmaf(-hr, g[7], fmaf(-a1, g[5], fmaf(-a0, g[4], X[2])));
    const float x3 = fmaf(-(gamma * p[3]), hdiv, fmaf(-a1, g[7], fmaf(-a0, g[6], X[3])));
    if (!(x0 < 0.f || x3 < 0.f)) {
        X[0] = x0;
        X[1] = x1;
        X[2] = x2;
        X[3] = x3;
    }
}

// FP32 GIZMO pair limit for one field (reconstruction.pyx:877-915, gizmo_pair of
// phd_physics.cuh) without the reference's case split on the cells' order.  The
// boosted states s_l, s_r are the cells' primitives less one common face velocity, and
// a common shift rounds monotonically, so d = s_r - s_l has the sign of p_j - p_i (or is
// zero).  Then the two ordered cases are one rule per side: the extrapolated state is
// clamped to the interval between an outer bound on its own side, s_l - d/2 (phi_minus
// when p_i < p_j, phi_plus when p_i > p_j; pulled towards zero as phi / (1 + delta1/|phi|)
// = phi |phi| / (|phi| + delta1) where it would change sign), and an inner bound
// s_l + (q_i + 1/4) d (phibar_l + delta2, resp. phibar_l - delta2); the right side
// mirrors it with s_r + d/2 and s_r - (q_j + 1/4) d.  Equal cells give d = 0 and the
// interval {s_l}: the reference's third case.  In both ordered cases the outer bound
// lies on the far side of s_l from the inner one, so the interval is never empty and
// the reference's max(lo, min(hi, x)) and min(hi, max(lo, x)) are the same clamp.
// qi4, qj4: the face's separation quotients plus 1/4.
__device__ __forceinline__ void gizmo_pair32(float sl, float sr, float qi4, float qj4, float &xl, float &xr) {
    const float d = sr - sl;
    float ol = fmaf(-0.5f, d, sl), orr = fmaf(0.5f, d, sr);
    const float il = fmaf(qi4, d, sl), ir = fmaf(-qj4, d, sr);
    if (__builtin_expect(ol * sl < 0.f, 0)) {
        const float a = fabsf(sl);
        ol = (sl * a) / (a + 0.5f * fabsf(d));
    }
    if (__builtin_expect(orr * sr < 0.f, 0)) {
        const float a = fabsf(sr);
        orr = (sr * a) / (a + 0.5f * fabsf(d));
    }
    xl = fminf(fmaxf(xl, fminf(ol, il)), fmaxf(ol, il));
    xr = fminf(fmaxf(xr, fminf(orr, ir)), fmaxf(orr, ir));
}

// 64 bytes of a cell record in two 256-bit loads through the read-only path (the
// record is not written while the face kernel runs).
__device__ __forceinline__ void load_cellrec(const float4 *__restrict__ p, float4 &r0, float4 &r1, float4 &r2,
                                             float4 &r3) {
    asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(r0.x), "=f"(r0.y), "=f"(r0.z), "=f"(r0.w), "=f"(r1.x), "=f"(r1.y), "=f"(r1.z), "=f"(r1.w)
        : "l"(p));
    asm("ld.global.nc.v8.f32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];"
        : "=f"(r2.x), "=f"(r2.y), "=f"(r2.z), "=f"(r2.w), "=f"(r3.x), "=f"(r3.y), "=f"(r3.z), "=f"(r3.w)
        : "l"(p + 2));
}

// One face.  Linear reconstruction reads both cells' records (cellrec: primitives,
// limited gradient, centre offset, generator velocity); constant reconstruction reads
// the primitive rows (and the generator velocities when moving).
// A face's mesh record (pair ids and FP32 geometry).
struct FaceHead {
    int i, j;
    float4 g;
    float2 ar;
};

__device__ __forceinline__ FaceHead face_head(int m, const phd_mesh &M, const float4 *__restrict__ face_geo,
                                              const float2 *__restrict__ face_ar) {
    FaceHead h;
    h.i = h.j = -1;
    h.g = make_float4(0.f, 0.f, 0.f, 0.f);
    h.ar = make_float2(0.f, 0.f);
    if (m < M.n_faces) {
        h.i = M.pair_i[m];
        h.j = M.pair_j[m];
        h.g = face_geo[m];
        h.ar = face_ar[m];
    }
    return h;
}

// dt_run: the step's dt in FP32 when all faces belong to one run (read once per thread).
// BOOST: the reconstruction and the Riemann solver work in the face's frame (always for
// the exact solver, which the reference runs boosted).
template <int SOLVER, bool LINEAR, bool BOOST>
__device__ __forceinline__ void face32_face(int m, const FaceHead &H, const phd_mesh &M, const phd_params &P,
                                            int moving, const float4 *__restrict__ prim4,
                                            const float4 *__restrict__ cellrec, const float2 *__restrict__ w2,
                                            float4 *__restrict__ flux4, phd_clock *clocks,
                                            const int32_t *__restrict__ cell_run, const GasC &GC, float dt_run) {
    const int i = H.i, j = H.j;
    if (i < 0 || i >= M.n_cells || j < 0 || j >= M.n_cells) { set_status32(clocks, PHD_STATUS_BAD_INDEX); return; }
    phd_clock *clk = cell_run ? clocks + cell_run[i] : clocks;
    const float gamma = GC.g;
    const float dtf = cell_run ? narrow_f64(clk->dt) : dt_run;
    const float dt_half = 0.5f * dtf;
    const float4 g = H.g;
    const float2 ar = H.ar;
    const float nrm[2] = {g.x, g.y};
    const float inv_r = 1.f / ar.y;
    float4 a, b, gi0, gi1, gj0, gj1;
    float4 ci = make_float4(0.f, 0.f, 0.f, 0.f), cj = ci;     // (dcom_x, dcom_y, w_x, w_y)
    if (LINEAR) {
        load_cellrec(cellrec + 4 * (size_t)i, a, gi0, gi1, ci);
        load_cellrec(cellrec + 4 * (size_t)j, b, gj0, gj1, cj);
    } else {
        a = prim4[i];
        b = prim4[j];
        if (moving) {
            const float2 wi = w2[i], wj = w2[j];
            ci = make_float4(0.f, 0.f, wi.x, wi.y);
            cj = make_float4(0.f, 0.f, wj.x, wj.y);
        }
    }
    const float pi[4] = {a.x, a.y, a.z, a.w}, pj[4] = {b.x, b.y, b.z, b.w};
    float w[2] = {0.f, 0.f};
    if (moving) {   // Mesh.assign_face_velocities mesh.pyx:462-477: (w_i+w_j)/2 + ((w_i-w_j).c / r) n
        const float fac = ((ci.z - cj.z) * g.z + (ci.w - cj.w) * g.w) * inv_r;
        w[0] = 0.5f * (ci.z + cj.z) + fac * g.x;
        w[1] = 0.5f * (ci.w + cj.w) + fac * g.y;
    }
    float L[4], R[4];
#pragma unroll
    for (int f = 0; f < 4; f++) { L[f] = pi[f]; R[f] = pj[f]; }
    if (BOOST) { L[1] -= w[0]; L[2] -= w[1]; R[1] -= w[0]; R[2] -= w[1]; }
    if (LINEAR) {
        const float gi[8] = {gi0.x, gi0.y, gi0.z, gi0.w, gi1.x, gi1.y, gi1.z, gi1.w};
        const float gj[8] = {gj0.x, gj0.y, gj0.z, gj0.w, gj1.x, gj1.y, gj1.z, gj1.w};
        const float hr = 0.5f * ar.y;
        const float six = g.z + hr * g.x - ci.x, siy = g.w + hr * g.y - ci.y;   // f - (x_i + dcom_i)
        const float sjx = g.z - hr * g.x - cj.x, sjy = g.w - hr * g.y - cj.y;   // f - (x_j + dcom_j)
        float sl[4], sr[4];     // the states at the cells (in the face's frame when boosted)
#pragma unroll
        for (int f = 0; f < 4; f++) {
            sl[f] = L[f];
            sr[f] = R[f];
            L[f] += gi[2 * f] * six + gi[2 * f + 1] * siy;
            R[f] += gj[2 * f] * sjx + gj[2 * f + 1] * sjy;
        }
        if (P.gizmo) {
            const float smi = sqrtf(six * six + siy * siy), smj = sqrtf(sjx * sjx + sjy * sjy);
            const float qi4 = fmaf(smi, inv_r, 0.25f), qj4 = fmaf(smj, inv_r, 0.25f);
#pragma unroll
            for (int f = 0; f < 4; f++) gizmo_pair32(sl[f], sr[f], qi4, qj4, L[f], R[f]);
            if (L[0] < 0.f || L[3] < 0.f) {
#pragma unroll
                for (int f = 0; f < 4; f++) L[f] = sl[f];
            }
            if (R[0] < 0.f || R[3] < 0.f) {
#pragma unroll
                for (int f = 0; f < 4; f++) R[f] = sr[f];
            }
        }
        // the half step takes each cell's velocity in the states' frame: sl[1..2]
        half_step32(L, pi, gi, sl[1], sl[2], gamma, dt_half);
        half_step32(R, pj, gj, sr[1], sr[2], gamma, dt_half);
    }
    float f[4];
    bool failed = false;
    if (SOLVER == PHD_EXACT) exact_flux<float, 2>(L, R, nrm, w, gamma, P.exact_max_iter, f, &failed, &GC.X);
    else hll_family32<SOLVER == PHD_HLLC, BOOST>(L, R, nrm, w, GC, f);
    if (failed) set_status32(clk, PHD_STATUS_RIEMANN_NONCONVERGED);
    // the face's conserved increment dt*A*F (mesh.pyx:519-544), formed once here so both
    // cells of the face apply exactly the same value
    const float s = dtf * ar.x;
    flux4[m] = make_float4(s * f[0], s * f[1], s * f[2], s * f[3]);
}

// At most 256 threads per block and at least 5 blocks per SM: 48 registers per thread
// (no spills), 40 resident warps per SM to hide the face kernel's record -> gather
// latency (measured 4% faster than 56 registers at 384 x 3; at 40 registers it spills).
// The exact solver's kernel is bound by the FP64 pipe instead, and at these caps its
// FP64 Newton iteration spills; it takes one block per SM as its minimum (118-138
// registers, no spills; measured 4% faster).
constexpr int FACE_MAX_BLOCK = 256;

template <int SOLVER, bool LINEAR, int ITEMS, bool BOOST>
__global__ void __launch_bounds__(FACE_MAX_BLOCK, SOLVER == PHD_EXACT ? 1 : 5) k_face32(phd_mesh M, phd_params P, int moving,
                                                const float4 *__restrict__ face_geo,
                                                const float2 *__restrict__ face_ar,
                                                const float4 *__restrict__ prim4,
                                                const float4 *__restrict__ cellrec, const float2 *__restrict__ w2,
                                                float4 *__restrict__ flux4, phd_clock *clocks,
                                                const int32_t *__restrict__ cell_run, const __grid_constant__ GasC GC) {
    pdl_launch_dependents();
    const int tile = blockDim.x * ITEMS;
    pdl_wait();                                  // cellrec / prim4, w2 and the clock: earlier kernels'
    const float dt_run = cell_run ? 0.f : narrow_f64(clocks->dt);
    for (int base = blockIdx.x * tile; base < M.n_faces; base += gridDim.x * tile) {
#pragma unroll
        for (int k = 0; k < ITEMS; k++) {
            const int m = base + k * blockDim.x + threadIdx.x;
            if (m < M.n_faces)
                face32_face<SOLVER, LINEAR, BOOST>(m, face_head(m, M, face_geo, face_ar), M, P, moving, prim4,
                                                   cellrec, w2, flux4, clocks, cell_run, GC, dt_run);
        }
    }
}

// ---- segmented update, primitive recovery and CFL -----------------------------------
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e) {
    s = a + b;
    const float bb = s - a;
    e = (a - (s - bb)) + (b - bb);
}

// One cell of the update: segmented sum, FP64 totals, primitives; returns the CFL
// candidate (INFINITY for ghosts) and the cell's run.
// A cell's mesh rows for the update (tag and list bounds).
struct UpdHead {
    int real, e0, e1;
};

__device__ __forceinline__ UpdHead upd_head(int i, const phd_mesh &M) {
    UpdHead h;
    h.real = 0;
    h.e0 = h.e1 = 0;
    if (i < M.n_cells) {
        h.real = M.tag[i] == PHD_REAL_TAG;
        h.e0 = M.nbr_ptr[i];
        h.e1 = M.nbr_ptr[i + 1];
    }
    return h;
}

__device__ __forceinline__ float update32_cell(int i, const UpdHead &H, const phd_mesh &M, const phd_params &P,
                                               const int32_t *__restrict__ csr_face,
                                               const float4 *__restrict__ flux4,
                                               const float4 *__restrict__ cell_geo,
                                               const double *__restrict__ cons, double *__restrict__ cons_next,
                                               float4 *__restrict__ prim4, phd_clock *clocks,
                                               const int32_t *__restrict__ cell_run, float gam) {
    const int n = M.n_cells;
    phd_clock *clk = cell_run ? clocks + cell_run[i] : clocks;
    // the cell's own list bounds were loaded before its tag was known (a real cell's are
    // the ones it needs); a ghost reloads its image's
    const bool real = H.real;
    int e0 = H.e0, e1 = H.e1;
    const int c = real ? i : M.map[i];
    if (c < 0 || c >= n) { set_status32(clk, PHD_STATUS_BAD_INDEX); return INFINITY; }
    if (!real) {
        e0 = M.nbr_ptr[c];
        e1 = M.nbr_ptr[c + 1];
    }
    float hs[4] = {0.f, 0.f, 0.f, 0.f}, lo[4] = {0.f, 0.f, 0.f, 0.f};
    constexpr int CH = 8;          // measured best for this kernel (CH = 1, 2, 4, 8 tried)
    for (int eb = e0; eb < e1; eb += CH) {
        int code[CH];
#pragma unroll
        for (int k = 0; k < CH; k++) code[k] = csr_face[(eb + k < e1) ? eb + k : e0];
        float4 fl[CH];
#pragma unroll
        for (int k = 0; k < CH; k++) fl[k] = flux4[code[k] < 0 ? ~code[k] : code[k]];
#pragma unroll
        for (int k = 0; k < CH; k++) {
            if (eb + k >= e1) break;
            // the face's increment dt*A*F, identical for both of its cells (compensated
            // sum; packed FP32 pairs measured slower here: more registers, lower occupancy)
            const float inc[4] = {fl[k].x, fl[k].y, fl[k].z, fl[k].w};
#pragma unroll
            for (int q = 0; q < 4; q++) {
                float t, er;
                two_sum(hs[q], code[k] < 0 ? inc[q] : -inc[q], t, er);
                hs[q] = t;
                lo[q] += er;
            }
        }
    }
    // FP64 totals: the only FP64 arithmetic of the step (two adds per field)
    double U[4];
#pragma unroll
    for (int q = 0; q < 4; q++)
        U[q] = (cons[(size_t)q * n + c] + widen_f32_finite(hs[q])) + widen_f32_finite(lo[q]);
    // a blow-up (a total beyond the FP32 range, an infinite or NaN flux sum, which the
    // fast widening turns into a magnitude >= 2^128) is reported, and the cell's
    // primitives become NaN rather than a plausible finite value
    const bool blown = fp64_beyond_f32(U[0]) || fp64_beyond_f32(U[1]) || fp64_beyond_f32(U[2]) ||
                       fp64_beyond_f32(U[3]);
    float m = narrow_f64_finite(U[0]), mx = narrow_f64_finite(U[1]), my = narrow_f64_finite(U[2]);
    if (!fp64_positive(U[0])) set_status32(clk, PHD_STATUS_NEG_MASS);
    if (!fp64_positive(U[3])) set_status32(clk, PHD_STATUS_NEG_ENERGY);
    if (!real) {
        const int fl = M.flip[i];
        if (fl & 1) { U[1] = -U[1]; mx = -mx; }
        if (fl & 2) { U[2] = -U[2]; my = -my; }
    }
#pragma unroll
    for (int q = 0; q < 4; q++) cons_next[(size_t)q * n + i] = U[q];
    // IdealGas.primitive_from_conservative equation_state.pyx:106-117 with the
    // internal energy E - m v^2/2 formed in FP64
    const float4 cg = cell_geo[i];
    float rho = m * cg.z;
    const float rm = 1.f / m;
    float vx = mx * rm, vy = my * rm;
    const float ke = 0.5f * (mx * vx + my * vy);
    float p = (gam - 1.f) * narrow_f64_finite(U[3] - widen_f32_finite(ke)) * cg.z;
    if (blown || !(fabsf(rho) + fabsf(p) + fabsf(vx) + fabsf(vy) < INFINITY)) {
        set_status32(clk, PHD_STATUS_NONFINITE);
        rho = vx = vy = p = __uint_as_float(0x7fc00000u);
    }
    prim4[i] = make_float4(rho, vx, vy, p);
    if (!real) return INFINITY;
    // riemann.pyx:170-187, R = sqrt(vol/pi) precomputed
    const bool boost = (P.solver == PHD_EXACT) ? true : (P.boost != 0);
    const float cs = sqrtf(gam * p / rho);
    return cg.w / (boost ? cs : cs + sqrtf(vx * vx + vy * vy));
}

template <int ITEMS>
__global__ void __launch_bounds__(512) k_update32(phd_mesh M, phd_params P, const int32_t *__restrict__ csr_face,
                                                  const float4 *__restrict__ flux4, const float4 *__restrict__ cell_geo,
                                                  const double *__restrict__ cons, double *__restrict__ cons_next,
                                                  float4 *__restrict__ prim4, phd_clock *clocks,
                                                  const int32_t *__restrict__ cell_run, int n_runs) {
    pdl_launch_dependents();
    const int n = M.n_cells;
    const float gam = narrow_f64(P.gamma);
    const int tile = blockDim.x * ITEMS;
    const int stride = gridDim.x * tile;
    const int n_iter = (n + stride - 1) / stride;     // uniform trip count: all lanes reach the shuffles
    float cand_all = INFINITY;
    pdl_wait();                                       // flux4: the face kernel's; the clocks
    for (int it = 0; it < n_iter; it++) {
#pragma unroll
        for (int k = 0; k < ITEMS; k++) {
            const int i = blockIdx.x * tile + it * stride + k * blockDim.x + threadIdx.x;
            float cand = INFINITY;
            int run = 0;
            if (i < n) {
                cand = update32_cell(i, upd_head(i, M), M, P, csr_face, flux4, cell_geo, cons, cons_next, prim4,
                                     clocks, cell_run, gam);
                if (cell_run) run = cell_run[i];
            }
            if (!cell_run) {
                cand_all = fminf(cand_all, cand);
            } else {
                // per-run minimum: one atomic per warp when the warp lies in one run
                const int r0 = __shfl_sync(0xffffffffu, run, 0);
                if (__all_sync(0xffffffffu, run == r0 || cand == INFINITY)) {
                    const float wm = warp_min_f(cand);
                    if ((threadIdx.x & 31) == 0 && wm < INFINITY)
                        atomic_min_fenced(&clocks[r0].dtmin_bits, dbits((double)wm));
                } else if (cand < INFINITY) {
                    atomic_min_fenced(&clocks[run].dtmin_bits, dbits((double)cand));
                }
            }
        }
    }
    if (!cell_run) block_min_to_f(cand_all, &clocks[0].dtmin_bits);
    finish_cfl_multi(clocks, cell_run ? n_runs : 1, P.cfl, true);
}

// IdealGas.primitive_from_conservative equation_state.pyx:106-117 in FP32 from the FP64
// totals U (internal energy formed in FP64) and the CFL candidate riemann.pyx:170-187
// of a real cell (INFINITY for a ghost); R = sqrt(vol/pi).
__device__ __forceinline__ float prim32_of(const double (&U)[4], float inv_v, float R, bool real,
                                           const phd_params &P, float gam, float4 &out, bool &nonfinite) {
    const float m = narrow_f64(U[0]), mx = narrow_f64(U[1]), my = narrow_f64(U[2]);
    const float rm = 1.f / m;
    const float vx = mx * rm, vy = my * rm;
    const float ke = 0.5f * (mx * vx + my * vy);
    const float p = (gam - 1.f) * narrow_f64(U[3] - widen_f32(ke)) * inv_v;
    const float4 pr = make_float4(m * inv_v, vx, vy, p);
    out = pr;
    if (!(fabsf(pr.x) + fabsf(p) + fabsf(vx) + fabsf(vy) < INFINITY)) nonfinite = true;
    if (!real) return INFINITY;
    const bool boost = (P.solver == PHD_EXACT) ? true : (P.boost != 0);
    const float cs = sqrtf(gam * pr.w / pr.x);
    return R / (boost ? cs : cs + sqrtf(pr.y * pr.y + pr.z * pr.z));
}

// FP64 conserved totals -> FP32 primitive cells and each run's CFL step (clocks not
// advanced).  Same per-run reduction as k_update32.
__global__ void __launch_bounds__(512) k_prim32(phd_mesh M, phd_params P, const double *__restrict__ cons,
                                                float4 *__restrict__ prim4, phd_clock *clocks,
                                                const int32_t *__restrict__ cell_run, int n_runs,
                                                const float4 *__restrict__ cell_geo) {
    const int n = M.n_cells;
    const int stride = gridDim.x * blockDim.x;
    const int n_iter = (n + stride - 1) / stride;
    const float gam = narrow_f64(P.gamma);
    float cand_all = INFINITY;
    for (int it = 0; it < n_iter; it++) {
        const int i = blockIdx.x * blockDim.x + threadIdx.x + it * stride;
        float cand = INFINITY;
        int run = 0;
        if (i < n) {
            // the primitive recovery of k_update32 (FP32, internal energy formed in FP64)
            const double U[4] = {cons[i], cons[(size_t)n + i], cons[2 * (size_t)n + i], cons[3 * (size_t)n + i]};
            float inv_v, R;
            if (cell_geo) {                    // volumes formed on the device from the faces
                const float4 cg = cell_geo[i];
                inv_v = cg.z;
                R = cg.w;
            } else {
                const float v = narrow_f64(M.vol[i]);
                inv_v = 1.f / v;
                R = sqrtf(v * 0.3183098861837907f);
            }
            bool bad = false;
            cand = prim32_of(U, inv_v, R, M.tag[i] == PHD_REAL_TAG, P, gam, prim4[i], bad);
            if (cell_run) run = cell_run[i];
            if (bad) set_status32(clocks + run, PHD_STATUS_NONFINITE);
        }
        if (!cell_run) {
            cand_all = fminf(cand_all, cand);
        } else {
            const int r0 = __shfl_sync(0xffffffffu, run, 0);
            if (__all_sync(0xffffffffu, run == r0 || cand == INFINITY)) {
                const float wm = warp_min_f(cand);
                if ((threadIdx.x & 31) == 0 && wm < INFINITY) atomic_min_fenced(&clocks[r0].dtmin_bits, dbits((double)wm));
            } else if (cand < INFINITY) {
                atomic_min_fenced(&clocks[run].dtmin_bits, dbits((double)cand));
            }
        }
    }
    if (!cell_run) block_min_to_f(cand_all, &clocks[0].dtmin_bits);
    finish_cfl_multi(clocks, cell_run ? n_runs : 1, P.cfl, false);
}

// The tail of a mesh hand-over in one pass per cell: the cell geometry from the faces
// (k_cells_from_faces32) with the real cells' gradient records (k_entry_rec32) from the
// same loads, a ghost's FP64 totals from its image with the momentum
// flipped across reflective walls (k_ghost_cons), the primitives and the CFL step
// (k_prim32) -- the same expressions as the three kernels, so the same bits.
__global__ void __launch_bounds__(512) k_cells_prim32(phd_mesh M, phd_params P, const float4 *__restrict__ face_geo,
                                                      const float2 *__restrict__ face_ar,
                                                      const int32_t *__restrict__ csr_face,
                                                      float4 *__restrict__ entry_rec,
                                                      float4 *__restrict__ cell_geo, double *__restrict__ cons,
                                                      float4 *__restrict__ prim4, phd_clock *clocks) {
    const int n = M.n_cells;
    const int stride = gridDim.x * blockDim.x;
    const int n_iter = (n + stride - 1) / stride;
    const float gam = narrow_f64(P.gamma);
    float cand_all = INFINITY;
    for (int it = 0; it < n_iter; it++) {
        const int i = blockIdx.x * blockDim.x + threadIdx.x + it * stride;
        if (i >= n) continue;
        const float4 cg = cell_geo_of(M, i, face_geo, face_ar, csr_face, entry_rec);
        cell_geo[i] = cg;
        const bool real = M.tag[i] == PHD_REAL_TAG;
        const int c = real ? i : M.map[i];
        double U[4];
        if (real || c < 0 || c >= n) {
#pragma unroll
            for (int q = 0; q < 4; q++) U[q] = cons[(size_t)q * n + i];
        } else {
            const int fl = M.flip ? M.flip[i] : 0;
#pragma unroll
            for (int q = 0; q < 4; q++) {
                double u = cons[(size_t)q * n + c];
                if (q >= 1 && q <= 2 && (fl & (1 << (q - 1)))) u *= -1;
                U[q] = u;
                cons[(size_t)q * n + i] = u;
            }
        }
        bool bad = false;
        cand_all = fminf(cand_all, prim32_of(U, cg.z, cg.w, real, P, gam, prim4[i], bad));
        if (bad) set_status32(clocks, PHD_STATUS_NONFINITE);
    }
    block_min_to_f(cand_all, &clocks[0].dtmin_bits);
    finish_cfl_multi(clocks, 1, P.cfl, false);
}

int cells_prim_f32(const phd_mesh *mesh, const phd_params *par, const phd_geom32_out *out, double *cons,
                   float *prim4, phd_clock *clk, cudaStream_t stream) {
    if (!mesh || mesh->dim != 2 || mesh->n_cells <= 0 || !par || !out || !out->cell_geo || !cons || !prim4 || !clk) return PHD_ERR_ARG;
    k_cells_prim32<<<(mesh->n_cells + B32 - 1) / B32, B32, 0, stream>>>(
        *mesh, *par, reinterpret_cast<const float4 *>(out->face_geo), reinterpret_cast<const float2 *>(out->face_ar),
        out->csr_face, reinterpret_cast<float4 *>(out->entry_rec), reinterpret_cast<float4 *>(out->cell_geo), cons,
        reinterpret_cast<float4 *>(prim4), clk);
    return cudaPeekAtLastError() == cudaSuccess ? PHD_OK : PHD_ERR_LAUNCH;
}

// A step kernel launched with programmatic stream serialization: it may be scheduled
// while the previous kernel of the stream drains (the kernels wait for it with
// pdl_wait before reading what it writes).  Captured into CUDA graphs as programmatic
// edges.
template <typename... KArgs, typename... Args>
cudaError_t launch_pdl(void (*kernel)(KArgs...), int grid, int block, cudaStream_t s, Args &&...args) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, std::forward<Args>(args)...);
}

template <int SOLVER, int ITEMS>
void launch_face32_items(bool linear, int grid, int block, cudaStream_t s, const phd_mesh &M, const phd_params &P,
                         int moving, const phd_geom32 *G, const float4 *prim4, const float4 *cellrec, const float2 *w2,
                         float4 *flux4, phd_clock *clocks, const int32_t *cell_run) {
    const float4 *fg = reinterpret_cast<const float4 *>(G->face_geo);
    const float2 *fa = reinterpret_cast<const float2 *>(G->face_ar);
    const GasC gc = gas_consts(P.gamma);
    constexpr bool EX = SOLVER == PHD_EXACT;      // the exact solver always works boosted
    if (EX || P.boost) {
        if (linear)
            launch_pdl(k_face32<SOLVER, true, ITEMS, true>, grid, block, s, M, P, moving, fg, fa, prim4, cellrec, w2,
                       flux4, clocks, cell_run, gc);
        else
            launch_pdl(k_face32<SOLVER, false, ITEMS, true>, grid, block, s, M, P, moving, fg, fa, prim4, cellrec, w2,
                       flux4, clocks, cell_run, gc);
    } else if constexpr (!EX) {
        if (linear)
            launch_pdl(k_face32<SOLVER, true, ITEMS, false>, grid, block, s, M, P, moving, fg, fa, prim4, cellrec,
                       w2, flux4, clocks, cell_run, gc);
        else
            launch_pdl(k_face32<SOLVER, false, ITEMS, false>, grid, block, s, M, P, moving, fg, fa, prim4, cellrec,
                       w2, flux4, clocks, cell_run, gc);
    }
}

// The exact solver's face kernel is bound by the FP64 pipe and holds 120+ registers:
// it runs one face per thread whatever the requested items.
template <int SOLVER>
void launch_face32(bool linear, int items, int grid, int block, cudaStream_t s, const phd_mesh &M,
                   const phd_params &P, int moving, const phd_geom32 *G, const float4 *prim4, const float4 *cellrec,
                   const float2 *w2, float4 *flux4, phd_clock *clocks, const int32_t *cell_run) {
    if (SOLVER == PHD_EXACT || items == 1)
        launch_face32_items<SOLVER, 1>(linear, grid, block, s, M, P, moving, G, prim4, cellrec, w2, flux4, clocks,
                                       cell_run);
    else if (items == 2)
        launch_face32_items<SOLVER, 2>(linear, grid, block, s, M, P, moving, G, prim4, cellrec, w2, flux4, clocks,
                                       cell_run);
    else
        launch_face32_items<SOLVER, 4>(linear, grid, block, s, M, P, moving, G, prim4, cellrec, w2, flux4, clocks,
                                       cell_run);
}

// grid for n items: one thread per item, or at most `cap` blocks looping over the rest
inline int grid_for(int n, int block, int cap) {
    const int g = (n + block - 1) / block;
    return (cap > 0 && g > cap) ? cap : (g > 0 ? g : 1);
}

inline bool block_ok(int b) { return b >= 32 && b <= 512 && (b % 32) == 0; }

// items per thread: 0 (default) or 1 -> 1, 2, 4
inline bool items_ok(int k) { return k == 0 || k == 1 || k == 2 || k == 4; }
inline int items_of(int k) { return k <= 1 ? 1 : k; }

template <int LIMITER>
void launch_grad32_rec(int items, int grid, int block, cudaStream_t s, const phd_mesh &M, const phd_params &P,
                       int moving, const EntrySrc &S, const int32_t *csr_nbr, const float4 *cg, const float4 *p4,
                       float4 *cr, float2 *w, phd_clock *clocks) {
    if (items == 1)
        launch_pdl(k_grad32<LIMITER, 1, true>, grid, block, s, M, P, moving, S, csr_nbr, cg, p4, cr, w, clocks);
    else if (items == 2)
        launch_pdl(k_grad32<LIMITER, 2, true>, grid, block, s, M, P, moving, S, csr_nbr, cg, p4, cr, w, clocks);
    else
        launch_pdl(k_grad32<LIMITER, 4, true>, grid, block, s, M, P, moving, S, csr_nbr, cg, p4, cr, w, clocks);
}

// without entry records (S.entry_rec null): one item per thread, the records formed
// from the faces (the launch a freshly handed-over mesh's first step takes)
template <int LIMITER>
void launch_grad32(int items, int grid, int block, cudaStream_t s, const phd_mesh &M, const phd_params &P, int moving,
                   const EntrySrc &S, const int32_t *csr_nbr, const float4 *cg, const float4 *p4, float4 *cr,
                   float2 *w, phd_clock *clocks) {
    if (S.entry_rec)
        launch_grad32_rec<LIMITER>(items, grid, block, s, M, P, moving, S, csr_nbr, cg, p4, cr, w, clocks);
    else if (items == 1)
        launch_pdl(k_grad32<LIMITER, 1, false>, grid, block, s, M, P, moving, S, csr_nbr, cg, p4, cr, w, clocks);
    else
        launch_pdl(k_grad32<LIMITER, 2, false>, grid, block, s, M, P, moving, S, csr_nbr, cg, p4, cr, w, clocks);
}

inline int g32(int n) { return n > 0 ? (n + B32 - 1) / B32 : 1; }

// The compact face geometry from one interleaved (area, offset) array face32 [F][2].
int prepare_faces32_interleaved(const phd_mesh *mesh, const float *face32, phd_geom32_out *out, cudaStream_t stream) {
    if (mesh->n_faces)
        k_prepare_faces32_compact<<<g32(mesh->n_faces), B32, 0, stream>>>(
            *mesh, face32, face32 + 1, 2, reinterpret_cast<float4 *>(out->face_geo),
            reinterpret_cast<float2 *>(out->face_ar));
    return cudaPeekAtLastError() == cudaSuccess ? PHD_OK : PHD_ERR_LAUNCH;
}

}  // namespace phd

using namespace phd;

extern "C" {

int phd_prepare_f32_parts(const phd_mesh *mesh, const int32_t *twin, phd_geom32_out *out, int32_t parts,
                          cudaStream_t stream) {
    phd::NvtxRange nvtx_range("phd_prepare_f32");
    if (!mesh || mesh->dim != 2 || !out || parts < 0 ||
        parts > (PHD_PREP_ALL | PHD_PREP_CELLS_FROM_FACES | PHD_PREP_RECORDS))
        return PHD_ERR_ARG;
    if ((parts & PHD_PREP_RECORDS) && (!out->entry_rec || !out->face_geo || !out->face_ar || !out->csr_face))
        return PHD_ERR_ARG;
    if ((parts & PHD_PREP_CELLS) && (parts & PHD_PREP_CELLS_FROM_FACES)) return PHD_ERR_ARG;
    if ((parts & PHD_PREP_CELLS_FROM_FACES) &&
        (!out->cell_geo || !out->face_geo || !out->face_ar || !out->csr_face))
        return PHD_ERR_ARG;
    if ((parts & PHD_PREP_FACES) && (!out->face_geo || !out->face_ar)) return PHD_ERR_ARG;
    if ((parts & PHD_PREP_CELLS) && !out->cell_geo) return PHD_ERR_ARG;
    if ((parts & PHD_PREP_LISTS) && (!out->csr_face || !out->csr_nbr)) return PHD_ERR_ARG;
    if ((parts & PHD_PREP_FACES) && mesh->n_faces)
        k_prepare_faces32<<<g32(mesh->n_faces), B32, 0, stream>>>(*mesh, reinterpret_cast<float4 *>(out->face_geo),
                                                                 reinterpret_cast<float2 *>(out->face_ar));
    if (parts & PHD_PREP_CELLS)
        k_prepare_cells32<<<g32(mesh->n_cells), B32, 0, stream>>>(*mesh,
                                                                 reinterpret_cast<float4 *>(out->cell_geo));
    if (parts & PHD_PREP_LISTS)
        k_prepare_csr32<<<g32(mesh->n_cells), B32, 0, stream>>>(*mesh, twin, out->csr_face, out->csr_nbr);
    if (parts & PHD_PREP_CELLS_FROM_FACES)     // after the faces and lists (stream order)
        k_cells_from_faces32<<<g32(mesh->n_cells), B32, 0, stream>>>(
            *mesh, reinterpret_cast<const float4 *>(out->face_geo), reinterpret_cast<const float2 *>(out->face_ar),
            out->csr_face, reinterpret_cast<float4 *>(out->cell_geo));
    if (parts & PHD_PREP_RECORDS)              // after the faces and lists (stream order)
        k_entry_rec32<<<g32(mesh->n_cells), B32, 0, stream>>>(
            *mesh, reinterpret_cast<const float4 *>(out->face_geo), reinterpret_cast<const float2 *>(out->face_ar),
            out->csr_face, reinterpret_cast<float4 *>(out->entry_rec));
    return cudaPeekAtLastError() == cudaSuccess ? PHD_OK : PHD_ERR_LAUNCH;
}

int phd_prepare_f32_faces_compact(const phd_mesh *mesh, const float *area32, const float *ct32,
                                  phd_geom32_out *out, cudaStream_t stream) {
    phd::NvtxRange nvtx_range("phd_prepare_f32_faces_compact");
    if (!mesh || mesh->dim != 2 || !out || !out->face_geo || !out->face_ar) return PHD_ERR_ARG;
    if (mesh->n_faces && (!area32 || !ct32 || !mesh->pair_i || !mesh->pair_j || !mesh->x)) return PHD_ERR_ARG;
    if (mesh->n_faces)
        k_prepare_faces32_compact<<<g32(mesh->n_faces), B32, 0, stream>>>(
            *mesh, area32, ct32, 1, reinterpret_cast<float4 *>(out->face_geo),
            reinterpret_cast<float2 *>(out->face_ar));
    return cudaPeekAtLastError() == cudaSuccess ? PHD_OK : PHD_ERR_LAUNCH;
}


int phd_pair_i_from_face_ptr(const phd_mesh *mesh, const int32_t *face_ptr, int32_t *pair_i, int32_t *bad,
                             cudaStream_t stream) {
    phd::NvtxRange nvtx_range("phd_pair_i_from_face_ptr");
    if (!mesh || !face_ptr || !pair_i || !bad || mesh->n_real < 1 || mesh->n_faces < 0) return PHD_ERR_ARG;
    k_pair_i_from_ptr<<<g32(mesh->n_real), B32, 0, stream>>>(mesh->n_real, mesh->n_faces, face_ptr, pair_i, bad);
    return cudaPeekAtLastError() == cudaSuccess ? PHD_OK : PHD_ERR_LAUNCH;
}

int phd_prepare_f32(const phd_mesh *mesh, const int32_t *twin, phd_geom32_out *out, cudaStream_t stream) {
    return phd_prepare_f32_parts(mesh, twin, out, PHD_PREP_ALL | (out && out->entry_rec ? PHD_PREP_RECORDS : 0),
                                 stream);
}

int phd_prim_f32_batched(const phd_mesh *mesh, const phd_params *par, const double *cons, float *prim4,
                         phd_clock *clocks, int32_t n_runs, const int32_t *cell_run, cudaStream_t stream) {
    if (!mesh || mesh->dim != 2 || !par || !cons || !prim4 || !clocks) return PHD_ERR_ARG;
    if (n_runs < 1 || (n_runs > 1 && !cell_run)) return PHD_ERR_ARG;
    k_prim32<<<g32(mesh->n_cells), B32, 0, stream>>>(*mesh, *par, cons, reinterpret_cast<float4 *>(prim4), clocks,
                                                     n_runs > 1 ? cell_run : nullptr, n_runs, nullptr);
    return cudaPeekAtLastError() == cudaSuccess ? PHD_OK : PHD_ERR_LAUNCH;
}

int phd_prim_f32(const phd_mesh *mesh, const phd_params *par, const double *cons, float *prim4, phd_clock *clk,
                 cudaStream_t stream) {
    return phd_prim_f32_batched(mesh, par, cons, prim4, clk, 1, nullptr, stream);
}

int phd_prim_f32_cells(const phd_mesh *mesh, const float *cell_geo, const phd_params *par, const double *cons,
                       float *prim4, phd_clock *clk, cudaStream_t stream) {
    if (!mesh || mesh->dim != 2 || !cell_geo || !par || !cons || !prim4 || !clk) return PHD_ERR_ARG;
    k_prim32<<<g32(mesh->n_cells), B32, 0, stream>>>(*mesh, *par, cons, reinterpret_cast<float4 *>(prim4), clk,
                                                     nullptr, 1, reinterpret_cast<const float4 *>(cell_geo));
    return cudaPeekAtLastError() == cudaSuccess ? PHD_OK : PHD_ERR_LAUNCH;
}

int phd_step_f32_batched(const phd_mesh *mesh, const phd_geom32 *geo, const phd_params *par, int32_t moving,
                         const phd_launch *launch, float *prim4, const double *cons, double *cons_next, float *cellrec,
                         float *w2, float *flux4, phd_clock *clocks, int32_t n_runs, const int32_t *cell_run,
                         cudaStream_t stream, cudaEvent_t *marks) {
    phd::NvtxRange nvtx_range("phd_step_f32");
    if (!mesh || mesh->dim != 2 || !geo || !par || !prim4 || !cons || !cons_next || !flux4 || !clocks)
        return PHD_ERR_ARG;
    const bool linear = par->reconstruction == PHD_LINEAR;
    if ((linear || moving) && (!cellrec || !geo->csr_nbr)) return PHD_ERR_ARG;
    if ((linear || moving) && !geo->entry_rec && (!geo->face_geo || !geo->face_ar || !geo->csr_face))
        return PHD_ERR_ARG;
    if (moving && !w2) return PHD_ERR_ARG;
    if ((reinterpret_cast<uintptr_t>(cellrec) & 31u) != 0) return PHD_ERR_ARG;    // 256-bit loads
    if (par->solver < PHD_HLL || par->solver > PHD_EXACT) return PHD_ERR_ARG;
    if (n_runs < 1 || (n_runs > 1 && !cell_run)) return PHD_ERR_ARG;
    phd_launch L = {B32, B32, B32, 0, 0, 0, 1, 1, 1};
    if (launch) {
        if (!block_ok(launch->block_grad) || !block_ok(launch->block_face) || !block_ok(launch->block_update) ||
            launch->block_face > FACE_MAX_BLOCK || !items_ok(launch->items_grad) || !items_ok(launch->items_face) ||
            !items_ok(launch->items_update))
            return PHD_ERR_ARG;
        L = *launch;
    }
    const int ig = items_of(L.items_grad), ifc = par->solver == PHD_EXACT ? 1 : items_of(L.items_face),
              iu = items_of(L.items_update);
    const phd_mesh &M = *mesh;
    const int gc = grid_for((M.n_cells + ig - 1) / ig, L.block_grad, L.grid_cap_grad);
    const int gf = grid_for((M.n_faces + ifc - 1) / ifc, L.block_face, L.grid_cap_face);
    const int gu = grid_for((M.n_cells + iu - 1) / iu, L.block_update, L.grid_cap_update);
    float4 *p4 = reinterpret_cast<float4 *>(prim4);
    float4 *cr = reinterpret_cast<float4 *>(cellrec);
    float2 *w = reinterpret_cast<float2 *>(w2);
    float4 *fx = reinterpret_cast<float4 *>(flux4);
    const EntrySrc er = {reinterpret_cast<const float4 *>(geo->entry_rec), geo->csr_face,
                         reinterpret_cast<const float4 *>(geo->face_geo), reinterpret_cast<const float2 *>(geo->face_ar),
                         M.n_faces};
    const float4 *cg = reinterpret_cast<const float4 *>(geo->cell_geo);
    const int32_t *runs = n_runs > 1 ? cell_run : nullptr;
    if (marks) cudaEventRecord(marks[0], stream);
    if (linear || moving) {
        if (par->limiter == PHD_LIMITER_TESS)
            launch_grad32<PHD_LIMITER_TESS>(ig, gc, L.block_grad, stream, M, *par, (int)moving, er, geo->csr_nbr, cg,
                                            p4, cr, w, clocks);
        else
            launch_grad32<PHD_LIMITER_AREPO>(ig, gc, L.block_grad, stream, M, *par, (int)moving, er, geo->csr_nbr, cg,
                                             p4, cr, w, clocks);
    }
    if (marks) cudaEventRecord(marks[1], stream);
    if (M.n_faces) {
        switch (par->solver) {
            case PHD_HLL:
                launch_face32<PHD_HLL>(linear, ifc, gf, L.block_face, stream, M, *par, moving, geo, p4, cr, w, fx, clocks,
                                       runs);
                break;
            case PHD_HLLC:
                launch_face32<PHD_HLLC>(linear, ifc, gf, L.block_face, stream, M, *par, moving, geo, p4, cr, w, fx, clocks,
                                        runs);
                break;
            default:
                launch_face32<PHD_EXACT>(linear, 1, gf, L.block_face, stream, M, *par, moving, geo, p4, cr, w, fx,
                                         clocks, runs);
                break;
        }
    }
    if (marks) cudaEventRecord(marks[2], stream);
    if (iu == 1)
        launch_pdl(k_update32<1>, gu, L.block_update, stream, M, *par, geo->csr_face, (const float4 *)fx, cg, cons,
                   cons_next, p4, clocks, runs, (int)n_runs);
    else if (iu == 2)
        launch_pdl(k_update32<2>, gu, L.block_update, stream, M, *par, geo->csr_face, (const float4 *)fx, cg, cons,
                   cons_next, p4, clocks, runs, (int)n_runs);
    else
        launch_pdl(k_update32<4>, gu, L.block_update, stream, M, *par, geo->csr_face, (const float4 *)fx, cg, cons,
                   cons_next, p4, clocks, runs, (int)n_runs);
    if (marks) cudaEventRecord(marks[3], stream);
    return cudaPeekAtLastError() == cudaSuccess ? PHD_OK : PHD_ERR_LAUNCH;
}

int phd_step_f32_marked(const phd_mesh *mesh, const phd_geom32 *geo, const phd_params *par, int32_t moving,
                        float *prim4, const double *cons, double *cons_next, float *cellrec, float *w2,
                        float *flux4, phd_clock *clk, cudaStream_t stream, cudaEvent_t *marks) {
    return phd_step_f32_batched(mesh, geo, par, moving, nullptr, prim4, cons, cons_next, cellrec, w2, flux4, clk, 1,
                                nullptr, stream, marks);
}

int phd_step_f32(const phd_mesh *mesh, const phd_geom32 *geo, const phd_params *par, int32_t moving,
                 float *prim4, const double *cons, double *cons_next, float *cellrec, float *w2, float *flux4,
                 phd_clock *clk, cudaStream_t stream) {
    return phd_step_f32_batched(mesh, geo, par, moving, nullptr, prim4, cons, cons_next, cellrec, w2, flux4, clk, 1,
                                nullptr, stream, nullptr);
}

}  // extern "C"
