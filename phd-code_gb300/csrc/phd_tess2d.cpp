// phd_tess2d.cpp -- host 2D Delaunay / Voronoi tessellation (libphdtess.so).
//
// The reference tessellates on the host with CGAL (phd/mesh/tess.cpp, an exact-
// predicates Delaunay_triangulation_2) and hands the flux path a face list.  CGAL is
// not part of this build, so this file provides the same service from scratch:
//
//  * Delaunay triangulation by Bowyer-Watson insertion (cavity of triangles whose
//    circumcircle strictly contains the new point, re-triangulated as a fan), inside
//    a large enclosing triangle, with points inserted in a biased randomised order
//    (rounds of doubling size, each along a Hilbert curve) so that cavities stay small
//    and the visibility walk that locates each point stays short;
//  * robust orientation and in-circle tests: a floating-point evaluation with the
//    forward error bounds of Shewchuk (1997, "Adaptive precision floating-point
//    arithmetic and fast robust geometric predicates", ccwerrboundA / iccerrboundA),
//    and, when the sign is not certain, an exact evaluation with the paper's
//    expansion arithmetic (Two-Sum, Two-Product via fma, Grow-Expansion,
//    Scale-Expansion with zero elimination); exactly cocircular points are decided by
//    a symbolic perturbation of the lift (incircle_sos), so the triangulation is unique;
//  * Voronoi extraction in the conventions of Tess2d::extract_geometry
//    (tess.cpp:238-398) and of the host mesh builder that feeds the flux path: faces
//    per real cell in counter-clockwise neighbour order from angle -pi, volume and
//    centroid sums over the incident edges, face lists in ascending face id.
//
// Circumcentres use the same closed form as the numpy mesh builder, so faces agree
// with it to rounding.  Built with -ffp-contract=off: the error-bound filters assume
// separately rounded products and sums.
#include "phdtess.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <new>
#include <thread>
#include <utility>
#include <vector>

namespace {

// ---- exact arithmetic (Shewchuk 1997, sections 2.3-2.6) ---------------------------
inline void two_sum(double a, double b, double &x, double &y) {
    x = a + b;
    const double bv = x - a;
    const double av = x - bv;
    y = (a - av) + (b - bv);
}

inline void fast_two_sum(double a, double b, double &x, double &y) {   // |a| >= |b|
    x = a + b;
    const double bv = x - a;
    y = b - bv;
}

inline void two_diff(double a, double b, double &x, double &y) {
    x = a - b;
    const double bv = a - x;
    const double av = x + bv;
    y = (a - av) + (bv - b);
}

inline void two_prod(double a, double b, double &x, double &y) {
    x = a * b;
    y = std::fma(a, b, -x);
}

// nonoverlapping expansion, components in increasing magnitude, zeros removed
typedef std::vector<double> Exp;

Exp exp_of_diff(double a, double b) {
    double x, y;
    two_diff(a, b, x, y);
    Exp e;
    if (y != 0.) e.push_back(y);
    if (x != 0.) e.push_back(x);
    return e;
}

// Grow-Expansion: e + b
Exp exp_grow(const Exp &e, double b) {
    Exp h;
    h.reserve(e.size() + 1);
    double q = b;
    for (double ei : e) {
        double qn, hh;
        two_sum(q, ei, qn, hh);
        if (hh != 0.) h.push_back(hh);
        q = qn;
    }
    if (q != 0.) h.push_back(q);
    return h;
}

Exp exp_add(const Exp &e, const Exp &f) {
    Exp h = e;
    for (double fj : f) h = exp_grow(h, fj);
    return h;
}

Exp exp_neg(Exp e) {
    for (double &v : e) v = -v;
    return e;
}

// Scale-Expansion: b * e
Exp exp_scale(const Exp &e, double b) {
    Exp h;
    if (e.empty() || b == 0.) return h;
    h.reserve(2 * e.size());
    double q, hh;
    two_prod(e[0], b, q, hh);
    if (hh != 0.) h.push_back(hh);
    for (size_t i = 1; i < e.size(); i++) {
        double T, t, qn;
        two_prod(e[i], b, T, t);
        two_sum(q, t, qn, hh);
        if (hh != 0.) h.push_back(hh);
        fast_two_sum(T, qn, q, hh);
        if (hh != 0.) h.push_back(hh);
    }
    if (q != 0.) h.push_back(q);
    return h;
}

Exp exp_mul(const Exp &e, const Exp &f) {
    Exp h;
    for (double fj : f) h = exp_add(h, exp_scale(e, fj));
    return h;
}

int exp_sign(const Exp &e) { return e.empty() ? 0 : (e.back() > 0. ? 1 : -1); }

const double EPS = 1.1102230246251565e-16;                 // 2^-53
const double CCW_ERR_A = (3.0 + 16.0 * EPS) * EPS;
const double ICC_ERR_A = (10.0 + 96.0 * EPS) * EPS;

// > 0 when a, b, c turn counter-clockwise
int orient2d(double ax, double ay, double bx, double by, double cx, double cy) {
    const double detleft = (ax - cx) * (by - cy);
    const double detright = (ay - cy) * (bx - cx);
    const double det = detleft - detright;
    double detsum;
    if (detleft > 0.) {
        if (detright <= 0.) return det > 0. ? 1 : (det < 0. ? -1 : 0);
        detsum = detleft + detright;
    } else if (detleft < 0.) {
        if (detright >= 0.) return det > 0. ? 1 : (det < 0. ? -1 : 0);
        detsum = -detleft - detright;
    } else {
        return det > 0. ? 1 : (det < 0. ? -1 : 0);
    }
    const double bound = CCW_ERR_A * detsum;
    if (det >= bound || -det >= bound) return det > 0. ? 1 : -1;
    const Exp acx = exp_of_diff(ax, cx), bcy = exp_of_diff(by, cy);
    const Exp acy = exp_of_diff(ay, cy), bcx = exp_of_diff(bx, cx);
    return exp_sign(exp_add(exp_mul(acx, bcy), exp_neg(exp_mul(acy, bcx))));
}

int incircle_sos(double ax, double ay, double bx, double by, double cx, double cy, double dx, double dy);

// > 0 when d lies inside the circle through the counter-clockwise a, b, c; exactly
// cocircular points are decided by a symbolic perturbation (incircle_sos), so the
// result is never 0 for four distinct points in general position of the lift
int incircle(double ax, double ay, double bx, double by, double cx, double cy, double dx, double dy) {
    const double adx = ax - dx, bdx = bx - dx, cdx = cx - dx;
    const double ady = ay - dy, bdy = by - dy, cdy = cy - dy;
    const double bdxcdy = bdx * cdy, cdxbdy = cdx * bdy;
    const double alift = adx * adx + ady * ady;
    const double cdxady = cdx * ady, adxcdy = adx * cdy;
    const double blift = bdx * bdx + bdy * bdy;
    const double adxbdy = adx * bdy, bdxady = bdx * ady;
    const double clift = cdx * cdx + cdy * cdy;
    const double det = alift * (bdxcdy - cdxbdy) + blift * (cdxady - adxcdy) + clift * (adxbdy - bdxady);
    const double perm = (std::fabs(bdxcdy) + std::fabs(cdxbdy)) * alift +
                        (std::fabs(cdxady) + std::fabs(adxcdy)) * blift +
                        (std::fabs(adxbdy) + std::fabs(bdxady)) * clift;
    const double bound = ICC_ERR_A * perm;
    if (det > bound || -det > bound) return det > 0. ? 1 : -1;
    const Exp eax = exp_of_diff(ax, dx), eay = exp_of_diff(ay, dy);
    const Exp ebx = exp_of_diff(bx, dx), eby = exp_of_diff(by, dy);
    const Exp ecx = exp_of_diff(cx, dx), ecy = exp_of_diff(cy, dy);
    const Exp la = exp_add(exp_mul(eax, eax), exp_mul(eay, eay));
    const Exp lb = exp_add(exp_mul(ebx, ebx), exp_mul(eby, eby));
    const Exp lc = exp_add(exp_mul(ecx, ecx), exp_mul(ecy, ecy));
    const Exp ka = exp_add(exp_mul(ebx, ecy), exp_neg(exp_mul(ecx, eby)));
    const Exp kb = exp_add(exp_mul(ecx, eay), exp_neg(exp_mul(eax, ecy)));
    const Exp kc = exp_add(exp_mul(eax, eby), exp_neg(exp_mul(ebx, eay)));
    const int sgn = exp_sign(exp_add(exp_add(exp_mul(la, ka), exp_mul(lb, kb)), exp_mul(lc, kc)));
    return sgn != 0 ? sgn : incircle_sos(ax, ay, bx, by, cx, cy, dx, dy);
}

// Exactly cocircular a, b, c, d (a generator, its neighbour and their mirror images at
// a wall; four lattice points): lift every point to l = x^2 + y^2 + e_p with
// infinitesimals e_p ordered by the points' lexicographic (x, y) order (the smallest
// point's the largest).  The in-circle determinant is linear in the lifts, so its sign
// is that of the first non-zero coefficient in that order: e_a orient(b,c,d),
// -e_b orient(a,c,d), e_c orient(a,b,d), -e_d orient(a,b,c).  The triangulation is then
// the unique Delaunay triangulation of the perturbed lift -- the same whatever the
// insertion order or the strip that builds it.
int incircle_sos(double ax, double ay, double bx, double by, double cx, double cy, double dx, double dy) {
    struct P { double x, y; int k; } pt[4] = {{ax, ay, 0}, {bx, by, 1}, {cx, cy, 2}, {dx, dy, 3}};
    std::sort(pt, pt + 4, [](const P &u, const P &v) { return u.x < v.x || (u.x == v.x && u.y < v.y); });
    for (const P &q : pt) {
        int c = 0;
        switch (q.k) {
            case 0: c = orient2d(bx, by, cx, cy, dx, dy); break;
            case 1: c = -orient2d(ax, ay, cx, cy, dx, dy); break;
            case 2: c = orient2d(ax, ay, bx, by, dx, dy); break;
            default: c = -orient2d(ax, ay, bx, by, cx, cy); break;
        }
        if (c != 0) return c;
    }
    return 0;
}

// ---- Hilbert key (phd/hilbert/hilbert.pyx:9-23) -------------------------------------
const int KEY_INDEX_2D[4] = {0, 1, 3, 2};

int64_t hilbert_key_2d(int32_t x, int32_t y, int order) {
    int64_t key = 0;
    for (int i = order - 1; i >= 0; i--) {
        const int xbit = (x & (int32_t(1) << i)) ? 1 : 0;
        const int ybit = (y & (int32_t(1) << i)) ? 1 : 0;
        if (xbit == 0 && ybit == 0) {
            std::swap(x, y);
        } else if (xbit == 1 && ybit == 0) {
            const int32_t nx = ~y, ny = ~x;
            x = nx;
            y = ny;
        }
        key = (key << 2) + KEY_INDEX_2D[(xbit << 1) + ybit];
    }
    return key;
}

// ---- triangulation --------------------------------------------------------------
struct Tri {
    int v[3];      // counter-clockwise; < 0: a vertex of the enclosing triangle
    int n[3];      // n[k]: triangle across the edge opposite v[k] (-1: none)
};

struct Geometry {   // one phd_mesh2d_build result
    int n_real = 0, n_cells = 0, n_faces = 0;
    double pad_used = 0.;
    std::vector<double> x, y, vol, dcx, dcy, area, comx, comy, nx, ny;
    std::vector<int32_t> map, pair_i, pair_j, nbr_ptr, nbr_idx;
    std::vector<int8_t> gcode;      // per kept ghost: how it images its real cell (ghost_code)
};

}  // namespace

struct phd_tess2d {
    std::vector<double> X, Y;          // inserted generators, by particle id
    std::vector<char> inserted;
    double SX[3] = {0, 0, 0}, SY[3] = {0, 0, 0};
    std::vector<Tri> tris;
    std::vector<int> free_tris;
    std::vector<int> vt;               // one triangle incident to each generator
    std::vector<int> bad_mark, seen_mark;
    int stamp = 0;
    int last = -1;
    int n_real = 0, n_total = 0;
    // scratch for one insertion
    std::vector<int> bad, stack, nt;
    struct BEdge { int a, b, outer, outer_k; };
    std::vector<BEdge> bnd;
    Geometry G;

    double px(int v) const { return v >= 0 ? X[v] : SX[-v - 1]; }
    double py(int v) const { return v >= 0 ? Y[v] : SY[-v - 1]; }

    void reset() {
        X.clear(); Y.clear(); inserted.clear(); tris.clear(); free_tris.clear(); vt.clear();
        bad_mark.clear(); seen_mark.clear(); stamp = 0; last = -1; n_real = n_total = 0;
    }

    int new_tri() {
        if (!free_tris.empty()) {
            const int t = free_tris.back();
            free_tris.pop_back();
            return t;
        }
        tris.push_back(Tri());
        bad_mark.push_back(0);
        seen_mark.push_back(0);
        return int(tris.size()) - 1;
    }

    void init_super(double x0, double y0, double x1, double y1) {
        const double cx = 0.5 * (x0 + x1), cy = 0.5 * (y0 + y1);
        double ext = std::max(x1 - x0, y1 - y0);
        if (!(ext > 0.)) ext = 1.;
        const double M = 1.0e4 * ext;
        SX[0] = cx - 2. * M; SY[0] = cy - M;
        SX[1] = cx + 2. * M; SY[1] = cy - M;
        SX[2] = cx;          SY[2] = cy + 2. * M;
        tris.clear(); free_tris.clear(); bad_mark.clear(); seen_mark.clear();
        const int t = new_tri();
        tris[t].v[0] = -1; tris[t].v[1] = -2; tris[t].v[2] = -3;
        tris[t].n[0] = tris[t].n[1] = tris[t].n[2] = -1;
        last = t;
    }

    bool in_circle(const Tri &T, int p) const {
        return incircle(px(T.v[0]), py(T.v[0]), px(T.v[1]), py(T.v[1]), px(T.v[2]), py(T.v[2]), X[p], Y[p]) > 0;
    }

    // visibility walk from the last created triangle
    int locate(int p) {
        int t = last;
        const double x = X[p], y = Y[p];
        int start = 0;
        const long max_steps = 4L * long(tris.size()) + 64;
        for (long step = 0; step < max_steps; step++) {
            const Tri &T = tris[t];
            int next = -1;
            bool outside = false;
            for (int kk = 0; kk < 3; kk++) {
                const int k = (kk + start) % 3;
                const int a = T.v[(k + 1) % 3], b = T.v[(k + 2) % 3];
                if (orient2d(px(a), py(a), px(b), py(b), x, y) < 0) { next = T.n[k]; outside = true; break; }
            }
            if (!outside) return t;
            if (next < 0) return -1;                      // outside the enclosing triangle
            t = next;
            start = (start + 1) % 3;
        }
        return -1;
    }

    // insert generator p (coordinates already in X, Y); 0 or an error code
    int insert(int p) {
        const int t0 = locate(p);
        if (t0 < 0) return -4;
        {
            const Tri &T = tris[t0];
            for (int k = 0; k < 3; k++)
                if (T.v[k] >= 0 && X[T.v[k]] == X[p] && Y[T.v[k]] == Y[p]) return -3;
        }
        if (++stamp == 0x7fffffff) {
            std::fill(bad_mark.begin(), bad_mark.end(), 0);
            std::fill(seen_mark.begin(), seen_mark.end(), 0);
            stamp = 1;
        }
        bad.clear();
        stack.clear();
        bad_mark[t0] = stamp;
        seen_mark[t0] = stamp;
        stack.push_back(t0);
        while (!stack.empty()) {
            const int t = stack.back();
            stack.pop_back();
            bad.push_back(t);
            for (int k = 0; k < 3; k++) {
                const int nb = tris[t].n[k];
                if (nb < 0 || seen_mark[nb] == stamp) continue;
                seen_mark[nb] = stamp;
                if (in_circle(tris[nb], p)) {
                    bad_mark[nb] = stamp;
                    stack.push_back(nb);
                }
            }
        }
        bnd.clear();
        for (int t : bad) {
            const Tri &T = tris[t];
            for (int k = 0; k < 3; k++) {
                const int nb = T.n[k];
                if (nb >= 0 && bad_mark[nb] == stamp) continue;
                int ok = -1;                                   // the outer triangle's edge back to t
                if (nb >= 0)
                    for (int m = 0; m < 3; m++)
                        if (tris[nb].n[m] == t) ok = m;
                if (nb >= 0 && ok < 0) return -4;
                bnd.push_back({T.v[(k + 1) % 3], T.v[(k + 2) % 3], nb, ok});
            }
        }
        // the cavity is star-shaped from p: one new triangle (p, a, b) per boundary edge
        const size_t m = bnd.size();
        if (m != bad.size() + 2) return -4;
        nt.resize(m);
        for (size_t j = 0; j < m; j++) nt[j] = j < bad.size() ? bad[j] : new_tri();
        for (size_t j = 0; j < m; j++) {
            Tri &T = tris[nt[j]];
            T.v[0] = p; T.v[1] = bnd[j].a; T.v[2] = bnd[j].b;
            T.n[0] = bnd[j].outer;
            bad_mark[nt[j]] = 0;
            if (bnd[j].outer >= 0) tris[bnd[j].outer].n[bnd[j].outer_k] = nt[j];
        }
        for (size_t j = 0; j < m; j++) {
            Tri &T = tris[nt[j]];
            T.n[1] = T.n[2] = -1;
            for (size_t q = 0; q < m; q++) {
                if (bnd[q].a == bnd[j].b) T.n[1] = nt[q];       // across (b, p)
                if (bnd[q].b == bnd[j].a) T.n[2] = nt[q];       // across (p, a)
            }
            if (T.n[1] < 0 || T.n[2] < 0) return -4;
            if (bnd[j].a >= 0) vt[bnd[j].a] = nt[j];
            if (bnd[j].b >= 0) vt[bnd[j].b] = nt[j];
        }
        vt[p] = nt[0];
        last = nt[0];
        inserted[p] = 1;
        return 0;
    }

    // insert generators [begin, end) in a biased randomised insertion order (Amenta,
    // Choi and Rote 2003): a seeded shuffle split into rounds of doubling size, each
    // round sorted along a Hilbert curve over the bounding box -- later rounds land inside
    // the triangulation already built (small cavities), and consecutive points are close
    // (short walks).  The seed is fixed, so the result is reproducible.
    int insert_range(int begin, int end) {
        if (end <= begin) return 0;
        double x0 = X[begin], x1 = X[begin], y0 = Y[begin], y1 = Y[begin];
        for (int i = begin; i < end; i++) {
            x0 = std::min(x0, X[i]); x1 = std::max(x1, X[i]);
            y0 = std::min(y0, Y[i]); y1 = std::max(y1, Y[i]);
        }
        double box = std::max(x1 - x0, y1 - y0);
        if (!(box > 0.)) box = 1.;
        const double scale = double(1 << 16) / box;
        const int n = end - begin;
        std::vector<int> perm(n);
        for (int k = 0; k < n; k++) perm[k] = begin + k;
        uint64_t st = 0x9E3779B97F4A7C15ull;                  // xorshift64* shuffle, fixed seed
        for (int k = n - 1; k > 0; k--) {
            st ^= st >> 12; st ^= st << 25; st ^= st >> 27;
            const uint64_t r = (st * 0x2545F4914F6CDD1Dull) >> 11;
            std::swap(perm[k], perm[int(r % uint64_t(k + 1))]);
        }
        std::vector<std::pair<int64_t, int>> round;
        int lo = 0;
        for (int hi = std::min(n, 64); lo < n; hi = std::min(n, 2 * hi)) {
            round.resize(hi - lo);
            for (int k = lo; k < hi; k++) {
                const int i = perm[k];
                int32_t qx = int32_t((X[i] - x0) * scale), qy = int32_t((Y[i] - y0) * scale);
                qx = std::min<int32_t>(std::max<int32_t>(qx, 0), 65535);
                qy = std::min<int32_t>(std::max<int32_t>(qy, 0), 65535);
                round[k - lo] = std::make_pair(hilbert_key_2d(qx, qy, 16), i);
            }
            std::sort(round.begin(), round.end());
            for (const auto &o : round) {
                const int rc = insert(o.second);
                if (rc != 0) return rc;
            }
            lo = hi;
        }
        return 0;
    }

    // circumcentre of triangle t: the closed form of the numpy mesh builder
    void circumcentre(int t, double &ux, double &uy) const {
        const Tri &T = tris[t];
        const double ax = px(T.v[0]), ay = py(T.v[0]);
        const double bx = px(T.v[1]) - ax, by = py(T.v[1]) - ay;
        const double cx = px(T.v[2]) - ax, cy = py(T.v[2]) - ay;
        const double d = 2.0 * (bx * cy - by * cx);
        const double b2 = bx * bx + by * by;
        const double c2 = cx * cx + cy * cy;
        ux = ax + (cy * b2 - by * c2) / d;
        uy = ay + (bx * c2 - cx * b2) / d;
    }

    struct Spoke { int j; int t1, t2; };   // neighbour j, triangles on both sides of edge (i, j)

    // the edges around generator i in circulation order; false where i touches the
    // enclosing triangle (an unbounded Voronoi cell)
    bool spokes(int i, std::vector<Spoke> &out) const {
        out.clear();
        const int t0 = vt[i];
        int t = t0;
        for (int guard = 0; guard < 4096; guard++) {
            const Tri &T = tris[t];
            int k = 0;
            while (k < 3 && T.v[k] != i) k++;
            if (k == 3) return false;
            const int b = T.v[(k + 1) % 3];
            const int across = T.n[(k + 2) % 3];
            if (b < 0 || T.v[(k + 2) % 3] < 0 || across < 0) return false;
            out.push_back({b, t, across});
            t = T.n[(k + 1) % 3];
            if (t < 0) return false;
            if (t == t0) return true;
        }
        return false;
    }

    int radius_of(int i, std::vector<Spoke> &sp, double &r) const {
        if (!spokes(i, sp)) { r = -1.; return 1; }
        double m = 0.;
        for (const Spoke &s : sp) {
            double ux, uy;
            circumcentre(s.t1, ux, uy);
            m = std::max(m, (ux - X[i]) * (ux - X[i]) + (uy - Y[i]) * (uy - Y[i]));
        }
        r = 2.0 * std::sqrt(m);
        return 0;
    }
};

namespace {

struct Edge1 {                 // one incident edge of a real cell
    int j;
    double h, ln, fx, fy, xr, yr;
};

// angular order of atan2(y, x) in (-pi, pi]: lower half-plane, the positive x axis,
// upper half-plane, the negative x axis (a signed-zero y there is -pi: first)
inline int angle_class(double x, double y) {
    if (y < 0.) return 1;
    if (y > 0.) return 3;
    if (x >= 0.) return 2;
    return std::signbit(y) ? 0 : 4;
}

inline bool angle_less(double ax, double ay, double bx, double by) {
    const int ca = angle_class(ax, ay), cb = angle_class(bx, by);
    if (ca != cb) return ca < cb;
    return ax * by - ay * bx > 0.;            // same open half-plane: b turns counter-clockwise from a
}

inline int gid_of(const int *gid, int v) { return gid ? gid[v] : v; }

// circumcentre of triangle t with its vertices rotated so the smallest global id comes
// first (the closed form of the numpy mesh builder): the same bits whichever
// triangulation -- the whole box or a strip of it -- holds the triangle
void circumcentre_canon(const phd_tess2d &T, const int *gid, int t, double &ux, double &uy) {
    const Tri &tr = T.tris[t];
    int k0 = 0;
    for (int k = 1; k < 3; k++)
        if (gid_of(gid, tr.v[k]) < gid_of(gid, tr.v[k0])) k0 = k;
    const int va = tr.v[k0], vb = tr.v[(k0 + 1) % 3], vc = tr.v[(k0 + 2) % 3];
    const double ax = T.px(va), ay = T.py(va);
    const double bx = T.px(vb) - ax, by = T.py(vb) - ay;
    const double cx = T.px(vc) - ax, cy = T.py(vc) - ay;
    const double d = 2.0 * (bx * cy - by * cx);
    const double b2 = bx * bx + by * by;
    const double c2 = cx * cx + cy * cy;
    ux = ax + (cy * b2 - by * c2) / d;
    uy = ay + (bx * c2 - cx * b2) / d;
}

struct CCache {                 // circumcentres of one triangulation, formed on first use
    std::vector<double> x, y;
    std::vector<char> done;
    explicit CCache(size_t n) : x(n), y(n), done(n, 0) {}
};

// incident edges of cell i (local id) sorted counter-clockwise from -pi; false if the
// cell is unbounded, or -- when lo < hi are finite bounds -- if a circumcircle of one of
// its triangles reaches outside the x-range [lo, hi] the triangulation's points cover
// (then the triangle may not be Delaunay for the whole point set)
bool cell_edges(const phd_tess2d &T, const int *gid, int i, double lo, double hi, std::vector<phd_tess2d::Spoke> &sp,
                std::vector<Edge1> &E, CCache &C) {
    if (!T.spokes(i, sp)) return false;
    E.clear();
    auto cc = [&](int t, double &ux, double &uy) {
        if (!C.done[t]) {
            circumcentre_canon(T, gid, t, C.x[t], C.y[t]);
            C.done[t] = 1;
        }
        ux = C.x[t];
        uy = C.y[t];
    };
    for (const auto &s : sp) {
        double x1, y1, x2, y2;
        cc(s.t1, x1, y1);
        cc(s.t2, x2, y2);
        if (lo > -INFINITY || hi < INFINITY) {
            const double dx = x1 - T.X[i], dy = y1 - T.Y[i];
            const double R = std::sqrt(dx * dx + dy * dy);
            if (!(x1 - R > lo && x1 + R < hi)) return false;
        }
        Edge1 e;
        e.j = s.j;
        e.xr = T.X[s.j] - T.X[i];
        e.yr = T.Y[s.j] - T.Y[i];
        e.h = std::sqrt(e.xr * e.xr + e.yr * e.yr);
        const double xe = x2 - x1, ye = y2 - y1;
        e.ln = std::sqrt(xe * xe + ye * ye);
        e.fx = 0.5 * (x1 + x2);
        e.fy = 0.5 * (y1 + y2);
        E.push_back(e);
    }
    // the circulation runs counter-clockwise: start it at the smallest angle in (-pi, pi]
    // (atan2's range), so the edges come in ascending angle without computing one
    size_t k0 = 0;
    for (size_t k = 1; k < E.size(); k++)
        if (angle_less(E[k].xr, E[k].yr, E[k0].xr, E[k0].yr)) k0 = k;
    std::rotate(E.begin(), E.begin() + k0, E.end());
    return E.size() >= 3;
}

struct FaceRec {                // a face owned by a real cell, before ghost pruning
    int j;                      // global id of the other cell
    double ln, fx, fy, nx, ny;
};

// faces, volume and centroid offset of the owned real cells (local ids, ascending global
// ids) of one triangulation (extract_geometry): volume / dcom into the global arrays,
// faces appended in cell order, face counts into nf[global id].  False if a cell is
// unbounded or leaves [lo, hi] (see cell_edges).
bool extract_cells(const phd_tess2d &T, const int *gid, const std::vector<int> &owned, double lo, double hi,
                   double *vol, double *dcx, double *dcy, std::vector<FaceRec> &faces, int32_t *nf) {
    std::vector<phd_tess2d::Spoke> sp;
    std::vector<Edge1> E;
    CCache C(T.tris.size());
    faces.clear();
    faces.reserve(3 * owned.size() + 64);
    for (int i : owned) {
        if (!cell_edges(T, gid, i, lo, hi, sp, E, C)) return false;
        const int gi = gid_of(gid, i);
        const double xp = T.X[i], yp = T.Y[i];
        double v = 0., cx = 0., cy = 0.;
        int cnt = 0;
        for (const Edge1 &e : E) {
            const double a = 0.25 * e.ln * e.h;
            const double tx = 2.0 * e.fx / 3.0 + xp / 3.0;
            const double ty = 2.0 * e.fy / 3.0 + yp / 3.0;
            v += a;
            cx += a * tx;
            cy += a * ty;
            const int gj = gid_of(gid, e.j);
            if (gj > gi) {
                faces.push_back({gj, e.ln, e.fx, e.fy, e.xr / e.h, e.yr / e.h});
                cnt++;
            }
        }
        vol[gi] = v;
        dcx[gi] = cx / v - xp;
        dcy[gi] = cy / v - yp;
        nf[gi] = cnt;
    }
    return true;
}

// faces, volumes and centroids of all real cells of one whole triangulation; returns
// the face count or -1.  Face j indices are generator ids (before any ghost pruning).
int extract(const phd_tess2d &T, std::vector<double> &vol, std::vector<double> &dcx, std::vector<double> &dcy,
            std::vector<double> &area, std::vector<double> &comx, std::vector<double> &comy,
            std::vector<double> &nx, std::vector<double> &ny, std::vector<int32_t> &pi, std::vector<int32_t> &pj) {
    const int n = T.n_real;
    std::vector<int> owned(n);
    for (int i = 0; i < n; i++) owned[i] = i;
    vol.assign(n, 0.); dcx.assign(n, 0.); dcy.assign(n, 0.);
    std::vector<int32_t> nf(n, 0);
    std::vector<FaceRec> faces;
    if (!extract_cells(T, nullptr, owned, -INFINITY, INFINITY, vol.data(), dcx.data(), dcy.data(), faces, nf.data()))
        return -1;
    const size_t F = faces.size();
    area.resize(F); comx.resize(F); comy.resize(F); nx.resize(F); ny.resize(F); pi.resize(F); pj.resize(F);
    size_t f = 0;
    for (int i = 0; i < n; i++)
        for (int k = 0; k < nf[i]; k++, f++) {
            const FaceRec &r = faces[f];
            pi[f] = i; pj[f] = r.j; area[f] = r.ln; comx[f] = r.fx; comy[f] = r.fy; nx[f] = r.nx; ny[f] = r.ny;
        }
    return int(F);
}

// per-cell face lists in ascending face id (CSR over n_cells)
void face_lists(int n_cells, const std::vector<int32_t> &pi, const std::vector<int32_t> &pj,
                std::vector<int32_t> &ptr, std::vector<int32_t> &idx) {
    const int F = int(pi.size());
    ptr.assign(n_cells + 1, 0);
    for (int f = 0; f < F; f++) { ptr[pi[f] + 1]++; ptr[pj[f] + 1]++; }
    for (int c = 0; c < n_cells; c++) ptr[c + 1] += ptr[c];
    idx.assign(2 * size_t(F), 0);
    std::vector<int32_t> fill(ptr.begin(), ptr.end() - 1);
    for (int f = 0; f < F; f++) {
        idx[fill[pi[f]]++] = f;
        idx[fill[pj[f]]++] = f;
    }
}

// ghost images of the real generators (the numpy builder's _ghosts)
// Ghost codes (phdtess.h): periodic shift (sx, sy) -> 1 + 3 (sx + 1) + (sy + 1);
// reflective mirror across axis k at its low / high wall -> 16 + 2 k + (high).
void make_ghosts(const double *x, const double *y, int n, int boundary, const double xmin[2], const double xmax[2],
                 double pad, std::vector<double> &gx, std::vector<double> &gy, std::vector<int32_t> &gmap,
                 std::vector<int8_t> &gcode) {
    gx.clear(); gy.clear(); gmap.clear(); gcode.clear();
    const double L0 = xmax[0] - xmin[0], L1 = xmax[1] - xmin[1];
    if (boundary == 0) {
        for (int sx = -1; sx <= 1; sx++)
            for (int sy = -1; sy <= 1; sy++) {
                if (sx == 0 && sy == 0) continue;
                for (int i = 0; i < n; i++) {
                    const double xs = x[i] + double(sx) * L0, ys = y[i] + double(sy) * L1;
                    if (xs > xmin[0] - pad && xs < xmax[0] + pad && ys > xmin[1] - pad && ys < xmax[1] + pad) {
                        gx.push_back(xs); gy.push_back(ys); gmap.push_back(i);
                        gcode.push_back(int8_t(1 + 3 * (sx + 1) + (sy + 1)));
                    }
                }
            }
    } else {
        for (int k = 0; k < 2; k++)
            for (int lo = 1; lo >= 0; lo--) {
                const double edge = lo ? xmin[k] : xmax[k];
                for (int i = 0; i < n; i++) {
                    const double c = k == 0 ? x[i] : y[i];
                    const bool near = lo ? (c - edge < pad) : (edge - c < pad);
                    if (!near) continue;
                    double xs = x[i], ys = y[i];
                    if (k == 0) xs = xs - 2.0 * (xs - edge);
                    else ys = ys - 2.0 * (ys - edge);
                    gx.push_back(xs); gy.push_back(ys); gmap.push_back(i);
                    gcode.push_back(int8_t(16 + 2 * k + (lo ? 0 : 1)));
                }
            }
    }
}

// ---- strip-parallel extraction ------------------------------------------------------
// The box is cut into K strips by the real generators' x quantiles.  Each strip is
// tessellated on its own from every generator (real or ghost) within a halo of it;
// a triangle of that tessellation is a triangle of the whole one when its circumcircle
// lies inside the x-range the strip's points cover (no other generator can then fall in
// it), which extract_cells checks for every triangle around an owned cell -- a strip
// that fails widens its halo (up to every point).  Circumcentres are formed in a
// canonical vertex order, so a face gets the same bits from any strip; K depends only
// on the number of real cells, so the mesh does not depend on the thread count.
int auto_strips(int n_real) { return n_real >= 65536 ? std::min(16, n_real / 32768) : 1; }

struct StripJob {
    double s_lo, s_hi;          // owned x-range [s_lo, s_hi)
    bool first, last;
    std::vector<int> owned;     // global ids, ascending
    std::vector<FaceRec> faces;
};

int strip_pass(StripJob &J, int n_real, const std::vector<double> &ax, const std::vector<double> &ay, double H0,
               double *vol, double *dcx, double *dcy, int32_t *nf) {
    const int n_all = int(ax.size());
    J.owned.clear();                                     // the real cells in [s_lo, s_hi), ascending
    for (int i = 0; i < n_real; i++)
        if (ax[i] >= J.s_lo && ax[i] < J.s_hi) J.owned.push_back(i);
    if (J.owned.empty()) return 0;
    phd_tess2d T;
    std::vector<int> gids;
    std::vector<int> owned_local(J.owned.size());
    for (double H = H0;; H *= 2.0) {
        const double lo = J.first ? -INFINITY : J.s_lo - H;
        const double hi = J.last ? INFINITY : J.s_hi + H;
        gids.clear();                                    // every generator within the halo, ascending
        for (int i = 0; i < n_all; i++)
            if (ax[i] >= lo && ax[i] <= hi) gids.push_back(i);
        const bool whole = (int(gids.size()) == n_all);
        const int m = int(gids.size());
        T.reset();
        T.X.resize(m);
        T.Y.resize(m);
        double x0 = ax[gids[0]], x1 = x0, y0 = ay[gids[0]], y1 = y0;
        for (int k = 0; k < m; k++) {
            T.X[k] = ax[gids[k]];
            T.Y[k] = ay[gids[k]];
            x0 = std::min(x0, T.X[k]); x1 = std::max(x1, T.X[k]);
            y0 = std::min(y0, T.Y[k]); y1 = std::max(y1, T.Y[k]);
        }
        T.inserted.assign(m, 0);
        T.vt.assign(m, -1);
        T.n_total = m;
        T.n_real = 0;
        T.init_super(x0, y0, x1, y1);
        const int rc = T.insert_range(0, m);
        if (rc != 0) return rc;
        size_t q = 0;                                    // owned global ids -> local ids
        for (size_t k = 0; k < J.owned.size(); k++) {
            while (gids[q] != J.owned[k]) q++;
            owned_local[k] = int(q);
        }
        if (extract_cells(T, gids.data(), owned_local, whole ? -INFINITY : lo, whole ? INFINITY : hi, vol, dcx,
                          dcy, J.faces, nf))
            return 0;
        if (whole) return -1;                            // a real cell of the whole box is unbounded
    }
}

// all real cells' faces, volumes and centroid offsets with K strips on up to K threads;
// faces in (cell, angle) order with generator ids; returns the face count or an error
int extract_strips(int K, int n_real, const std::vector<double> &ax, const std::vector<double> &ay, double H0,
                   std::vector<double> &vol, std::vector<double> &dcx, std::vector<double> &dcy,
                   std::vector<double> &area, std::vector<double> &comx, std::vector<double> &comy,
                   std::vector<double> &nx, std::vector<double> &ny, std::vector<int32_t> &pi,
                   std::vector<int32_t> &pj) {
    // strip bounds at x quantiles of a regular sample of the real generators (any bounds
    // give the same mesh; these only balance the strips)
    const int stride = std::max(1, n_real / 65536);
    std::vector<double> xr;
    for (int i = 0; i < n_real; i += stride) xr.push_back(ax[i]);
    std::sort(xr.begin(), xr.end());
    const size_t ns = xr.size();
    std::vector<StripJob> jobs(K);
    for (int k = 0; k < K; k++) {
        jobs[k].s_lo = k == 0 ? -INFINITY : xr[size_t(k) * ns / K];
        jobs[k].s_hi = k == K - 1 ? INFINITY : xr[size_t(k + 1) * ns / K];
        jobs[k].first = k == 0;
        jobs[k].last = k == K - 1;
    }
    vol.assign(n_real, 0.); dcx.assign(n_real, 0.); dcy.assign(n_real, 0.);
    std::vector<int32_t> nf(n_real, 0);
    std::atomic<int> next(0), status(0);
    auto worker = [&]() {
        for (;;) {
            const int k = next.fetch_add(1);
            if (k >= K) return;
            int rc;
            try {
                rc = strip_pass(jobs[k], n_real, ax, ay, H0, vol.data(), dcx.data(), dcy.data(), nf.data());
            } catch (...) {
                rc = -4;
            }
            if (rc != 0) {
                int expected = 0;
                status.compare_exchange_strong(expected, rc);
            }
        }
    };
    const unsigned hw = std::max(1u, std::thread::hardware_concurrency());
    const int n_threads = std::min<int>(K, int(hw));
    std::vector<std::thread> threads;
    for (int t = 1; t < n_threads; t++) threads.emplace_back(worker);
    worker();
    for (auto &th : threads) th.join();
    if (status.load() != 0) return status.load();
    std::vector<int64_t> off(size_t(n_real) + 1, 0);
    for (int i = 0; i < n_real; i++) off[i + 1] = off[i] + nf[i];
    const size_t F = size_t(off[n_real]);
    area.resize(F); comx.resize(F); comy.resize(F); nx.resize(F); ny.resize(F); pi.resize(F); pj.resize(F);
    std::atomic<int> next_copy(0);
    auto copier = [&]() {                               // each strip fills its own cells' face ranges
        for (;;) {
            const int k = next_copy.fetch_add(1);
            if (k >= K) return;
            const StripJob &J = jobs[k];
            size_t r = 0;
            for (int gi : J.owned)
                for (int64_t f = off[gi]; f < off[gi + 1]; f++, r++) {
                    const FaceRec &rec = J.faces[r];
                    pi[f] = gi; pj[f] = rec.j; area[f] = rec.ln; comx[f] = rec.fx; comy[f] = rec.fy;
                    nx[f] = rec.nx; ny[f] = rec.ny;
                }
        }
    };
    threads.clear();
    for (int t = 1; t < n_threads; t++) threads.emplace_back(copier);
    copier();
    for (auto &th : threads) th.join();
    return int(F);
}

}  // namespace

extern "C" {

phd_tess2d *phd_tess2d_create(void) { return new (std::nothrow) phd_tess2d(); }

void phd_tess2d_destroy(phd_tess2d *t) { delete t; }

int phd_tess2d_build_initial(phd_tess2d *t, const double *x, const double *y, int n_real, double *radius) {
    if (!t || !x || !y || n_real < 3) return -2;
    try {
        t->reset();
        t->X.assign(x, x + n_real);
        t->Y.assign(y, y + n_real);
        t->inserted.assign(n_real, 0);
        t->vt.assign(n_real, -1);
        t->n_real = t->n_total = n_real;
        double x0 = x[0], x1 = x[0], y0 = y[0], y1 = y[0];
        for (int i = 0; i < n_real; i++) {
            if (!std::isfinite(x[i]) || !std::isfinite(y[i])) return -2;
            x0 = std::min(x0, x[i]); x1 = std::max(x1, x[i]);
            y0 = std::min(y0, y[i]); y1 = std::max(y1, y[i]);
        }
        t->init_super(x0, y0, x1, y1);
        const int rc = t->insert_range(0, n_real);
        if (rc != 0) return rc;
        if (radius) {
            std::vector<phd_tess2d::Spoke> sp;
            for (int i = 0; i < n_real; i++) t->radius_of(i, sp, radius[i]);
        }
        return 0;
    } catch (...) {
        return -4;
    }
}

int phd_tess2d_update_initial(phd_tess2d *t, const double *x, const double *y, int begin, int end) {
    if (!t || !x || !y || begin != t->n_total || end < begin) return -2;
    if (begin == end) return 0;
    try {
        for (int i = begin; i < end; i++) {
            if (!std::isfinite(x[i]) || !std::isfinite(y[i])) return -2;
            // the enclosing triangle is sized for the real generators' box: far ghosts
            // would fall outside it
            const double cx = 0.5 * (t->SX[0] + t->SX[1]);
            if (std::fabs(x[i] - cx) > 0.25 * (t->SX[1] - t->SX[0]) ||
                std::fabs(y[i] - t->SY[0]) > 0.5 * (t->SY[2] - t->SY[0]))
                return -2;
        }
        t->X.insert(t->X.end(), x + begin, x + end);
        t->Y.insert(t->Y.end(), y + begin, y + end);
        t->inserted.resize(end, 0);
        t->vt.resize(end, -1);
        t->n_total = end;
        return t->insert_range(begin, end);
    } catch (...) {
        return -4;
    }
}

int phd_tess2d_count_faces(phd_tess2d *t) {
    if (!t || t->n_real == 0) return -2;
    std::vector<phd_tess2d::Spoke> sp;
    int F = 0;
    for (int i = 0; i < t->n_real; i++) {
        if (!t->spokes(i, sp)) return -1;
        for (const auto &s : sp) F += s.j > i;
    }
    return F;
}

int phd_tess2d_update_radius(phd_tess2d *t, const int32_t *ids, int n_ids, double *radius) {
    if (!t || (n_ids > 0 && (!ids || !radius))) return -2;
    std::vector<phd_tess2d::Spoke> sp;
    int open = 0;
    for (int k = 0; k < n_ids; k++) {
        const int i = ids[k];
        if (i < 0 || i >= t->n_total) return -2;
        open += t->radius_of(i, sp, radius[i]);
    }
    return open;
}

int phd_tess2d_extract_geometry(phd_tess2d *t, double *dcom_x, double *dcom_y, double *volume, double *face_area,
                                double *com_x, double *com_y, double *normal_x, double *normal_y, int32_t *pair_i,
                                int32_t *pair_j, int32_t *nbr_ptr, int32_t *nbr_idx) {
    if (!t || t->n_real == 0) return -2;
    try {
        std::vector<double> vol, dcx, dcy, area, comx, comy, nx, ny;
        std::vector<int32_t> pi, pj, ptr, idx;
        const int F = extract(*t, vol, dcx, dcy, area, comx, comy, nx, ny, pi, pj);
        if (F < 0) return F;
        face_lists(t->n_total, pi, pj, ptr, idx);
        auto put = [](const auto &v, auto *dst) { if (dst && !v.empty()) std::memcpy(dst, v.data(), v.size() * sizeof(v[0])); };
        put(dcx, dcom_x); put(dcy, dcom_y); put(vol, volume); put(area, face_area);
        put(comx, com_x); put(comy, com_y); put(nx, normal_x); put(ny, normal_y);
        put(pi, pair_i); put(pj, pair_j); put(ptr, nbr_ptr); put(idx, nbr_idx);
        return F;
    } catch (...) {
        return -4;
    }
}

int phd_mesh2d_build(phd_tess2d *t, const double *x, const double *y, int n_real, int boundary, double xmin0,
                     double xmin1, double xmax0, double xmax1, double pad) {
    return phd_mesh2d_build_strips(t, x, y, n_real, boundary, xmin0, xmin1, xmax0, xmax1, pad, 0);
}

int phd_mesh2d_build_strips(phd_tess2d *t, const double *x, const double *y, int n_real, int boundary,
                            double xmin0, double xmin1, double xmax0, double xmax1, double pad, int n_strips) {
    if (!t || !x || !y || n_real < 3 || (boundary != 0 && boundary != 1) || !(xmax0 > xmin0) ||
        !(xmax1 > xmin1) || !(pad > 0.) || n_strips < 0 || n_strips > 256)
        return -2;
    const int K = n_strips ? std::min(n_strips, std::max(1, n_real / 64)) : auto_strips(n_real);
    const double xmin[2] = {xmin0, xmin1}, xmax[2] = {xmax0, xmax1};
    try {
        std::vector<double> gx, gy, ax, ay;
        std::vector<int32_t> gmap;
        std::vector<int8_t> gcode;
        for (int attempt = 0; attempt < 6; attempt++, pad *= 2.0) {
            make_ghosts(x, y, n_real, boundary, xmin, xmax, pad, gx, gy, gmap, gcode);
            const int n_all = n_real + int(gx.size());
            ax.assign(x, x + n_real);
            ax.insert(ax.end(), gx.begin(), gx.end());
            ay.assign(y, y + n_real);
            ay.insert(ay.end(), gy.begin(), gy.end());
            double x0 = ax[0], x1 = ax[0], y0 = ay[0], y1 = ay[0];
            for (int i = 0; i < n_all; i++) {
                if (!std::isfinite(ax[i]) || !std::isfinite(ay[i])) return -2;
                x0 = std::min(x0, ax[i]); x1 = std::max(x1, ax[i]);
                y0 = std::min(y0, ay[i]); y1 = std::max(y1, ay[i]);
            }
            Geometry &G = t->G;
            std::vector<double> vol, dcx, dcy;
            int F;
            if (K > 1) {
                t->reset();
                const double H0 = 4.0 * std::sqrt((xmax0 - xmin0) * (xmax1 - xmin1) / double(n_real));
                F = extract_strips(K, n_real, ax, ay, H0, vol, dcx, dcy, G.area, G.comx, G.comy, G.nx, G.ny,
                                   G.pair_i, G.pair_j);
            } else {
                t->reset();
                t->X = ax;
                t->Y = ay;
                t->inserted.assign(n_all, 0);
                t->vt.assign(n_all, -1);
                t->n_real = n_real;
                t->n_total = n_all;
                t->init_super(x0, y0, x1, y1);
                int rc;
                if ((rc = t->insert_range(0, n_real)) != 0) return rc;
                if ((rc = t->insert_range(n_real, n_all)) != 0) return rc;
                F = extract(*t, vol, dcx, dcy, G.area, G.comx, G.comy, G.nx, G.ny, G.pair_i, G.pair_j);
            }
            if (F == -1) continue;                         // a real cell is unbounded: wider pad
            if (F < 0) return F;
            // keep ghosts that share a face with a real cell, in creation order
            std::vector<char> used(n_all, 0);
            for (int f = 0; f < F; f++) used[G.pair_j[f]] = 1;
            std::vector<int32_t> newidx(n_all, -1);
            for (int i = 0; i < n_real; i++) newidx[i] = i;
            int nc = n_real;
            for (int g = n_real; g < n_all; g++)
                if (used[g]) newidx[g] = nc++;
            for (int f = 0; f < F; f++) G.pair_j[f] = newidx[G.pair_j[f]];
            G.n_real = n_real;
            G.n_cells = nc;
            G.n_faces = F;
            G.pad_used = pad;
            G.x.resize(nc); G.y.resize(nc); G.map.resize(nc); G.vol.resize(nc); G.dcx.resize(nc); G.dcy.resize(nc);
            G.gcode.assign(nc - n_real, 0);
            for (int i = 0; i < n_real; i++) {
                G.x[i] = x[i]; G.y[i] = y[i]; G.map[i] = i;
                G.vol[i] = vol[i]; G.dcx[i] = dcx[i]; G.dcy[i] = dcy[i];
            }
            for (int g = n_real; g < n_all; g++) {
                const int c = newidx[g];
                if (c < 0) continue;
                const int img = gmap[g - n_real];
                G.x[c] = ax[g]; G.y[c] = ay[g]; G.map[c] = img;
                G.gcode[c - n_real] = gcode[g - n_real];
                G.vol[c] = vol[img]; G.dcx[c] = dcx[img]; G.dcy[c] = dcy[img];
            }
            face_lists(nc, G.pair_i, G.pair_j, G.nbr_ptr, G.nbr_idx);
            return F;
        }
        return -1;
    } catch (...) {
        return -4;
    }
}

int phd_mesh2d_sizes(const phd_tess2d *t, int32_t *n_cells, int32_t *n_faces, double *pad_used) {
    if (!t) return -2;
    if (n_cells) *n_cells = t->G.n_cells;
    if (n_faces) *n_faces = t->G.n_faces;
    if (pad_used) *pad_used = t->G.pad_used;
    return 0;
}

int phd_mesh2d_copy(const phd_tess2d *t, double *x, double *y, int32_t *map, double *vol, double *dcom_x,
                    double *dcom_y, int32_t *pair_i, int32_t *pair_j, double *area, double *com_x, double *com_y,
                    double *normal_x, double *normal_y, int32_t *nbr_ptr, int32_t *nbr_idx) {
    if (!t || t->G.n_cells == 0) return -2;
    const Geometry &G = t->G;
    auto put = [](const auto &v, auto *dst) { if (dst && !v.empty()) std::memcpy(dst, v.data(), v.size() * sizeof(v[0])); };
    put(G.x, x); put(G.y, y); put(G.map, map); put(G.vol, vol); put(G.dcx, dcom_x); put(G.dcy, dcom_y);
    put(G.pair_i, pair_i); put(G.pair_j, pair_j); put(G.area, area); put(G.comx, com_x); put(G.comy, com_y);
    put(G.nx, normal_x); put(G.ny, normal_y); put(G.nbr_ptr, nbr_ptr); put(G.nbr_idx, nbr_idx);
    return 0;
}

// pair_j, or (pair_j == NULL) pair_dj + pair_x[2 x_cap] with *n_pair_x escapes
static int copy_compact(const phd_tess2d *t, int32_t *face_ptr, int32_t *pair_j, uint16_t *pair_dj, int32_t *pair_x,
                        int32_t x_cap, int32_t *n_pair_x, float *area32, float *ct32, int stride, double *x,
                        int32_t *map, int8_t *tag, int8_t *type, int8_t *ghost_code) {
    const Geometry &G = t->G;
    const int nr = G.n_real, n = G.n_cells, F = G.n_faces;
    // FP64 -> FP32, round to nearest even; magnitudes below 2^-126 to signed zero (the
    // device's own rounding of the same quantities)
    auto round32 = [](double v) -> float {
        return std::fabs(v) < 1.1754943508222875e-38 ? std::copysign(0.0f, float(v)) : float(v);
    };
    int c = 0;
    face_ptr[0] = 0;
    for (int f = 0; f < F; f++) {
        const int i = G.pair_i[f], j = G.pair_j[f];
        while (c < i) face_ptr[++c] = f;
        if (pair_j) {
            pair_j[f] = j;
        } else {
            const int64_t d = int64_t(j) - int64_t(i);
            if (d >= 1 && d <= 65534) {
                pair_dj[f] = uint16_t(d);
            } else {
                pair_dj[f] = PHD_PAIR16_ESCAPE;
                if (*n_pair_x < x_cap) {
                    pair_x[2 * *n_pair_x] = f;
                    pair_x[2 * *n_pair_x + 1] = j;
                }
                ++*n_pair_x;
            }
        }
        area32[(size_t)f * stride] = round32(G.area[f]);
        // the centroid offset along the face (phdflux.h, compact hand-over): built with
        // -ffp-contract=off, so every operation rounds as the device's does
        const double dx = G.x[j] - G.x[i], dy = G.y[j] - G.y[i];
        const double cx = G.comx[f] - 0.5 * (G.x[i] + G.x[j]), cy = G.comy[f] - 0.5 * (G.y[i] + G.y[j]);
        const double r = std::sqrt(dx * dx + dy * dy);
        ct32[(size_t)f * stride] = round32(r > 0.0 ? (cx * (-dy) + cy * dx) / r : 0.0);
    }
    while (c < nr) face_ptr[++c] = F;
    if (x) {
        std::memcpy(x, G.x.data(), sizeof(double) * n);
        std::memcpy(x + n, G.y.data(), sizeof(double) * n);
    }
    if (ghost_code && n > nr) std::memcpy(ghost_code, G.gcode.data(), sizeof(int8_t) * (n - nr));
    std::memcpy(map, G.map.data(), sizeof(int32_t) * n);
    for (int k = 0; k < n; k++) {
        tag[k] = k < nr ? 0 : 1;                        // Real / Ghost (particle_tags.py:1-6)
        type[k] = k < nr ? 4 : 2;                       // Undefined / Exterior
    }
    return (n_pair_x && *n_pair_x > x_cap) ? -5 : 0;
}

int phd_mesh2d_copy_compact(const phd_tess2d *t, int32_t *face_ptr, int32_t *pair_j, float *area32, float *ct32,
                            double *x, int32_t *map, int8_t *tag, int8_t *type, int8_t *ghost_code) {
    if (!t || t->G.n_cells == 0 || !face_ptr || !pair_j || !area32 || !ct32 || !map || !tag || !type)
        return -2;
    return copy_compact(t, face_ptr, pair_j, nullptr, nullptr, 0, nullptr, area32, ct32, 1, x, map, tag, type,
                        ghost_code);
}

int phd_mesh2d_copy_compact16(const phd_tess2d *t, int32_t *face_ptr, uint16_t *pair_dj, int32_t *pair_x,
                              int32_t x_cap, int32_t *n_pair_x, uint8_t *list_len, float *face32, double *x,
                              int32_t *map, int8_t *tag, int8_t *type, int8_t *ghost_code) {
    if (!t || t->G.n_cells == 0 || !face_ptr || !pair_dj || !n_pair_x || x_cap < 0 || (x_cap > 0 && !pair_x) ||
        !face32 || !map || !tag || !type)
        return -2;
    *n_pair_x = 0;
    const int rc = copy_compact(t, face_ptr, nullptr, pair_dj, pair_x, x_cap, n_pair_x, face32, face32 + 1, 2, x, map,
                                tag, type, ghost_code);
    if (rc < 0 || !list_len) return rc;
    // each face adds one entry to the lists of both its cells (tess.cpp:378-379)
    const Geometry &G = t->G;
    std::vector<int32_t> len(G.n_cells, 0);
    for (int f = 0; f < G.n_faces; f++) {
        len[G.pair_i[f]]++;
        len[G.pair_j[f]]++;
    }
    bool fits = true;
    for (int c = 0; c < G.n_cells; c++) {
        fits = fits && len[c] <= 255;
        list_len[c] = uint8_t(len[c] <= 255 ? len[c] : 255);
    }
    return fits ? 0 : -6;
}

void phd_hilbert_keys_2d_host(const int32_t *xh, const int32_t *yh, int64_t n, int order, int64_t *keys) {
    for (int64_t i = 0; i < n; i++) keys[i] = hilbert_key_2d(xh[i], yh[i], order);
}

}  // extern "C"
