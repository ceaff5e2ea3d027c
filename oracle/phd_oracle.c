/*
 * phd_oracle.c -- CPU restatement of the reference's per-step flux path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the parity checker for the CUDA path: it
 * is compiled into oracle/libphd_oracle.so and called from tests/, from
 * __graft_entry__.smoke() and from bench.py's CPU-baseline leg.  The product path
 * never links or calls it.
 *
 * Every function restates one routine of rickyfernandez/phd-code in FP64 with the
 * reference's operation order (the Cython sources lower Python expressions with
 * their parse-tree grouping).  Squares: where the reference's typed Cython emits a
 * C-level pow(x, 2.0) the compiler folds it into the product x*x, here as there; the
 * face-velocity residual (mesh.pyx:472) squares through Python's float power on boxed
 * operands, i.e. libm pow at run time, which can differ from x*x by an ulp -- that one
 * calls libm through a pointer the compiler cannot fold (py_pow).  Build with
 * -ffp-contract=off so no multiply-add is fused.
 *
 * Layout: structure-of-arrays, row-major [field][index]:
 *   prim  [dim+2][n]  density, velocity-x..., pressure     (particle_creator.pyx:50-55)
 *   cons  [dim+2][n]  mass, momentum-x..., energy          (particle_creator.pyx:56-58)
 *   grad  [(dim+2)*dim][n]  grad[f*dim+k] = d prim_f / d x_k (reconstruction.pyx:470-484)
 *   states/fluxes [dim+2][F] in the same field order as prim / cons.
 */
#include <math.h>
#include <stdint.h>
#include <string.h>
#include <stdlib.h>

#include "phd_oracle.h"

#define REAL_TAG 0       /* particle_tags.py:2 */
#define EXTERIOR_TYPE 2  /* particle_tags.py:4 */
#define PI_D 3.141592653589793

#define X(a, k, i, n) ((a)[(size_t)(k) * (size_t)(n) + (size_t)(i)])

/* ---------------------------------------------------------------------------
 * PieceWiseLinear.compute_gradients  reconstruction.pyx:563-739
 * + DomainManager.update_ghost_gradients (serial) domain_manager.pyx:819-835
 * + Reflective.update_gradients boundary.pyx:265-307
 * ------------------------------------------------------------------------- */
int orc_compute_gradients(const orc_mesh *M, const double *prim, int limiter, double *grad)
{
    const int dim = M->dim, nf = dim + 2, n = M->n_cells, F = M->n_faces;
    double phi_max[5], phi_min[5], alpha[5], df[15];
    double xi[3], xj[3], cx[3], cfx[3], dr[3];
    int status = 0;

    for (int i = 0; i < n; i++) {
        if (M->tag[i] != REAL_TAG) continue;
        for (int k = 0; k < dim; k++) {
            xi[k] = X(M->x, k, i, n);
            cx[k] = xi[k] + X(M->dcom, k, i, n);
        }
        const double vol = M->vol[i];
        for (int f = 0; f < nf; f++) {
            phi_max[f] = phi_min[f] = X(prim, f, i, n);
            alpha[f] = 1.0;
            for (int k = 0; k < dim; k++) df[dim * f + k] = 0;
        }
        for (int m = M->nbr_ptr[i]; m < M->nbr_ptr[i + 1]; m++) {
            const int fid = M->nbr_idx[m];
            const double area = M->area[fid];
            int j;
            if (i == M->pair_i[fid]) j = M->pair_j[fid];
            else if (i == M->pair_j[fid]) j = M->pair_i[fid];
            else { status |= ORC_BAD_INDEX; continue; }   /* "incorrect neighbors" */
            double r = 0.0;
            for (int k = 0; k < dim; k++) {
                xj[k] = X(M->x, k, j, n);
                cfx[k] = X(M->com, k, fid, F) - 0.5 * (xi[k] + xj[k]);
                dr[k] = xi[k] - xj[k];
                r = r + pow(dr[k], 2.0);
            }
            r = sqrt(r);
            for (int f = 0; f < nf; f++) {
                const double pj = X(prim, f, j, n), pi_ = X(prim, f, i, n);
                phi_max[f] = fmax(phi_max[f], pj);
                phi_min[f] = fmin(phi_min[f], pj);
                const double d_dif = pj - pi_;
                const double d_sum = pj + pi_;
                for (int k = 0; k < dim; k++)
                    df[dim * f + k] = df[dim * f + k] +
                        (area * ((d_dif * cfx[k]) - ((0.5 * d_sum) * dr[k]))) / (r * vol);
            }
        }
        if (limiter == 0) {                       /* AREPO, Eq. 30, :683-703 */
            for (int f = 0; f < nf; f++) {
                for (int m = M->nbr_ptr[i]; m < M->nbr_ptr[i + 1]; m++) {
                    const int fid = M->nbr_idx[m];
                    double dphi = 0.0, psi;
                    for (int k = 0; k < dim; k++)
                        dphi = dphi + df[dim * f + k] * (X(M->com, k, fid, F) - cx[k]);
                    if (dphi > 0) psi = (phi_max[f] - X(prim, f, i, n)) / dphi;
                    else if (dphi < 0) psi = (phi_min[f] - X(prim, f, i, n)) / dphi;
                    else psi = 1.0;
                    alpha[f] = fmin(alpha[f], fmax(psi, 0.));
                }
            }
        } else if (limiter == 1) {                /* TESS, Eq. 22, :705-731 */
            for (int f = 0; f < nf; f++) {
                int j = i;
                for (int m = M->nbr_ptr[i]; m < M->nbr_ptr[i + 1]; m++) {
                    const int fid = M->nbr_idx[m];
                    if (i == M->pair_i[fid]) j = M->pair_j[fid];
                    else if (i == M->pair_j[fid]) j = M->pair_i[fid];
                    double dphi = 0.0, psi;
                    for (int k = 0; k < dim; k++)
                        dphi = dphi + df[dim * f + k] * (X(M->com, k, fid, F) - cx[k]);
                    if (dphi > 0.0 || dphi < 0.0) {
                        const double t = (X(prim, f, j, n) - X(prim, f, i, n)) / dphi;
                        psi = (0. > t) ? 0. : t;
                    } else psi = 1.0;
                    alpha[0] = fmin(alpha[0], fmax(psi, 0.));   /* only alpha[0], :731 */
                }
            }
        }
        for (int f = 0; f < nf; f++)
            for (int k = 0; k < dim; k++)
                X(grad, dim * f + k, i, n) = alpha[f] * df[dim * f + k];
    }

    /* ghosts take their image's gradient (domain_manager.pyx:819-835) ... */
    for (int i = 0; i < n; i++) {
        if (M->tag[i] == REAL_TAG) continue;
        const int im = M->map[i];
        for (int r = 0; r < nf * dim; r++) X(grad, r, i, n) = X(grad, r, im, n);
    }
    /* ... then reflective walls flip the normal diagonal of grad v (boundary.pyx:287-307) */
    if (M->reflective) {
        for (int i = 0; i < n; i++) {
            if (M->type[i] != EXTERIOR_TYPE) continue;
            for (int j = 0; j < dim; j++) {
                const int row = dim * (1 + j) + j;
                if (X(M->x, j, i, n) < M->xmin[j]) X(grad, row, i, n) *= -1;
                if (X(M->x, j, i, n) > M->xmax[j]) X(grad, row, i, n) *= -1;
            }
        }
    }
    return status;
}

/* PieceWiseConstant.compute_states  reconstruction.pyx:254-353 */
void orc_pwc_states(const orc_mesh *M, const double *prim, const double *face_w, int boost,
                    double *left, double *right)
{
    const int dim = M->dim, n = M->n_cells, F = M->n_faces;
    for (int m = 0; m < F; m++) {
        const int i = M->pair_i[m], j = M->pair_j[m];
        X(left, 0, m, F) = X(prim, 0, i, n);
        X(right, 0, m, F) = X(prim, 0, j, n);
        X(left, dim + 1, m, F) = X(prim, dim + 1, i, n);
        X(right, dim + 1, m, F) = X(prim, dim + 1, j, n);
        for (int k = 0; k < dim; k++) {
            if (boost) {
                X(left, 1 + k, m, F) = X(prim, 1 + k, i, n) - X(face_w, k, m, F);
                X(right, 1 + k, m, F) = X(prim, 1 + k, j, n) - X(face_w, k, m, F);
            } else {
                X(left, 1 + k, m, F) = X(prim, 1 + k, i, n);
                X(right, 1 + k, m, F) = X(prim, 1 + k, j, n);
            }
        }
    }
}

/* PieceWiseLinear.add_spatial  reconstruction.pyx:741-921 */
void orc_add_spatial(const orc_mesh *M, const double *prim, const double *grad,
                     const double *face_w, int boost, int gizmo, double *left, double *right)
{
    const int dim = M->dim, nf = dim + 2, n = M->n_cells, F = M->n_faces;
    const double psi1 = 0.5, psi2 = 0.25;
    double sl[5], sr[5];
    for (int m = 0; m < F; m++) {
        const int i = M->pair_i[m], j = M->pair_j[m];
        for (int f = 0; f < nf; f++) {
            X(left, f, m, F) = X(prim, f, i, n);
            X(right, f, m, F) = X(prim, f, j, n);
        }
        for (int k = 0; k < dim; k++) {
            if (boost) {
                X(left, 1 + k, m, F) = X(prim, 1 + k, i, n) - X(face_w, k, m, F);
                X(right, 1 + k, m, F) = X(prim, 1 + k, j, n) - X(face_w, k, m, F);
            }
        }
        for (int f = 0; f < nf; f++) {
            sl[f] = X(left, f, m, F);
            sr[f] = X(right, f, m, F);
        }
        double diff_mag = 0.0, sepi_mag = 0.0, sepj_mag = 0.0;
        for (int k = 0; k < dim; k++) {
            const double sepi = X(M->com, k, m, F) - (X(M->x, k, i, n) + X(M->dcom, k, i, n));
            const double sepj = X(M->com, k, m, F) - (X(M->x, k, j, n) + X(M->dcom, k, j, n));
            sepi_mag = sepi_mag + sepi * sepi;
            sepj_mag = sepj_mag + sepj * sepj;
            diff_mag = diff_mag + pow(X(M->x, k, j, n) - X(M->x, k, i, n), 2.0);
            for (int f = 0; f < nf; f++) {
                X(left, f, m, F) = X(left, f, m, F) + X(grad, f * dim + k, i, n) * sepi;
                X(right, f, m, F) = X(right, f, m, F) + X(grad, f * dim + k, j, n) * sepj;
            }
        }
        sepi_mag = sqrt(sepi_mag);
        sepj_mag = sqrt(sepj_mag);
        diff_mag = sqrt(diff_mag);
        if (gizmo) {                                  /* GIZMO appendix B4, :877-921 */
            for (int f = 0; f < nf; f++) {
                const double delta1 = psi1 * fabs(sl[f] - sr[f]);
                const double delta2 = psi2 * fabs(sl[f] - sr[f]);
                const double phi_min = fmin(sl[f], sr[f]);
                const double phi_max = fmax(sl[f], sr[f]);
                const double phibar_l = sl[f] + ((sepi_mag / diff_mag) * (sr[f] - sl[f]));
                const double phibar_r = sr[f] + ((sepj_mag / diff_mag) * (sl[f] - sr[f]));
                double phi_plus, phi_minus;
                if (((phi_max + delta1) * phi_max) >= 0.) phi_plus = phi_max + delta1;
                else phi_plus = phi_max / (1 + (delta1 / fabs(phi_max)));
                if (((phi_min - delta1) * phi_min) >= 0.) phi_minus = phi_min - delta1;
                else phi_minus = phi_min / (1 + (delta1 / fabs(phi_min)));
                const double ci = X(prim, f, i, n), cj = X(prim, f, j, n);
                if (ci < cj) {
                    X(left, f, m, F) = fmax(phi_minus, fmin(phibar_l + delta2, X(left, f, m, F)));
                    X(right, f, m, F) = fmin(phi_plus, fmax(phibar_r - delta2, X(right, f, m, F)));
                } else if (ci > cj) {
                    X(left, f, m, F) = fmin(phi_plus, fmax(phibar_l - delta2, X(left, f, m, F)));
                    X(right, f, m, F) = fmax(phi_minus, fmin(phibar_r + delta2, X(right, f, m, F)));
                } else {
                    X(left, f, m, F) = sl[f];
                    X(right, f, m, F) = sr[f];
                }
            }
            if (X(left, 0, m, F) < 0.0 || X(left, dim + 1, m, F) < 0.0)
                for (int f = 0; f < nf; f++) X(left, f, m, F) = sl[f];
            if (X(right, 0, m, F) < 0.0 || X(right, dim + 1, m, F) < 0.0)
                for (int f = 0; f < nf; f++) X(right, f, m, F) = sr[f];
        }
    }
}

/* PieceWiseLinear.add_temporal  reconstruction.pyx:923-1072 (dt is the half step) */
void orc_add_temporal(const orc_mesh *M, const double *prim, const double *grad,
                      const double *face_w, double gamma, double dt, int boost,
                      double *left, double *right)
{
    const int dim = M->dim, nf = dim + 2, n = M->n_cells, F = M->n_faces;
    double sl[5], sr[5], vi[3], vj[3];
#define DD(k, c) X(grad, 0 * dim + (k), c, n)
#define DV(r, c) X(grad, dim + (r), c, n)           /* dv[r] = d v_(r/dim) / d x_(r%dim) */
#define DP(k, c) X(grad, (dim + 1) * dim + (k), c, n)
    for (int m = 0; m < F; m++) {
        const int i = M->pair_i[m], j = M->pair_j[m];
        for (int f = 0; f < nf; f++) {
            sl[f] = X(left, f, m, F);
            sr[f] = X(right, f, m, F);
        }
        const double di = X(prim, 0, i, n), dj = X(prim, 0, j, n);
        const double pi_ = X(prim, dim + 1, i, n), pj = X(prim, dim + 1, j, n);
        for (int k = 0; k < dim; k++) {
            if (boost) {
                vi[k] = X(prim, 1 + k, i, n) - X(face_w, k, m, F);
                vj[k] = X(prim, 1 + k, j, n) - X(face_w, k, m, F);
            } else {
                vi[k] = X(prim, 1 + k, i, n);
                vj[k] = X(prim, 1 + k, j, n);
            }
            X(left, 1 + k, m, F) = X(left, 1 + k, m, F) - ((dt * DP(k, i)) / di);
            X(right, 1 + k, m, F) = X(right, 1 + k, m, F) - ((dt * DP(k, j)) / dj);
        }
        for (int k = 0; k < dim; k++) {
            X(left, 0, m, F) = X(left, 0, m, F) - (dt * ((di * DV((dim + 1) * k, i)) + (vi[k] * DD(k, i))));
            X(right, 0, m, F) = X(right, 0, m, F) - (dt * ((dj * DV((dim + 1) * k, j)) + (vj[k] * DD(k, j))));
            X(left, dim + 1, m, F) = X(left, dim + 1, m, F) -
                (dt * (((gamma * pi_) * DV((dim + 1) * k, i)) + (vi[k] * DP(k, i))));
            X(right, dim + 1, m, F) = X(right, dim + 1, m, F) -
                (dt * (((gamma * pj) * DV((dim + 1) * k, j)) + (vj[k] * DP(k, j))));
            for (int c = 0; c < dim; c++) {
                X(left, 1 + c, m, F) = X(left, 1 + c, m, F) - ((dt * vi[k]) * DV(c * dim + k, i));
                X(right, 1 + c, m, F) = X(right, 1 + c, m, F) - ((dt * vj[k]) * DV(c * dim + k, j));
            }
        }
        if (X(left, 0, m, F) < 0.0 || X(left, dim + 1, m, F) < 0.0)
            for (int f = 0; f < nf; f++) X(left, f, m, F) = sl[f];
        if (X(right, 0, m, F) < 0.0 || X(right, dim + 1, m, F) < 0.0)
            for (int f = 0; f < nf; f++) X(right, f, m, F) = sr[f];
    }
#undef DD
#undef DV
#undef DP
}

/* HLL.get_waves  riemann.pyx:375-504 */
static void get_waves(double dl, double ul, double pl, double dr, double ur, double pr,
                      double gamma, double *sl, double *sc, double *sr)
{
    const double Q = 2., c_floor = 1.0E-10;
    double p_star, u_star;
    const double cl = fmax(sqrt((gamma * pl) / dl), c_floor);
    const double cr = fmax(sqrt((gamma * pr) / dr), c_floor);
    const double d_avg = .5 * (dl + dr);
    const double c_avg = .5 * (cl + cr);
    p_star = fmax(0., ((.5 * (pl + pr)) + (((.5 * (ul - ur)) * d_avg) * c_avg)));
    const double p_min = fmin(pl, pr);
    const double p_max = fmax(pl, pr);
    if (((p_max / p_min) < Q) && ((p_min < p_star) && (p_star < p_max))) {
        u_star = (.5 * (ul + ur)) + ((.5 * (pl - pr)) / (d_avg * c_avg));
    } else if (p_star <= p_min) {
        const double z = (gamma - 1.) / (2. * gamma);
        const double plr = pow(pl / pr, z);
        u_star = ((((plr * ul) / cl) + (ur / cr)) + ((2. * (plr - 1.)) / (gamma - 1.))) /
                 ((plr / cl) + (1. / cr));
        p_star = (.5 * pl) * pow((1. + (((gamma - 1.) * (ul - u_star)) / (2. * cl))), (1. / z));
        p_star = p_star + ((.5 * pr) * pow((1. + (((gamma - 1.) * (u_star - ur)) / (2. * cr))), (1. / z)));
    } else {
        const double Al = 2. / ((gamma + 1.) * dl);
        const double Ar = 2. / ((gamma + 1.) * dr);
        const double Bl = pl * ((gamma - 1.) / (gamma + 1.));
        const double Br = pr * ((gamma - 1.) / (gamma + 1.));
        const double gl = sqrt(Al / (p_star + Bl));
        const double gr = sqrt(Ar / (p_star + Br));
        p_star = (((gl * pl) + (gr * pr)) - (ur - ul)) / (gl + gr);
        u_star = (.5 * (ul + ur)) + (.5 * ((gr * (p_star - pr)) - (gl * (p_star - pl))));
    }
    (void)u_star;
    double _sl, _sr;
    if (p_star <= pl) _sl = ul - cl;
    else _sl = ul - (cl * sqrt((1. + (((gamma + 1.) / (2. * gamma)) * ((p_star / pl) - 1.)))));
    if (p_star <= pr) _sr = ur + cr;
    else _sr = ur + (cr * sqrt((1. + (((gamma + 1.) / (2. * gamma)) * ((p_star / pr) - 1.)))));
    const double _sc = (((pr - pl) + ((dl * ul) * (_sl - ul))) - ((dr * ur) * (_sr - ur))) /
                       ((dl * (_sl - ul)) - (dr * (_sr - ur)));
    *sl = _sl;
    *sc = _sc;
    *sr = _sr;
}

/* RiemannBase.deboost  riemann.pyx:190-222 */
static void deboost(int dim, int F, const double *face_w, double *flux)
{
    for (int m = 0; m < F; m++) {
        for (int k = 0; k < dim; k++) {
            const double w = X(face_w, k, m, F), fm = X(flux, 0, m, F);
            X(flux, dim + 1, m, F) = X(flux, dim + 1, m, F) + (w * (((0.5 * w) * fm) + X(flux, 1 + k, m, F)));
            X(flux, 1 + k, m, F) = X(flux, 1 + k, m, F) + (w * fm);
        }
    }
}

/* HLL.riemann_solver riemann.pyx:243-373 and HLLC.riemann_solver riemann.pyx:521-682 */
static void hll_family(const orc_mesh *M, int hllc, double gamma, int boost,
                       const double *left, const double *right, const double *face_w,
                       double *flux)
{
    const int dim = M->dim, F = M->n_faces, E = dim + 1;
    for (int i = 0; i < F; i++) {
        const double _dl = X(left, 0, i, F), _pl = X(left, E, i, F);
        const double _dr = X(right, 0, i, F), _pr = X(right, E, i, F);
        double Vnl = 0.0, Vnr = 0.0, vl_sq = 0.0, vr_sq = 0.0, wn = 0.0;
        for (int k = 0; k < dim; k++) {
            const double vl = X(left, 1 + k, i, F), vr = X(right, 1 + k, i, F);
            const double nk = X(M->normal, k, i, F);
            vl_sq = vl_sq + vl * vl;
            vr_sq = vr_sq + vr * vr;
            Vnl = Vnl + vl * nk;
            Vnr = Vnr + vr * nk;
            wn = wn + X(face_w, k, i, F) * nk;
        }
        if (boost) wn = 0.;
        double sl, sc, sr;
        get_waves(_dl, Vnl, _pl, _dr, Vnr, _pr, gamma, &sl, &sc, &sr);
        if (wn <= sl) {
            X(flux, 0, i, F) = _dl * (Vnl - wn);
            X(flux, E, i, F) = ((((0.5 * _dl) * vl_sq) + (_pl / (gamma - 1.0))) * (Vnl - wn)) + (_pl * Vnl);
            for (int k = 0; k < dim; k++)
                X(flux, 1 + k, i, F) = ((_dl * X(left, 1 + k, i, F)) * (Vnl - wn)) + (_pl * X(M->normal, k, i, F));
        } else if ((sl < wn) && (wn <= sr)) {
            if (!hllc) {
                const double fac1 = sr - wn, fac2 = sl - wn, fac3 = sr - sl;
                X(flux, 0, i, F) = (((((_dl * Vnl) * fac1) - ((_dr * Vnr) * fac2)) - ((sl * _dl) * fac1)) +
                                    ((sr * _dr) * fac2)) / fac3;
                for (int k = 0; k < dim; k++) {
                    const double vl = X(left, 1 + k, i, F), vr = X(right, 1 + k, i, F);
                    const double nk = X(M->normal, k, i, F);
                    X(flux, 1 + k, i, F) =
                        ((((((((_dl * vl) * Vnl) + (_pl * nk)) * fac1) - ((((_dr * vr) * Vnr) + (_pr * nk)) * fac2)) -
                           ((sl * (_dl * vl)) * fac1)) + ((sr * (_dr * vr)) * fac2))) / fac3;
                }
                const double el = ((0.5 * _dl) * vl_sq) + (_pl / (gamma - 1.0));
                const double er = ((0.5 * _dr) * vr_sq) + (_pr / (gamma - 1.0));
                X(flux, E, i, F) = ((((((el + _pl) * Vnl) * fac1) - (((er + _pr) * Vnr) * fac2)) -
                                     ((sl * el) * fac1)) + ((sr * er) * fac2)) / fac3;
            } else if (wn <= sc) {
                const double factor_1 = (_dl * (sl - Vnl)) / (sl - sc);
                const double factor_2 = ((factor_1 * (sl - wn)) * (sc - Vnl)) + _pl;
                const double frho = (_dl * (Vnl - sl)) + (factor_1 * (sl - wn));
                const double el = ((0.5 * _dl) * vl_sq) + (_pl / (gamma - 1.0));
                X(flux, 0, i, F) = frho;
                X(flux, E, i, F) = (((el + _pl) * Vnl) - (sl * el)) +
                    (((sl - wn) * factor_1) * ((el / _dl) + ((sc - Vnl) * (sc + (_pl / (_dl * (sl - Vnl)))))));
                for (int k = 0; k < dim; k++)
                    X(flux, 1 + k, i, F) = (frho * X(left, 1 + k, i, F)) + (factor_2 * X(M->normal, k, i, F));
            } else {
                const double factor_1 = (_dr * (sr - Vnr)) / (sr - sc);
                const double factor_2 = ((factor_1 * (sr - wn)) * (sc - Vnr)) + _pr;
                const double frho = (_dr * (Vnr - sr)) + (factor_1 * (sr - wn));
                const double er = ((0.5 * _dr) * vr_sq) + (_pr / (gamma - 1.0));
                X(flux, 0, i, F) = frho;
                X(flux, E, i, F) = (((er + _pr) * Vnr) - (sr * er)) +
                    (((sr - wn) * factor_1) * ((er / _dr) + ((sc - Vnr) * (sc + (_pr / (_dr * (sr - Vnr)))))));
                for (int k = 0; k < dim; k++)
                    X(flux, 1 + k, i, F) = (frho * X(right, 1 + k, i, F)) + (factor_2 * X(M->normal, k, i, F));
            }
        } else {
            X(flux, 0, i, F) = _dr * (Vnr - wn);
            X(flux, E, i, F) = ((((0.5 * _dr) * vr_sq) + (_pr / (gamma - 1.0))) * (Vnr - wn)) + (_pr * Vnr);
            for (int k = 0; k < dim; k++)
                X(flux, 1 + k, i, F) = ((_dr * X(right, 1 + k, i, F)) * (Vnr - wn)) + (_pr * X(M->normal, k, i, F));
        }
    }
    if (boost) deboost(dim, F, face_w, flux);
}

/* Exact.p_guess / p_func / p_func_deriv / get_pstar  riemann.pyx:974-1090 */
static double p_guess(double dl, double ul, double pl, double cl, double dr, double ur,
                      double pr, double cr, double gamma)
{
    const double ppv = (.5 * (pl + pr)) - (((.125 * (ur - ul)) * (dl + dr)) * (cl + cr));
    const double p_max = (pr > pl) ? pr : pl;
    const double p_min = (pr < pl) ? pr : pl;
    const double q_max = p_max / p_min;
    double p0;
    if ((q_max <= 2.) && (p_min <= ppv && ppv <= p_max)) {
        p0 = ppv;
    } else if (ppv <= p_min) {
        const double p_lr = pow(pl / pr, (gamma - 1.) / (2. * gamma));
        double u_star = (((p_lr * ul) / cl) + (ur / cr)) + ((2. * (p_lr - 1.)) / (gamma - 1.));
        u_star = u_star / ((p_lr / cl) + (1. / cr));
        const double p_tl = pow((1. + (((gamma - 1.) * (ul - u_star)) / (2. * cl))), ((2. * gamma) / (gamma - 1.)));
        const double p_tr = pow((1. + (((gamma - 1.) * (u_star - ur)) / (2. * cr))), ((2. * gamma) / (gamma - 1.)));
        p0 = .5 * ((pl * p_tl) + (pr * p_tr));
    } else {
        const double gl = sqrt((2. / (dl * (gamma + 1.))) / ((((gamma - 1.) * pl) / (gamma + 1.)) + ppv));
        const double gr = sqrt((2. / (dr * (gamma + 1.))) / ((((gamma - 1.) * pr) / (gamma + 1.)) + ppv));
        p0 = (((gl * pl) + (gr * pr)) - (ur - ul)) / (gr + gl);
    }
    return p0;
}

static double p_func(double d, double p, double c, double gamma, double p_old)
{
    if (p_old <= p)
        return ((2. * c) / (gamma - 1.)) * (pow(p_old / p, (gamma - 1.) / (2. * gamma)) - 1.);
    const double Ak = 2. / (d * (gamma + 1.));
    const double Bk = (p * (gamma - 1.)) / (gamma + 1.);
    return (p_old - p) * sqrt(Ak / (p_old + Bk));
}

static double p_func_deriv(double d, double p, double c, double gamma, double p_old)
{
    if (p_old <= p)
        return pow(p_old / p, ((-(gamma + 1.)) / (2. * gamma))) / (c * d);
    const double Ak = 2. / (d * (gamma + 1.));
    const double Bk = (p * (gamma - 1.)) / (gamma + 1.);
    return sqrt(Ak / (p_old + Bk)) * (1. - ((.5 * (p_old - p)) / (Bk + p_old)));
}

static double get_pstar(double dl, double ul, double pl, double cl, double dr, double ur,
                        double pr, double cr, double gamma, int max_iter, int *failed)
{
    const double TOL = 1.0e-6;
    double p_old = p_guess(dl, ul, pl, cl, dr, ur, pr, cr, gamma), p_new = p_old;
    for (int it = 0; it < max_iter; it++) {
        const double fl = p_func(dl, pl, cl, gamma, p_old);
        const double fr = p_func(dr, pr, cr, gamma, p_old);
        const double dfl = p_func_deriv(dl, pl, cl, gamma, p_old);
        const double dfr = p_func_deriv(dr, pr, cr, gamma, p_old);
        p_new = p_old - ((((fl + fr) + ur) - ul) / (dfl + dfr));
        if ((2. * fabs((p_new - p_old) / (p_new + p_old))) <= TOL) return p_new;
        if (p_new < 0.) p_new = TOL;
        p_old = p_new;
    }
    *failed = 1;     /* 'No convergence in Exact Riemann Solver' */
    return p_new;
}

/* Exact.riemann_solver  riemann.pyx:700-972 (always deboosts) */
static int exact_solver(const orc_mesh *M, double gamma, const double *left, const double *right,
                        const double *face_w, double *flux, int max_iter)
{
    const int dim = M->dim, F = M->n_faces, E = dim + 1;
    int status = 0;
    double v[3];
    for (int i = 0; i < F; i++) {
        const double _dl = X(left, 0, i, F), _pl = X(left, E, i, F);
        const double _dr = X(right, 0, i, F), _pr = X(right, E, i, F);
        const double cl = sqrt((gamma * _pl) / _dl);
        const double cr = sqrt((gamma * _pr) / _dr);
        double vnl = 0.0, vnr = 0.0, vl_sq = 0.0, vr_sq = 0.0;
        for (int k = 0; k < dim; k++) {
            const double a = X(left, 1 + k, i, F), b = X(right, 1 + k, i, F), nk = X(M->normal, k, i, F);
            vnl = vnl + a * nk;
            vnr = vnr + b * nk;
            vl_sq = vl_sq + a * a;
            vr_sq = vr_sq + b * b;
        }
        int failed = 0;
        const double p_star = get_pstar(_dl, vnl, _pl, cl, _dr, vnr, _pr, cr, gamma, max_iter, &failed);
        if (failed) status |= ORC_RIEMANN_NONCONVERGED;
        const double fl = p_func(_dl, _pl, cl, gamma, p_star);
        const double fr = p_func(_dr, _pr, cr, gamma, p_star);
        const double u_star = 0.5 * (((vnl + vnr) + fr) - fl);
        /* sampled state: kind 0 = left data, 1 = right data, 2 = generic (d,p,u-shift,side) */
        int kind;
        double _d = 0, _p = 0, ushift = 0;
        int side = 0;    /* 0: left states, 1: right states */
        if (0.0 <= u_star) {
            if (p_star <= _pl) {
                const double s_hl = vnl - cl;
                if (0.0 <= s_hl) kind = 0;
                else {
                    const double c_star_l = cl * pow(p_star / _pl, (gamma - 1.0) / (2.0 * gamma));
                    const double s_tl = u_star - c_star_l;
                    if (0.0 >= s_tl) {
                        kind = 2; _d = _dl * pow(p_star / _pl, 1.0 / gamma); _p = p_star; ushift = u_star - vnl;
                    } else {
                        const double c = (2.0 / (gamma + 1.0)) * (cl + ((0.5 * (gamma - 1.0)) * vnl));
                        kind = 2; _d = _dl * pow(c / cl, 2.0 / (gamma - 1.0));
                        _p = _pl * pow(c / cl, (2.0 * gamma) / (gamma - 1.0)); ushift = c - vnl;
                    }
                }
            } else {
                const double sl = vnl - (cl * sqrt(((((gamma + 1.0) * p_star) / ((2.0 * gamma) * _pl)) +
                                                    ((gamma - 1.0) / (2.0 * gamma)))));
                if (0.0 <= sl) kind = 0;
                else {
                    kind = 2;
                    _d = (_dl * ((p_star / _pl) + ((gamma - 1.0) / (gamma + 1.0)))) /
                         (((p_star * (gamma - 1.0)) / ((gamma + 1.0) * _pl)) + 1.0);
                    _p = p_star; ushift = u_star - vnl;
                }
            }
        } else {
            side = 1;
            if (p_star >= _pr) {
                const double sr = vnr + (cr * sqrt(((((gamma + 1.0) * p_star) / ((2.0 * gamma) * _pr)) +
                                                    ((gamma - 1.0) / (2.0 * gamma)))));
                if (0.0 >= sr) kind = 1;
                else {
                    kind = 2;
                    _d = (_dr * ((p_star / _pr) + ((gamma - 1.0) / (gamma + 1.0)))) /
                         (((p_star * (gamma - 1.0)) / ((gamma + 1.0) * _pr)) + 1.0);
                    _p = p_star; ushift = u_star - vnr;
                }
            } else {
                const double s_hr = vnr + cr;
                if (0.0 >= s_hr) kind = 1;
                else {
                    const double c_star_r = cr * pow(p_star / _pr, (gamma - 1.0) / (2.0 * gamma));
                    const double s_tr = u_star + c_star_r;
                    if (0.0 <= s_tr) {
                        kind = 2; _d = _dr * pow(p_star / _pr, 1.0 / gamma); _p = p_star; ushift = u_star - vnr;
                    } else {
                        const double c = (2.0 / (gamma + 1.0)) * (cr - ((0.5 * (gamma - 1.0)) * vnr));
                        const double u_tmp = (2.0 / (gamma + 1.0)) * ((-cr) + ((0.5 * (gamma - 1.0)) * vnr));
                        (void)c;
                        kind = 2; _d = _dr * pow(c / cr, 2.0 / (gamma - 1.0));
                        _p = _pr * pow(c / cr, (2.0 * gamma) / (gamma - 1.0)); ushift = u_tmp - vnr;
                    }
                }
            }
        }
        if (kind == 0) {
            X(flux, 0, i, F) = _dl * vnl;
            X(flux, E, i, F) = (((0.5 * _dl) * vl_sq) + ((gamma * _pl) / (gamma - 1.0))) * vnl;
            for (int k = 0; k < dim; k++)
                X(flux, 1 + k, i, F) = ((_dl * X(left, 1 + k, i, F)) * vnl) + (_pl * X(M->normal, k, i, F));
        } else if (kind == 1) {
            X(flux, 0, i, F) = _dr * vnr;
            X(flux, E, i, F) = (((0.5 * _dr) * vr_sq) + ((gamma * _pr) / (gamma - 1.0))) * vnr;
            for (int k = 0; k < dim; k++)
                X(flux, 1 + k, i, F) = ((_dr * X(right, 1 + k, i, F)) * vnr) + (_pr * X(M->normal, k, i, F));
        } else {
            const double *st = side ? right : left;
            double vn = 0., v_sq = 0.;
            for (int k = 0; k < dim; k++) {
                v[k] = X(st, 1 + k, i, F) + (ushift * X(M->normal, k, i, F));
                vn = vn + v[k] * X(M->normal, k, i, F);
                v_sq = v_sq + v[k] * v[k];
            }
            X(flux, 0, i, F) = _d * vn;
            X(flux, E, i, F) = (((0.5 * _d) * v_sq) + ((gamma * _p) / (gamma - 1.0))) * vn;
            for (int k = 0; k < dim; k++)
                X(flux, 1 + k, i, F) = ((_d * v[k]) * vn) + (_p * X(M->normal, k, i, F));
        }
    }
    deboost(dim, F, face_w, flux);
    return status;
}

int orc_riemann(const orc_mesh *M, int solver, double gamma, int boost, const double *left,
                const double *right, const double *face_w, double *flux, int exact_max_iter)
{
    if (solver == ORC_EXACT) return exact_solver(M, gamma, left, right, face_w, flux, exact_max_iter);
    hll_family(M, solver == ORC_HLLC, gamma, boost, left, right, face_w, flux);
    return 0;
}

/* Mesh.update_from_fluxes  mesh.pyx:479-551 (positivity checks become status bits) */
int orc_update_from_fluxes(const orc_mesh *M, const double *flux, double dt, double *cons)
{
    const int dim = M->dim, n = M->n_cells, F = M->n_faces, E = dim + 1;
    int status = 0;
    for (int f = 0; f < F; f++) {
        const int i = M->pair_i[f], j = M->pair_j[f];
        const double a = M->area[f];
        if (M->tag[i] == REAL_TAG) {
            X(cons, 0, i, n) = X(cons, 0, i, n) - ((dt * a) * X(flux, 0, f, F));
            X(cons, E, i, n) = X(cons, E, i, n) - ((dt * a) * X(flux, E, f, F));
            for (int k = 0; k < dim; k++)
                X(cons, 1 + k, i, n) = X(cons, 1 + k, i, n) - ((dt * a) * X(flux, 1 + k, f, F));
        }
        if (M->tag[j] == REAL_TAG) {
            X(cons, 0, j, n) = X(cons, 0, j, n) + ((dt * a) * X(flux, 0, f, F));
            X(cons, E, j, n) = X(cons, E, j, n) + ((dt * a) * X(flux, E, f, F));
            for (int k = 0; k < dim; k++)
                X(cons, 1 + k, j, n) = X(cons, 1 + k, j, n) + ((dt * a) * X(flux, 1 + k, f, F));
        }
        if (X(cons, 0, i, n) <= 0.0 || X(cons, 0, j, n) <= 0.0) status |= ORC_NEG_MASS;
        if (X(cons, E, i, n) <= 0.0 || X(cons, E, j, n) <= 0.0) status |= ORC_NEG_ENERGY;
    }
    return status;
}

/* DomainManager.update_ghost_fields(conservative, True), serial branch
 * (domain_manager.pyx:750-774) + Reflective.update_fields (boundary.pyx:309-348) */
void orc_ghost_refresh_cons(const orc_mesh *M, double *cons)
{
    const int dim = M->dim, n = M->n_cells, nf = dim + 2;
    for (int i = 0; i < n; i++) {
        if (M->tag[i] == REAL_TAG) continue;
        const int im = M->map[i];
        for (int f = 0; f < nf; f++) X(cons, f, i, n) = X(cons, f, im, n);
    }
    if (!M->reflective) return;
    for (int i = 0; i < n; i++) {
        if (M->type[i] != EXTERIOR_TYPE) continue;
        for (int k = 0; k < dim; k++) {
            if (X(M->x, k, i, n) < M->xmin[k]) X(cons, 1 + k, i, n) *= -1;
            if (X(M->x, k, i, n) > M->xmax[k]) X(cons, 1 + k, i, n) *= -1;
        }
    }
}

/* IdealGas.primitive_from_conservative  equation_state.pyx:81-117 (all cells) */
void orc_prim_from_cons(int dim, int n, double gamma, const double *vol, const double *cons, double *prim)
{
    const int E = dim + 1;
    for (int i = 0; i < n; i++) {
        const double m = X(cons, 0, i, n);
        const double d = m / vol[i];
        X(prim, 0, i, n) = d;
        double v_sq = 0.;
        for (int k = 0; k < dim; k++) {
            const double v = X(cons, 1 + k, i, n) / m;
            X(prim, 1 + k, i, n) = v;
            v_sq = v_sq + v * v;
        }
        X(prim, E, i, n) = ((X(cons, E, i, n) / vol[i]) - ((.5 * d) * v_sq)) * (gamma - 1.);
    }
}

/* IdealGas.conservative_from_primitive  equation_state.pyx:43-79 (all cells) */
void orc_cons_from_prim(int dim, int n, double gamma, const double *vol, const double *prim, double *cons)
{
    const int E = dim + 1;
    for (int i = 0; i < n; i++) {
        const double d = X(prim, 0, i, n);
        const double m = d * vol[i];
        X(cons, 0, i, n) = m;
        double v_sq = 0.;
        for (int k = 0; k < dim; k++) {
            const double v = X(prim, 1 + k, i, n);
            X(cons, 1 + k, i, n) = v * m;
            v_sq = v_sq + v * v;
        }
        X(cons, E, i, n) = (((.5 * d) * v_sq) + (X(prim, E, i, n) / (gamma - 1.))) * vol[i];
    }
}

/* RiemannBase.compute_time_step  riemann.pyx:120-188 */
double orc_time_step(const orc_mesh *M, const double *prim, double gamma, double cfl, int boost)
{
    const int dim = M->dim, n = M->n_cells;
    double c, R, dt, vsq;
    c = sqrt((gamma * X(prim, dim + 1, 0, n)) / X(prim, 0, 0, n));
    if (dim == 2) R = sqrt(M->vol[0] / PI_D);
    else R = pow((3.0 * M->vol[0]) / (4.0 * PI_D), 1.0 / 3.0);
    if (boost) dt = R / c;
    else {
        vsq = 0.0;
        for (int k = 0; k < dim; k++) vsq = vsq + X(prim, 1 + k, 0, n) * X(prim, 1 + k, 0, n);
        dt = R / (c + sqrt(vsq));
    }
    for (int i = 0; i < n; i++) {
        if (M->tag[i] != REAL_TAG) continue;
        c = sqrt((gamma * X(prim, dim + 1, i, n)) / X(prim, 0, i, n));
        if (dim == 2) R = sqrt(M->vol[i] / PI_D);
        else R = pow((3.0 * M->vol[i]) / (4.0 * PI_D), 1.0 / 3.0);
        if (boost) dt = fmin(R / c, dt);
        else {
            vsq = 0.0;
            for (int k = 0; k < dim; k++) vsq = vsq + X(prim, 1 + k, i, n) * X(prim, 1 + k, i, n);
            dt = fmin(R / (c + sqrt(vsq)), dt);
        }
    }
    return cfl * dt;
}

/* Mesh.assign_generator_velocities  mesh.pyx:363-426 (all cells) */
void orc_generator_velocities(const orc_mesh *M, const double *prim, double gamma, double eta,
                              int regularize, double *w)
{
    const int dim = M->dim, n = M->n_cells;
    for (int i = 0; i < n; i++) {
        for (int k = 0; k < dim; k++) X(w, k, i, n) = X(prim, 1 + k, i, n);
        if (!regularize) continue;
        const double c = sqrt((gamma * X(prim, dim + 1, i, n)) / X(prim, 0, i, n));
        double d = 0.0, R;
        for (int k = 0; k < dim; k++) d = d + pow(X(M->dcom, k, i, n), 2.0);
        d = sqrt(d);
        if (dim == 2) R = sqrt(M->vol[i] / PI_D);
        else R = pow((3.0 * M->vol[i]) / (4.0 * PI_D), 1.0 / 3.0);
        if ((0.9 <= (d / (eta * R))) && ((d / (eta * R)) < 1.1)) {
            for (int k = 0; k < dim; k++)
                X(w, k, i, n) = X(w, k, i, n) +
                    (((c * X(M->dcom, k, i, n)) * (d - ((0.9 * eta) * R))) / (((d * 0.2) * eta) * R));
        } else if (1.1 <= (d / (eta * R))) {
            for (int k = 0; k < dim; k++)
                X(w, k, i, n) = X(w, k, i, n) + ((c * X(M->dcom, k, i, n)) / d);
        }
    }
}

/* Python's float power (float_pow -> libm pow), which the reference's mesh.pyx:472
 * reaches through boxed operands: called through a volatile pointer so the compiler
 * does not fold pow(x, 2.0) into x*x. */
static double (*volatile py_pow)(double, double) = pow;

/* Mesh.assign_face_velocities  mesh.pyx:428-477 */
void orc_face_velocities(const orc_mesh *M, const double *w, double *face_w)
{
    const int dim = M->dim, n = M->n_cells, F = M->n_faces;
    for (int m = 0; m < F; m++) {
        const int i = M->pair_i[m], j = M->pair_j[m];
        double factor = 0.0, denom = 0.0;
        for (int k = 0; k < dim; k++) {
            factor = factor + ((X(w, k, i, n) - X(w, k, j, n)) *
                               (X(M->com, k, m, F) - (0.5 * (X(M->x, k, i, n) + X(M->x, k, j, n)))));
            denom = denom + py_pow(X(M->x, k, j, n) - X(M->x, k, i, n), 2.0);
        }
        factor = factor / denom;
        for (int k = 0; k < dim; k++)
            X(face_w, k, m, F) = (0.5 * (X(w, k, i, n) + X(w, k, j, n))) +
                                 (factor * (X(M->x, k, j, n) - X(M->x, k, i, n)));
    }
}

/* hilbert_key_2d  hilbert.pyx:9-23 */
void orc_hilbert_key_2d(int n, const int32_t *xh, const int32_t *yh, int order, int64_t *keys)
{
    static const int key_index_2d[4] = {0, 1, 3, 2};
    for (int p = 0; p < n; p++) {
        int32_t x = xh[p], y = yh[p];
        int64_t key = 0;
        for (int i = order - 1; i >= 0; i--) {
            const int xbit = (x & (1 << i)) ? 1 : 0;
            const int ybit = (y & (1 << i)) ? 1 : 0;
            if (xbit == 0 && ybit == 0) { int32_t t = x; x = y; y = t; }
            else if (xbit == 1 && ybit == 0) { int32_t t = x; x = ~y; y = ~t; }
            key = (key << 2) + key_index_2d[(xbit << 1) + ybit];
        }
        keys[p] = key;
    }
}

/* One step of the flux path on a fixed mesh, in the order of
 * MovingMeshMUSCLHancock.evolve_timestep (integrate.py:385-428) when `moving`, or
 * StaticMeshMUSCLHancock.evolve_timestep (integrate.py:349-378) otherwise; the
 * generators are not moved (the host re-mesh is outside the path).  `prim` and
 * `cons` (all cells) are advanced in place; returns status bits. */
int orc_step(const orc_mesh *M, const orc_params *P, double dt, double *prim, double *cons,
             double *w, double *face_w, double *grad, double *left, double *right, double *flux)
{
    const int dim = M->dim, n = M->n_cells;
    int status = 0;
    if (P->moving) {
        orc_generator_velocities(M, prim, P->gamma, P->eta, P->regularize, w);
        orc_face_velocities(M, w, face_w);
    }
    if (P->reconstruction == ORC_LINEAR) {
        status |= orc_compute_gradients(M, prim, P->limiter, grad);
        orc_add_spatial(M, prim, grad, face_w, P->boost, P->gizmo, left, right);
        orc_add_temporal(M, prim, grad, face_w, P->gamma, 0.5 * dt, P->boost, left, right);
    } else {
        orc_pwc_states(M, prim, face_w, P->boost, left, right);
    }
    status |= orc_riemann(M, P->solver, P->gamma, P->boost, left, right, face_w, flux, P->exact_max_iter);
    status |= orc_update_from_fluxes(M, flux, dt, cons);
    orc_ghost_refresh_cons(M, cons);
    orc_prim_from_cons(dim, n, P->gamma, M->vol, cons, prim);
    return status;
}
