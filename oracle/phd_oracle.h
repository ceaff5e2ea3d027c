/* phd_oracle.h -- CPU restatement of the reference flux path (test infrastructure). */
#ifndef PHD_ORACLE_H
#define PHD_ORACLE_H
#include <stdint.h>

/* status bits; same values as the PHD_STATUS_* bits of include/phdflux.h */
#define ORC_NEG_MASS 1
#define ORC_NEG_ENERGY 2
#define ORC_RIEMANN_NONCONVERGED 4
#define ORC_BAD_INDEX 8

#define ORC_HLL 0
#define ORC_HLLC 1
#define ORC_EXACT 2

#define ORC_CONSTANT 0
#define ORC_LINEAR 1

typedef struct {
    int dim, n_cells, n_faces, reflective;
    const int8_t *tag, *type;
    const int32_t *map;
    const double *x, *dcom, *vol;                  /* [dim][n], [dim][n], [n] */
    const int32_t *pair_i, *pair_j;
    const double *area, *com, *normal;             /* [F], [dim][F], [dim][F] */
    const int32_t *nbr_ptr, *nbr_idx;
    double xmin[3], xmax[3];
} orc_mesh;

typedef struct {
    double gamma, eta;
    int reconstruction, limiter, gizmo, solver, boost, moving, regularize, exact_max_iter;
} orc_params;

int orc_compute_gradients(const orc_mesh *M, const double *prim, int limiter, double *grad);
void orc_pwc_states(const orc_mesh *M, const double *prim, const double *face_w, int boost,
                    double *left, double *right);
void orc_add_spatial(const orc_mesh *M, const double *prim, const double *grad,
                     const double *face_w, int boost, int gizmo, double *left, double *right);
void orc_add_temporal(const orc_mesh *M, const double *prim, const double *grad,
                      const double *face_w, double gamma, double dt, int boost,
                      double *left, double *right);
int orc_riemann(const orc_mesh *M, int solver, double gamma, int boost, const double *left,
                const double *right, const double *face_w, double *flux, int exact_max_iter);
int orc_update_from_fluxes(const orc_mesh *M, const double *flux, double dt, double *cons);
void orc_ghost_refresh_cons(const orc_mesh *M, double *cons);
void orc_prim_from_cons(int dim, int n, double gamma, const double *vol, const double *cons, double *prim);
void orc_cons_from_prim(int dim, int n, double gamma, const double *vol, const double *prim, double *cons);
double orc_time_step(const orc_mesh *M, const double *prim, double gamma, double cfl, int boost);
void orc_generator_velocities(const orc_mesh *M, const double *prim, double gamma, double eta,
                              int regularize, double *w);
void orc_face_velocities(const orc_mesh *M, const double *w, double *face_w);
void orc_hilbert_key_2d(int n, const int32_t *xh, const int32_t *yh, int order, int64_t *keys);
int orc_step(const orc_mesh *M, const orc_params *P, double dt, double *prim, double *cons,
             double *w, double *face_w, double *grad, double *left, double *right, double *flux);
#endif
