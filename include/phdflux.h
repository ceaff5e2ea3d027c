/*
 * phdflux.h -- C ABI of the GB300 flux path for the AREPO-style moving-mesh code
 * rickyfernandez/phd-code.
 *
 * All pointers in the structures and arguments below are DEVICE pointers unless
 * marked host.  Arrays are structure-of-arrays, row-major [field][index]:
 *   cells  : n_cells = n_real real cells followed by ghost cells
 *   prim   : [dim+2][n_cells]  density, velocity-x.., pressure
 *   cons   : [dim+2][n_cells]  mass, momentum-x.., energy (cell totals)
 *   grad   : [(dim+2)*dim][n_cells]  row f*dim+k = d prim_f / d x_k
 *   states, fluxes : [dim+2][n_faces] (same field order as prim / cons)
 * Face f joins cells pair_i[f] (always real) and pair_j[f] (real with a larger
 * index, or a ghost); nbr_ptr/nbr_idx list each cell's faces in ascending face id.
 *
 * Every entry point takes a cudaStream_t, never synchronises, and returns a host
 * error code (PHD_OK or PHD_ERR_*) for argument / launch errors.  Physics status
 * (negative mass, non-converged Riemann solve, bad index) is OR-ed as PHD_STATUS_*
 * bits into phd_clock.status on the device; the host reads it when it chooses.
 */
#ifndef PHDFLUX_H
#define PHDFLUX_H

#include <stdint.h>
#include <cuda_runtime.h>

#ifdef __cplusplus
extern "C" {
#endif

#define PHDFLUX_ABI_VERSION 1

/* host return codes */
#define PHD_OK 0
#define PHD_ERR_ARG 1
#define PHD_ERR_LAUNCH 2
#define PHD_ERR_UNSUPPORTED 3
#define PHD_ERR_SCRATCH_TOO_SMALL 4        /* mesh larger than a fixed work array allows */

/* device status bits (phd_clock.status) -- same meaning as the reference's raises */
#define PHD_STATUS_NEG_MASS 1              /* "Mass less than zero in flux update"   mesh.pyx:546-548 */
#define PHD_STATUS_NEG_ENERGY 2            /* "Energy less than zero in flux update" mesh.pyx:549-551 */
#define PHD_STATUS_RIEMANN_NONCONVERGED 4  /* "No convergence in Exact Riemann Solver" riemann.pyx:1088-1090 */
#define PHD_STATUS_BAD_INDEX 8             /* "ERROR: incorrect neighbors!" reconstruction.pyx:651-652 */
#define PHD_STATUS_LEFT_DOMAIN 16          /* "particle left domain in reflective boundary condition!!" boundary.pyx:262-263 */
#define PHD_STATUS_NONFINITE 32            /* FP32 path: a recovered primitive is NaN or infinite (no reference
                                              counterpart: the FP64 reference carries such values on silently) */

/* solver / reconstruction selectors */
#define PHD_HLL 0                          /* riemann.pyx:225-504 */
#define PHD_HLLC 1                         /* riemann.pyx:507-682 */
#define PHD_EXACT 2                        /* riemann.pyx:684-1090 */
#define PHD_CONSTANT 0                     /* PieceWiseConstant reconstruction.pyx:131-353 */
#define PHD_LINEAR 1                       /* PieceWiseLinear   reconstruction.pyx:355-1079 */
#define PHD_LIMITER_AREPO 0                /* reconstruction.pyx:683-703 */
#define PHD_LIMITER_TESS 1                 /* reconstruction.pyx:705-731 */

/* One tessellated state as the host mesh hands it over (mesh.pyx:255-323). */
typedef struct phd_mesh {
    int32_t dim, n_cells, n_real, n_faces;
    const int8_t *tag;        /* [n_cells] 0 = Real, 1 = Ghost            (particle_tags.py) */
    const int32_t *map;       /* [n_cells] image of each ghost             (domain_manager.pyx:519) */
    const int8_t *flip;       /* [n_cells] bit k: reflective ghost outside the box in axis k */
    const double *x;          /* [dim][n_cells] generator positions */
    const double *dcom;       /* [dim][n_cells] centroid - generator (ghosts: the image's) */
    const double *vol;        /* [n_cells] (ghosts: the image's) */
    const int32_t *pair_i, *pair_j;   /* [n_faces] */
    const double *area;       /* [n_faces] */
    const double *com;        /* [dim][n_faces] face centroid */
    const double *normal;     /* [dim][n_faces] (x_j - x_i)/|x_j - x_i|; may be NULL for
                                 phd_prepare_f32 (which then forms FP32 normals), entries
                                 that read FP64 normals return PHD_ERR_ARG without them */
    const int32_t *nbr_ptr;   /* [n_cells+1] */
    const int32_t *nbr_idx;   /* [2*n_faces] */
} phd_mesh;

/* Per-step device clock: time step, time and the CFL reduction accumulator. */
typedef struct phd_clock {
    double dt;                /* time step of the current step */
    double t;                 /* time at the start of the current step */
    double t_end;             /* > 0: clip dt to land on t_end (simulation_finish.py:82-88) */
    double dt_hydro;          /* last unclipped cfl * min(R/c) */
    unsigned long long dtmin_bits;    /* accumulator; initialise to the bits of +inf */
    unsigned int arrive;      /* accumulator; initialise to 0 */
    int status;               /* PHD_STATUS_* bits, OR-ed by kernels */
    long long step;           /* completed steps */
    double dt_last;           /* time step of the last completed step */
} phd_clock;

/* Physics parameters of a run. */
typedef struct phd_params {
    double gamma;             /* IdealGas.gamma (equation_state.pyx:40) */
    double cfl;               /* RiemannBase.cfl */
    double eta;               /* Mesh.eta, regularisation (mesh.pyx:87-89) */
    int32_t reconstruction;   /* PHD_CONSTANT | PHD_LINEAR */
    int32_t limiter;          /* PHD_LIMITER_AREPO | PHD_LIMITER_TESS */
    int32_t gizmo;            /* PieceWiseLinear.gizmo_limiter */
    int32_t solver;           /* PHD_HLL | PHD_HLLC | PHD_EXACT */
    int32_t boost;            /* RiemannBase.boost (Exact: always 1) */
    int32_t regularize;       /* Mesh.regularize */
    int32_t exact_max_iter;   /* Exact.get_pstar MAX_ITER (1000) */
    int32_t pad_;
} phd_params;

/* Library identity. */
int phd_abi_version(void);
const char *phd_status_string(int status_bit);

/* ---- FP64 stage entry points: one per reference plugin method -------------------- */

/* PieceWiseLinear.compute_gradients + DomainManager.update_ghost_gradients
 * (reconstruction.pyx:563-739, domain_manager.pyx:776-835, boundary.pyx:265-307).
 * grad must hold (dim+2)*dim rows of n_cells. */
int phd_gradients_f64(const phd_mesh *mesh, const double *prim, int32_t limiter,
                      double *grad, phd_clock *clk, cudaStream_t stream);

/* PieceWiseLinear.add_spatial (stages & 1, reconstruction.pyx:741-921) and/or
 * add_temporal (stages & 2, :923-1072; reads left/right when stage 1 is not run)
 * with the half step dt_half -- stages = 3 is compute_states (:1074-1079) -- or
 * PieceWiseConstant.compute_states (:254-353) when reconstruction == PHD_CONSTANT
 * (grad may then be NULL). */
#define PHD_STAGE_SPATIAL 1
#define PHD_STAGE_TEMPORAL 2
int phd_states_f64(const phd_mesh *mesh, const double *prim, const double *grad,
                   const double *face_w, double gamma, double dt_half, int32_t boost,
                   int32_t reconstruction, int32_t gizmo, int32_t stages, double *left,
                   double *right, cudaStream_t stream);

/* RiemannBase.compute_fluxes with HLL / HLLC / Exact and deboost
 * (riemann.pyx:74-98, 190-222, 243-373, 521-682, 700-1090). */
int phd_riemann_f64(const phd_mesh *mesh, int32_t solver, double gamma, int32_t boost,
                    int32_t exact_max_iter, const double *left, const double *right,
                    const double *face_w, double *flux, phd_clock *clk, cudaStream_t stream);

/* Mesh.update_from_fluxes (mesh.pyx:479-551) as a per-cell segmented sum in
 * ascending face order; real cells only; cons updated in place. */
int phd_update_from_fluxes_f64(const phd_mesh *mesh, const double *flux, double dt,
                               double *cons, phd_clock *clk, cudaStream_t stream);

/* DomainManager.update_ghost_fields(conservative, True) (domain_manager.pyx:712-774,
 * boundary.pyx:309-348): ghost cons = image cons, reflective momentum flip. */
int phd_ghost_cons_f64(const phd_mesh *mesh, double *cons, cudaStream_t stream);

/* IdealGas.primitive_from_conservative / conservative_from_primitive
 * (equation_state.pyx:81-117 / 43-79), all cells. */
int phd_prim_from_cons_f64(int32_t dim, int32_t n, double gamma, const double *vol,
                           const double *cons, double *prim, cudaStream_t stream);
int phd_cons_from_prim_f64(int32_t dim, int32_t n, double gamma, const double *vol,
                           const double *prim, double *cons, cudaStream_t stream);

/* RiemannBase.compute_time_step (riemann.pyx:120-188): clk->dt = cfl * min over real
 * cells, a warp-shuffle min reduction.  advance != 0 also moves clk->t by the
 * previous clk->dt and counts a step. */
int phd_time_step_f64(const phd_mesh *mesh, const double *prim, double gamma, double cfl,
                      int32_t boost, int32_t advance, phd_clock *clk, cudaStream_t stream);

/* Mesh.assign_generator_velocities / assign_face_velocities (mesh.pyx:363-477). */
int phd_generator_velocities_f64(const phd_mesh *mesh, const double *prim, double gamma,
                                 double eta, int32_t regularize, double *w, cudaStream_t stream);
int phd_face_velocities_f64(const phd_mesh *mesh, const double *w, double *face_w,
                            cudaStream_t stream);

/* ---- fused FP64 step (parity mode) -------------------------------------------------
 * One step of the flux path on a fixed mesh in the order of
 * MovingMeshMUSCLHancock.evolve_timestep (integrate.py:385-428) up to the host re-mesh
 * (moving != 0: generator + face velocities first) or StaticMeshMUSCLHancock
 * (integrate.py:349-378): gradients, states + Riemann + deboost fused per face,
 * segmented conserved update with ghost refresh, primitive recovery and the next
 * CFL time step.  Uses clk->dt; leaves the next step's dt in clk->dt.
 * Work arrays: grad [(dim+2)*dim][n_cells], flux [dim+2][n_faces], w [dim][n_cells],
 * face_w [dim][n_faces], cons_next [dim+2][n_cells].  cons and cons_next are swapped
 * by the caller between steps (the step writes cons_next). */
int phd_step_f64(const phd_mesh *mesh, const phd_params *par, int32_t moving,
                 double *prim, const double *cons, double *cons_next, double *grad,
                 double *w, double *face_w, double *flux, phd_clock *clk, cudaStream_t stream);

/* phd_step_f64 with four stage-boundary events (see phd_step_f32_marked). */
int phd_step_f64_marked(const phd_mesh *mesh, const phd_params *par, int32_t moving,
                        double *prim, const double *cons, double *cons_next, double *grad,
                        double *w, double *face_w, double *flux, phd_clock *clk,
                        cudaStream_t stream, cudaEvent_t *marks);

/* Limiter record ("tape") of the FP64 gradients, for the adjoint (no reference
 * counterpart: the reference has no adjoint).  tape_f64 [PHD_GRAD_TAPE_F64_ROWS][n]:
 * the unlimited gradient estimate (8 rows) and the limiter values (4 rows); tape_i32
 * [PHD_GRAD_TAPE_I32_ROWS][n]: per field the CSR entry of the active limit (-1 none,
 * -2 a clamp at zero or a flat field), the entries of the neighbour maximum and
 * minimum (-1: the cell itself), and the TESS limiter's active field.  Written for real
 * cells; the gradients themselves are those of phd_gradients_f64 / phd_step_f64. */
#define PHD_GRAD_TAPE_F64_ROWS 12
#define PHD_GRAD_TAPE_I32_ROWS 13
int phd_gradients_f64_taped(const phd_mesh *mesh, const double *prim, int32_t limiter, double *grad,
                            double *tape_f64, int32_t *tape_i32, phd_clock *clk, cudaStream_t stream);
int phd_step_f64_taped(const phd_mesh *mesh, const phd_params *par, int32_t moving, double *prim,
                       const double *cons, double *cons_next, double *grad, double *w, double *face_w,
                       double *flux, double *tape_f64, int32_t *tape_i32, phd_clock *clk,
                       cudaStream_t stream);

/* The FP64 step of a static mesh (phd_step_f64 with moving = 0) with its branch
 * decisions recorded (mode PHD_FROZEN_RECORD) or replayed (PHD_FROZEN_REPLAY): for
 * checking the adjoint against central finite differences on the branch a run takes.
 * No reference counterpart (the reference has no adjoint).  RECORD computes the
 * ordinary step and writes the limiter's selections (tape_f64 / tape_i32, the rows of
 * phd_gradients_f64_taped) and 64 decision bits per face into face_bits [F]: the GIZMO
 * clamps, minima and sign tests, the spatial and temporal positivity reverts, the
 * sound-speed floors, the pressure estimate's branch, the shock / rarefaction tests and
 * the Riemann region.  REPLAY does the same arithmetic with every decision read back
 * (tape_f64 unused), so near the recorded state the step is the smooth map the adjoint
 * differentiates.  dt is the step's (host) time step, held fixed; prim is overwritten
 * with the next primitives, cons_next receives the next totals (all cells), flux the
 * face fluxes.  HLL / HLLC with the AREPO limiter or constant reconstruction (else
 * PHD_ERR_UNSUPPORTED). */
#define PHD_FROZEN_RECORD 0
#define PHD_FROZEN_REPLAY 1
int phd_step_f64_frozen(const phd_mesh *mesh, const phd_params *par, int32_t mode, double dt, double *prim,
                        const double *cons, double *cons_next, double *grad, const double *face_w, double *flux,
                        double *tape_f64, int32_t *tape_i32, uint64_t *face_bits, phd_clock *clk,
                        cudaStream_t stream);

/* ---- fused FP32 step (FP32 reconstruction / Riemann, FP64 conserved totals) --------
 * Mesh-relative FP32 geometry, formed once per mesh by phd_prepare_f32 (the
 * cancelling differences in FP64, each rounded once to FP32):
 *   face_geo [F][4] (n_x, n_y, c_x, c_y), c = face centroid - (x_i + x_j)/2; the
 *                   normal is mesh->normal rounded, or (x_j - x_i)/|x_j - x_i| in FP32
 *                   when mesh->normal is NULL
 *   face_ar  [F][2] (area, |x_j - x_i|)
 *   csr_face [2F]   per-cell face list (nbr_ptr order): face id where the cell is
 *                   pair-i, ~face id where it is pair-j
 *   csr_nbr  [2F]   the other cell of each listed face
 *   cell_geo [n][4] (dcom_x, dcom_y, 1/vol, sqrt(vol/pi))
 *   entry_rec [2F][4] per list entry (sigma = +1 where the cell is pair-i, -1 where it is
 *                   pair-j): (w_x, w_y, t_x, t_y), w = (area/r) c + sigma (area/2) n the
 *                   gradient weight, t = c + sigma (r/2) n the face centroid minus the
 *                   generator (r = |x_j - x_i|); the gradient kernel reads its geometry in
 *                   list order through it (PHD_PREP_RECORDS).  Optional: NULL makes the
 *                   gradient kernel form each entry's record from its face's records
 *                   (csr_face, face_geo, face_ar) with the same roundings, so the same
 *                   bits -- cheaper for a mesh stepped once, dearer per step when many
 *                   steps share one mesh
 * twin (optional, [F]): for periodic faces the reference computes twice (once from each
 * side, mesh.pyx:529-544), twin[f] = the kept copy's id for the dropped copy f, else -1;
 * both cells then exchange the same FP32 flux and the totals are conserved exactly. */
typedef struct phd_geom32 {
    const float *face_geo;
    const float *face_ar;
    const int32_t *csr_face;
    const int32_t *csr_nbr;
    const float *cell_geo;
    const float *entry_rec;
} phd_geom32;

typedef struct phd_geom32_out {
    float *face_geo;
    float *face_ar;
    int32_t *csr_face;
    int32_t *csr_nbr;
    float *cell_geo;
    float *entry_rec;           /* may be NULL where no part writes it */
} phd_geom32_out;

/* All parts (PHD_PREP_ALL, plus PHD_PREP_RECORDS when out->entry_rec is given). */
int phd_prepare_f32(const phd_mesh *mesh, const int32_t *twin, phd_geom32_out *out,
                    cudaStream_t stream);

/* phd_prepare_f32 in parts, so each part can run as soon as its inputs are on the
 * device: PHD_PREP_FACES (face_geo, face_ar: needs pair ids, x, com, area), PHD_PREP_CELLS
 * (cell_geo: dcom, vol), PHD_PREP_LISTS (csr_face, csr_nbr: neighbour lists, pair ids,
 * twin table). */
#define PHD_PREP_FACES 1
#define PHD_PREP_CELLS 2
#define PHD_PREP_LISTS 4
#define PHD_PREP_ALL 7
/* cell_geo formed from the prepared faces instead of mesh->vol / dcom (the volume and
 * centre of mass sums of tess.cpp:330-393, in FP32); needs PHD_PREP_FACES and
 * PHD_PREP_LISTS done before it (same call or earlier on the stream); excludes
 * PHD_PREP_CELLS.  The FP32 path then needs no volumes or centroids from the host. */
#define PHD_PREP_CELLS_FROM_FACES 8
/* entry_rec from the prepared faces and list codes; needs PHD_PREP_FACES and
 * PHD_PREP_LISTS done before it (same call or earlier on the stream). */
#define PHD_PREP_RECORDS 16
int phd_prepare_f32_parts(const phd_mesh *mesh, const int32_t *twin, phd_geom32_out *out,
                          int32_t parts, cudaStream_t stream);

/* DomainManager.move_generators + BoundaryCondition.migrate_particles
 * (domain_manager.pyx:566-590, boundary.pyx:236-263, 502-538) after a step: for every
 * real cell x_out[k][i] = x[k][i] + dt_last * w[k][i] (FP64, the product and the sum
 * rounded separately, as the reference does) with the step's generator velocities --
 * w2 [n][2] FP32 from the FP32 step, or w [2][n] FP64 from the FP64 step (exactly one
 * of them non-NULL) -- and clk->dt_last.  A generator outside [xmin, xmax] in some
 * axis is wrapped (periodic != 0: +L where it is <= xmin, -L where >= xmax, L = xmax -
 * xmin) or, for reflective walls, flagged PHD_STATUS_LEFT_DOMAIN in clk->status.
 * x_out is [2][n_real]. */
int phd_move_generators(const phd_mesh *mesh, const float *w2, const double *w, phd_clock *clk, int32_t periodic,
                        double xmin0, double xmin1, double xmax0, double xmax1, double *x_out, cudaStream_t stream);

/* The ghost rows of mesh->x from their images' rows (the real rows already hold the
 * current positions, e.g. from phd_move_generators): per ghost g, ghost_code[g - n_real]
 * = 1 + 3 (sx + 1) + (sy + 1) for a periodic copy shifted by (sx, sy) box lengths
 * (x + s (xmax - xmin)), 16 + 2 k + h for a mirror image across axis k at its low
 * (h = 0) or high (h = 1) wall (x - 2 (x - wall)) -- the host tessellation's own
 * arithmetic, so the positions equal the host's bit for bit.  Invalid codes or images
 * add to *bad (device) and leave the row unwritten.  With it a re-mesh hands over no
 * positions at all (mesh->x is written through the const mesh view). */
int phd_ghost_positions(const phd_mesh *mesh, const int8_t *ghost_code, double xmin0, double xmin1, double xmax0,
                        double xmax1, int32_t *bad, cudaStream_t stream);

/* Compact FP32 hand-over of a re-mesh (the per-step upload of the face list,
 * mesh.pyx:255-323, in 12 B per face instead of 32): the host sends pair-j, the area
 * and the centroid offset along the face rounded once to FP32, and pair-i as
 * per-real-cell face ranges.  The offset: with (dx, dy) = x_j - x_i, r = sqrt(dx dx +
 * dy dy) and c = com - (x_i + x_j)/2, all in FP64 with each operation rounded
 * separately (no fused multiply-add), s = (c_x (-dy) + c_y dx) / r, 0 where r = 0 (c
 * lies along the face: a Voronoi face is on the perpendicular bisector of x_i x_j).
 * pair-j may come packed in 2 B per face: pair_dj[f] = pair_j[f] - pair_i[f] where that
 * lies in [1, 65534], else 0 (PHD_PAIR16_ESCAPE), with the faces marked 0 listed in
 * pair_x as (face id, pair-j) pairs in ascending face id -- 10 B per face in all (65535
 * is not used: the device marks the listed faces with it while decoding).
 *
 * phd_pair_i_from_face_ptr: pair_i[m] = c for m in [face_ptr[c], face_ptr[c+1]);
 * face_ptr (n_real + 1 entries) must start at 0, end at n_faces and not decrease --
 * each real cell whose range breaks that adds 1 to *bad (device) and writes nothing.
 * phd_prepare_f32_faces_compact: out->face_geo / face_ar as PHD_PREP_FACES forms them,
 * from area32 [F] and ct32 [F] (the offsets s) instead of mesh->area / com (needs pair
 * ids and x); the values equal PHD_PREP_FACES's bit for bit (both form the FP32 offset
 * as s times the FP32 face tangent). */
int phd_pair_i_from_face_ptr(const phd_mesh *mesh, const int32_t *face_ptr, int32_t *pair_i, int32_t *bad,
                             cudaStream_t stream);
int phd_prepare_f32_faces_compact(const phd_mesh *mesh, const float *area32, const float *ct32,
                                  phd_geom32_out *out, cudaStream_t stream);

/* One hand-over of a re-mesh to an FP32 stepper in one call: the host tessellation of
 * integrate.py:410-417 arrives in the compact format and the device forms everything
 * else (steps 6-8 of the moving-mesh step) -- pair-i from the face ranges
 * (phd_pair_i_from_face_ptr), the neighbour lists (phd_build_csr), the ghost rows of
 * mesh->x (phd_ghost_positions) or all of mesh->x from the host, the periodic twins,
 * the FP32 list codes, face geometry and cell geometry (phd_prepare_f32_parts,
 * phd_prepare_f32_faces_compact), the flip bits (phd_flip_mask), the ghost totals
 * (phd_ghost_cons_f64) and the primitives with the next dt (phd_prim_f32_cells), and,
 * when out->entry_rec is not NULL, the gradient records from the same face loads.
 *
 * The copies run on `stream` with the large ones (area, centroid offset) issued right
 * after the small ones the lists need (arrays laid out back to back both on the host and
 * in their staging -- pair_x, face_ptr, pair_dj, list_len, ghost_code, in that order --
 * go over as one copy); the derivations run on side[0] (pair-i,
 * positions, neighbour lists, list codes, then the cell geometry) and side[1] (flip
 * bits, periodic twins from the face ranges, and the face geometry as soon as the face
 * records have landed, in two parts) while the copies are in flight, and are joined
 * back into `stream` at the end.  events: 8 CUDA events (created by the caller, reused
 * across calls).  The mesh's own arrays (pair_i, pair_j, map
 * ghost rows, x, nbr_ptr/nbr_idx, flip) are written through the const view; mesh->normal
 * must be NULL (the FP32 geometry forms its own normals).  The counts are the mesh's:
 * a tessellation with other counts needs the arrays re-sized first.  Faces or ghosts
 * whose indices are out of range add to *bad (device; read it after the call). */
#ifndef PHD_PAIR16_ESCAPE
#define PHD_PAIR16_ESCAPE 0       /* also in phdtess.h */
#endif
typedef struct phd_handover32 {
    /* host arrays (pinned, for the copies to overlap the derivations) */
    const int32_t *face_ptr;      /* [n_real + 1] faces of each real cell */
    const int32_t *pair_j;        /* [n_faces]; NULL: pair_dj and pair_x carry pair-j */
    const float *area32;          /* [n_faces] face areas, FP32 (NULL with face32) */
    const float *ct32;            /* [n_faces] centroid offset along the face, FP32 (see above) */
    const int32_t *ghost_map;     /* [n_cells - n_real] images of the ghosts; NULL: mesh->map holds them */
    const int8_t *ghost_code;     /* [n_cells - n_real] phd_ghost_positions codes (with x == NULL) */
    const double *x;              /* [2][n_cells] every position; NULL: real rows from x_real, ghost
                                     rows from ghost_code */
    /* device arrays */
    const double *x_real;         /* [2][n_real] real positions (phd_move_generators' x_out); NULL:
                                     mesh->x already holds them.  Ignored when x != NULL. */
    const int8_t *type;           /* [n_cells] particle types (the flip bits' Exterior test) */
    int32_t *d_face_ptr;          /* [n_real + 1] staging */
    float *d_area32;              /* [n_faces] staging */
    float *d_ct32;                /* [n_faces] staging */
    int8_t *d_ghost_code;         /* [n_cells - n_real] staging (with x == NULL) */
    int32_t *twin;                /* [n_faces] periodic twin table */
    int32_t *csr_work;            /* phd_csr_work_ints(n_cells) */
    int32_t *bad;                 /* [1] error counter, zeroed by the call */
    int32_t periodic;             /* 1: periodic box, 0: reflective walls */
    int32_t dedup_periodic;       /* 1: periodic twin faces counted once (phd_periodic_twins) */
    double xmin[2], xmax[2];      /* the box */
    /* packed pair-j (with pair_j == NULL; see above) */
    const uint16_t *pair_dj;      /* [n_faces] host: pair-j minus pair-i in [1, 65534], or PHD_PAIR16_ESCAPE */
    const int32_t *pair_x;        /* [2 n_pair_x] host: (face id, pair-j) of the escaped faces */
    int32_t n_pair_x;
    uint16_t *d_pair_dj;          /* [n_faces] staging (the call marks the listed faces in it) */
    int32_t *d_pair_x;            /* [2 n_pair_x] staging */
    /* optional: each cell's neighbour-list length (its faces; every length <= 255), so
     * the lists are laid out without counting them on the device.  Lengths that do not
     * match the faces add to *bad; the lists then stay inside their storage. */
    const uint8_t *list_len;      /* [n_cells] host, or NULL */
    uint8_t *d_list_len;          /* [n_cells] staging */
    /* optional: area and offset interleaved, one (area, offset) pair per face, in place of
     * area32 and ct32 (which are then NULL) */
    const float *face32;          /* [n_faces][2] host */
    float *d_face32;              /* [n_faces][2] staging */
} phd_handover32;

int phd_load_mesh_f32(const phd_mesh *mesh, const phd_handover32 *h, const phd_params *par, phd_geom32_out *out,
                      double *cons, float *prim4, phd_clock *clk, cudaStream_t stream, const cudaStream_t *side,
                      cudaEvent_t *events);

/* FP64 totals -> FP32 primitive cells prim4 [n][4] (rho, v_x, v_y, p) and clk->dt from
 * the CFL minimum (clock not advanced). */
int phd_prim_f32(const phd_mesh *mesh, const phd_params *par, const double *cons, float *prim4,
                 phd_clock *clk, cudaStream_t stream);

/* phd_prim_f32 with the volumes of a prepared cell_geo [n][4] (e.g. formed with
 * PHD_PREP_CELLS_FROM_FACES) instead of mesh->vol. */
int phd_prim_f32_cells(const phd_mesh *mesh, const float *cell_geo, const phd_params *par,
                       const double *cons, float *prim4, phd_clock *clk, cudaStream_t stream);

/* phd_prim_f32 for a batch of runs (see phd_step_f32_batched): each run's clock gets
 * its own CFL step. */
int phd_prim_f32_batched(const phd_mesh *mesh, const phd_params *par, const double *cons,
                         float *prim4, phd_clock *clocks, int32_t n_runs,
                         const int32_t *cell_run, cudaStream_t stream);

/* One fused step (same order as phd_step_f64): gradients (+ generator velocities when
 * moving) -> per-face states, Riemann flux and deboost (face velocities formed on the
 * fly) -> segmented update into cons_next, FP32 primitives, next dt.
 * prim4 [n][4], w2 [n][2], flux4 [F][4] (FP32; each face's conserved increment dt*A*F,
 * applied with opposite signs to its two cells); cons, cons_next [4][n] (FP64);
 * cellrec [n][16] (FP32, 32-byte aligned) the record the gradient stage writes for the
 * face stage: the cell's primitives, its limited gradient (d/dx, d/dy of rho, v_x,
 * v_y, p, the reference's grad[f*dim+k] order), dcom and generator velocity.  With
 * linear reconstruction or a moving mesh geo->csr_nbr and cellrec are required, and
 * geo->entry_rec or else geo->face_geo, face_ar and csr_face. */
int phd_step_f32(const phd_mesh *mesh, const phd_geom32 *geo, const phd_params *par,
                 int32_t moving, float *prim4, const double *cons, double *cons_next, float *cellrec,
                 float *w2, float *flux4, phd_clock *clk, cudaStream_t stream);

/* Launch shape of the three step kernels (chosen by an autotuner): threads per block
 * (multiple of 32, <= 512; the face kernel <= 256), a cap on blocks per grid (0: enough
 * blocks for every item; > 0: that many blocks, each looping over items -- a persistent
 * launch) and items per thread (0 or 1, 2, 4: a block covers block * items consecutive
 * cells or faces, thread t taking items t, t + block, ...; a warp then handles 32 *
 * items faces).  The exact solver's face kernel always runs one face per thread.  Every
 * shape gives the same bits. */
typedef struct phd_launch {
    int32_t block_grad, block_face, block_update;
    int32_t grid_cap_grad, grid_cap_face, grid_cap_update;
    int32_t items_grad, items_face, items_update;
} phd_launch;

/* Batched step: n_runs independent runs concatenated into one mesh (disjoint cell and
 * face ranges; ghosts map inside their run) advance together, one launch per stage.
 * clocks[n_runs] holds each run's dt / t / CFL accumulator; cell_run[n_cells] the run
 * of each cell (may be NULL when n_runs == 1).  launch may be NULL (defaults).  Status
 * bits of a run go to clocks[run] (index errors of the gradient stage to clocks[0]). */
int phd_step_f32_batched(const phd_mesh *mesh, const phd_geom32 *geo, const phd_params *par,
                         int32_t moving, const phd_launch *launch, float *prim4,
                         const double *cons, double *cons_next, float *cellrec, float *w2,
                         float *flux4, phd_clock *clocks, int32_t n_runs,
                         const int32_t *cell_run, cudaStream_t stream, cudaEvent_t *marks);

/* The same step with four caller-created events recorded on the stream around its
 * three stages (before gradients, before the face kernel, before the update, after),
 * so a caller can time each kernel inside a timed run; marks may be NULL. */
int phd_step_f32_marked(const phd_mesh *mesh, const phd_geom32 *geo, const phd_params *par,
                        int32_t moving, float *prim4, const double *cons, double *cons_next,
                        float *cellrec, float *w2, float *flux4, phd_clock *clk,
                        cudaStream_t stream, cudaEvent_t *marks);

/* ---- adjoint of one FP64 step ----------------------------------------------------
 * Reverse mode of U' = step(U) with the mesh, the face velocities and dt held fixed
 * (HLL / HLLC / exact -- the exact solver's p* by implicit differentiation of its
 * converged Newton root --, constant or linear reconstruction, both limiters).  Index
 * tables:
 *   partner [2F]          for each nbr_idx entry, the entry of the same face in the
 *                         other cell's list
 *   ghost_ptr [n_real+1], ghost_idx: the ghosts of each real cell (CSR by image).
 * Inputs: cons [4][n_cells] (ghost columns refreshed), prim and grad of that state
 * (as phd_prim_from_cons_f64 / phd_gradients_f64 produce them), face_w, dt, and
 * lam_next = dLoss/dU' [4][n_cells] (real columns).  Output lam = dLoss/dU (ghost
 * columns zero).  work: phd_adjoint_work_doubles(n_cells, n_faces) doubles. */
typedef struct phd_adj_index {
    const int32_t *partner;
    const int32_t *ghost_ptr;
    const int32_t *ghost_idx;
} phd_adj_index;

size_t phd_adjoint_work_doubles(int32_t n_cells, int32_t n_faces);
int phd_adjoint_step_f64(const phd_mesh *mesh, const phd_adj_index *index, const phd_params *par,
                         double dt, const double *cons, const double *prim, const double *grad,
                         const double *face_w, const double *lam_next, double *lam, double *work,
                         cudaStream_t stream);

/* phd_adjoint_step_f64 reading the limiter record that the taped forward step (or
 * phd_gradients_f64_taped) wrote for the same state, instead of recomputing the
 * limiter's selections. */
int phd_adjoint_step_f64_taped(const phd_mesh *mesh, const phd_adj_index *index,
                               const phd_params *par, double dt, const double *cons,
                               const double *prim, const double *grad, const double *face_w,
                               const double *lam_next, double *lam, double *work,
                               const double *tape_f64, const int32_t *tape_i32, cudaStream_t stream);

/* The same adjoint step for callers that cannot allocate device memory: a plugin
 * whose host program gives it no device allocator (a ctypes binding, or a process
 * whose device memory is owned by another framework's pool) can still run the
 * adjoint.  No counterpart in the reference (which has no adjoint).  The work space
 * is a fixed array compiled into the library (PHD_ADJ_NOALLOC_MAX_DOUBLES doubles =
 * 32 MiB, present on every GPU that loads the library until the process exits), so
 * the mesh must satisfy phd_adjoint_work_doubles(n_cells, n_faces) <=
 * PHD_ADJ_NOALLOC_MAX_DOUBLES -- about 36,000 cells in 2D at three faces per cell --
 * else PHD_ERR_SCRATCH_TOO_SMALL is returned and nothing runs.  Every call looks up
 * the array's device address for the device current at the call (so it stays right
 * after cudaDeviceReset or in another context); the first call on a device also loads
 * the library's device code there, so make it before any stream capture.  All calls
 * share the one array:
 * calls that overlap on the GPU (different streams, or two threads) race on it.
 * Nothing is allocated; the entries that must start at zero are cleared on the
 * stream by every call. */
#define PHD_ADJ_NOALLOC_MAX_DOUBLES 4194304
int phd_adjoint_step_f64_noalloc(const phd_mesh *mesh, const phd_adj_index *index,
                                 const phd_params *par, double dt, const double *cons,
                                 const double *prim, const double *grad, const double *face_w,
                                 const double *lam_next, double *lam, cudaStream_t stream);

/* ---- utilities ------------------------------------------------------------------ */

/* Reflective flip bits from ghost positions (boundary.pyx:287-307): bit k set when
 * type == Exterior and x_k lies outside [xmin_k, xmax_k].  xmin/xmax: host arrays. */
int phd_flip_mask(int32_t dim, int32_t n, const int8_t *type, const double *x,
                  const double *xmin, const double *xmax, int32_t reflective,
                  int8_t *flip, cudaStream_t stream);

/* hilbert_key_2d (hilbert.pyx:9-23) of positions quantised as in
 * LoadBalance.compute_hilbert_keys (load_balance.pyx:195-217). */
int phd_hilbert_keys_2d(int32_t n, const double *x, double corner_x, double corner_y,
                        double fac, int32_t order, int64_t *keys, cudaStream_t stream);

/* ---- quantities of an uploaded mesh derived on the device ------------------------
 * A host re-mesh hands over the face list (pair-i/j, area, centroid) and the cell
 * geometry every step; the normals and the neighbour lists follow from those, so the
 * device forms them instead of receiving them (Tess2d::extract_geometry tess.cpp:
 * 285-398 is where the reference forms them on the host). */

/* Face normals (x_j - x_i)/|x_j - x_i| (tess.cpp:320-327, 367-369) in IEEE
 * round-to-nearest FP64, bit-identical to the same formula evaluated on a host without
 * fused multiply-add.  normal: [2][n_faces].  Faces with out-of-range cells get a zero
 * normal and are counted into *bad (device int32, may be NULL). */
int phd_face_normals_f64(const phd_mesh *mesh, double *normal, int32_t *bad, cudaStream_t stream);

/* Neighbour lists (Mesh.neighbors mesh.pxd:34, filled at tess.cpp:378-379): for every
 * cell, the ids of the faces it belongs to in ascending order, as CSR nbr_ptr[n_cells+1],
 * nbr_idx[2*n_faces], from mesh->pair_i/pair_j only.  work: phd_csr_work_ints(n_cells)
 * device int32 of scratch.  Faces whose cells are out of range or equal are left out and
 * counted into *bad (device int32, may be NULL).  Deterministic: the same lists whatever
 * order the device visits the faces in. */
size_t phd_csr_work_ints(int32_t n_cells);
int phd_build_csr(const phd_mesh *mesh, int32_t *nbr_ptr, int32_t *nbr_idx, int32_t *work, int32_t *bad,
                  cudaStream_t stream);

/* Periodic twin table for phd_prepare_f32 (see phd_geom32): a boundary face emitted
 * from both sides (tess.cpp:363, mesh.pyx:529-544) as (i, ghost of k) and (k, ghost
 * of i) with opposite periodic shifts; twin[f] = the lower id for the higher-id copy f,
 * -1 elsewhere.  box_x/box_y: the periodic box lengths.  Needs mesh->map, x and the
 * neighbour lists.  periodic = 0 (reflective ghosts, whose mirror-image faces are
 * distinct faces) fills every entry with -1. */
int phd_periodic_twins(const phd_mesh *mesh, int32_t periodic, double box_x, double box_y,
                       int32_t *twin, cudaStream_t stream);

#ifdef __cplusplus
}
#endif
#endif /* PHDFLUX_H */
