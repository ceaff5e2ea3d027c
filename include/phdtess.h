/* phdtess.h -- host 2D Delaunay / Voronoi tessellation in the reference's mesh
 * conventions (C ABI of libphdtess.so).
 *
 * Replaces the CGAL-backed Tess2d of the reference (phd/mesh/tess.h:53-72,
 * phd/mesh/tess.cpp) on the host side of the flux path: the same method set
 * (build_initial_tess, update_initial_tess, count_number_of_faces,
 * extract_geometry, update_radius) over plain arrays, plus one call that builds a
 * whole mesh -- real cells, ghost images for a periodic or reflective box, faces,
 * volumes, centroid offsets and per-cell face lists -- in the layout the flux path
 * uploads.
 *
 * Conventions (tess.cpp:238-398): faces are emitted per real cell i, for each
 * Voronoi edge shared with a neighbour j > i, in counter-clockwise order of the
 * neighbour direction starting at angle -pi; area = edge length, com = edge
 * midpoint, normal = (x_j - x_i)/|x_j - x_i|; cell volume = sum of 0.25*area*h over
 * incident edges, dcom = (sum of 0.25*area*h*(2/3 f + 1/3 x))/vol - x (eqs. 27-31);
 * every cell's face list holds face ids in ascending order.
 *
 * Return codes: >= 0 success (a count where stated), -1 incomplete tessellation
 * (a real cell touches the hull: more ghosts are needed), -2 bad argument,
 * -3 duplicate generator, -4 out of memory / internal failure.
 */
#ifndef PHDTESS_H
#define PHDTESS_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct phd_tess2d phd_tess2d;

/* Tess2d::Tess2d / reset_tess (tess.cpp:22-33). */
phd_tess2d *phd_tess2d_create(void);
void phd_tess2d_destroy(phd_tess2d *t);

/* Tess2d::build_initial_tess (tess.cpp:35-142): Delaunay tessellation of the
 * n_real generators (x[i], y[i]); radius[i] = twice the largest distance from
 * generator i to its Voronoi vertices, or -1 where the Voronoi cell is unbounded.
 * radius may be NULL. */
int phd_tess2d_build_initial(phd_tess2d *t, const double *x, const double *y, int n_real, double *radius);

/* Tess2d::update_initial_tess (tess.cpp:144-187): insert generators begin..end-1
 * (ghosts), read from x[begin..end), y[begin..end). */
int phd_tess2d_update_initial(phd_tess2d *t, const double *x, const double *y, int begin, int end);

/* Tess2d::count_number_of_faces (tess.cpp:189-236): faces owned by real cells, or -1
 * while a real cell is unbounded. */
int phd_tess2d_count_faces(phd_tess2d *t);

/* Tess2d::update_radius (tess.cpp:400-470), for the listed generators:
 * radius[ids[k]] = twice the largest distance to the Voronoi vertices, or -1 while
 * unbounded.  Returns how many of them are still unbounded. */
int phd_tess2d_update_radius(phd_tess2d *t, const int32_t *ids, int n_ids, double *radius);

/* Tess2d::extract_geometry (tess.cpp:238-398).  Writes volume / dcom of the real
 * cells, the face arrays (length count_faces), and the per-cell face lists as CSR
 * over all inserted generators: nbr_ptr[n_total + 1], nbr_idx[2 * n_faces].
 * Returns the number of faces. */
int phd_tess2d_extract_geometry(phd_tess2d *t, double *dcom_x, double *dcom_y, double *volume, double *face_area,
                                double *com_x, double *com_y, double *normal_x, double *normal_y, int32_t *pair_i,
                                int32_t *pair_j, int32_t *nbr_ptr, int32_t *nbr_idx);

/* Whole mesh of a box [xmin, xmax] (Mesh.tessellate + Mesh.build_geometry,
 * mesh.pyx:188-330): ghosts are the images of the real generators within `pad` of
 * the box (periodic: the 8 shifted copies in shift order (-1,-1), (-1,0), ...,
 * (1,1); reflective: mirror images across each wall, x-low, x-high, y-low,
 * y-high), each group in real-index order; `pad` doubles (up to 6 attempts) while
 * a real cell is unbounded; ghosts sharing no face with a real cell are dropped.
 * boundary: 0 periodic, 1 reflective.  The result stays in the handle: read its
 * sizes with phd_mesh2d_sizes and copy it out with phd_mesh2d_copy. */
int phd_mesh2d_build(phd_tess2d *t, const double *x, const double *y, int n_real, int boundary, double xmin0,
                     double xmin1, double xmax0, double xmax1, double pad);

/* phd_mesh2d_build with the real cells' extraction split into n_strips strips (by the
 * generators' x quantiles) tessellated on parallel host threads; 0 chooses by the
 * number of real cells (1 below 65,536, at most 16).  A strip tessellates every
 * generator within a halo of it and keeps only triangles whose circumcircles lie inside
 * the x-range its generators cover (widening the halo until they do), so the result is
 * the whole box's tessellation; circumcentres are formed in a canonical vertex order,
 * so faces do not depend on the strip that formed them. */
int phd_mesh2d_build_strips(phd_tess2d *t, const double *x, const double *y, int n_real, int boundary,
                            double xmin0, double xmin1, double xmax0, double xmax1, double pad, int n_strips);

/* n_cells (real + kept ghosts), n_faces, and the pad the last build used. */
int phd_mesh2d_sizes(const phd_tess2d *t, int32_t *n_cells, int32_t *n_faces, double *pad_used);

/* Copy the last phd_mesh2d_build result: positions x/y[n_cells], image map[n_cells]
 * (own index for real cells), vol[n_cells], dcom_x/y[n_cells] (ghosts take their
 * image's), face arrays [n_faces], CSR nbr_ptr[n_cells + 1], nbr_idx[2 n_faces]. */
int phd_mesh2d_copy(const phd_tess2d *t, double *x, double *y, int32_t *map, double *vol, double *dcom_x,
                    double *dcom_y, int32_t *pair_i, int32_t *pair_j, double *area, double *com_x, double *com_y,
                    double *normal_x, double *normal_y, int32_t *nbr_ptr, int32_t *nbr_idx);

/* The last phd_mesh2d_build result as the flux path's compact FP32 hand-over
 * (phd_pair_i_from_face_ptr / phd_prepare_f32_faces_compact of phdflux.h): per-real-cell
 * face ranges face_ptr[n_real + 1], pair_j[n_faces], the area and the centroid offset
 * along the face (formed in FP64 as phdflux.h's compact hand-over states) rounded to
 * FP32 -- area32[n_faces], ct32[n_faces] -- and the cells' positions x[2][n_cells] (x row then y row), image
 * map, tags (Real 0 / Ghost 1) and types (Undefined 4 for real cells, Exterior 2 for
 * ghosts), written into caller buffers (e.g. pinned host memory reused across steps).
 * x may be NULL (the device already holds the real cells' positions, e.g. from its own
 * generator move); ghost_code[n_cells - n_real] (may be NULL) says how each ghost images
 * its real cell, so the device can form the ghost positions itself
 * (phd_ghost_positions of phdflux.h): 1 + 3 (sx + 1) + (sy + 1) for a periodic copy
 * shifted by (sx, sy) box lengths, 16 + 2 k + h for a mirror image across axis k at its
 * low (h = 0) or high (h = 1) wall. */
int phd_mesh2d_copy_compact(const phd_tess2d *t, int32_t *face_ptr, int32_t *pair_j, float *area32, float *ct32,
                            double *x, int32_t *map, int8_t *tag, int8_t *type, int8_t *ghost_code);

/* phd_mesh2d_copy_compact with pair-j packed (phdflux.h, phd_handover32.pair_dj) and
 * the area and offset interleaved, one (area, offset) pair per face in face32[n_faces][2]:
 * pair_dj[f] = pair_j - pair_i where that lies in [1, 65534], else PHD_PAIR16_ESCAPE,
 * and the escaped faces as (face id, pair-j) pairs in ascending face id in
 * pair_x[2 x_cap]; *n_pair_x receives their number.  Returns -5 (everything but
 * list_len written) when that number exceeds x_cap: call again with x_cap >= *n_pair_x.
 * list_len[n_cells] (may be NULL) receives each cell's number of faces (its neighbour
 * list's length); -6 (everything else written) when one exceeds 255. */
#ifndef PHD_PAIR16_ESCAPE
#define PHD_PAIR16_ESCAPE 0       /* also in phdflux.h */
#endif
int phd_mesh2d_copy_compact16(const phd_tess2d *t, int32_t *face_ptr, uint16_t *pair_dj, int32_t *pair_x,
                              int32_t x_cap, int32_t *n_pair_x, uint8_t *list_len, float *face32, double *x,
                              int32_t *map, int8_t *tag, int8_t *type, int8_t *ghost_code);

/* hilbert_key_2d (phd/hilbert/hilbert.pyx:9-23) for n integer coordinate pairs. */
void phd_hilbert_keys_2d_host(const int32_t *xh, const int32_t *yh, int64_t n, int order, int64_t *keys);

#ifdef __cplusplus
}
#endif

#endif
