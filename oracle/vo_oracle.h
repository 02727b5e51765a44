/*
 * vo_oracle.h -- CPU oracle for the Voroffset 3D dexel morphology path.
 *
 * TEST INFRASTRUCTURE ONLY. This is a plain-C restatement of the reference's
 * algorithm (geometryprocessing/voroffset, src/vor3d) used as the checker for
 * the CUDA path: only tests/, __graft_entry__.smoke() and bench.py's CPU
 * baseline leg may load it. The product never calls it and has no CPU fallback.
 *
 * Volumes are CSR: offs[nx*ny+1] (int32, in segments) and z[2*nseg] (FP64
 * pairs z1 <= z2, sorted and disjoint per column, dexel units). Column index
 * c = x + nx*y (CompressedVolume.h:28-29).
 */
#ifndef VO_ORACLE_H
#define VO_ORACLE_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
  int nx, ny;
  double origin[3]; /* stored origin (already shifted by -padding*spacing) */
  double extent[3];
  double spacing;
  int padding;
} vo_or_grid;

typedef struct {
  int32_t *offs; /* nx*ny+1 */
  double *z;     /* 2*offs[nx*ny] */
} vo_or_csr;

/* Status codes. */
#define VO_OR_OK 0
#define VO_OR_EINVAL -1
#define VO_OR_ENOMEM -2
#define VO_OR_ERADIUS -3 /* radius whose lattice reach depends on position */

/* Separable ("ours") dilation semantics, restated as an exact union. */
int vo_or_dilate(const vo_or_grid *g, const vo_or_csr *in, double radius, int nthreads,
                 vo_or_csr *out, double *t1_ms, double *t2_ms);
/* Separable dilation of selected output columns only (out CSR has ncols_sel+1 offsets). */
int vo_or_dilate_columns(const vo_or_grid *g, const vo_or_csr *in, double radius, const int32_t *cols,
                         int ncols_sel, int nthreads, vo_or_csr *out);
/* Any op (0 dilation, 1 erosion, 2 opening, 3 closing; separable method) at the
 * selected output columns only (out CSR has ncols_sel+1 offsets). */
int vo_or_morph_columns(int op, const vo_or_grid *g, const vo_or_csr *in, double radius, const int32_t *cols,
                        int ncols_sel, int nthreads, vo_or_csr *out);
/* Brute-force lattice-disc dilation (VoronoiBruteForce.cpp:16-100). */
int vo_or_dilate_brute(const vo_or_grid *g, const vo_or_csr *in, double radius, int nthreads,
                       vo_or_csr *out);
/* op: 0 dilation, 1 erosion, 2 opening, 3 closing; method: 0 separable, 1 brute. */
int vo_or_morph(int method, int op, const vo_or_grid *g, const vo_or_csr *in, double radius,
                int nthreads, vo_or_csr *out);
/* 2D images (src/vor2d CompressedImage): op 0 dilate, 1 erode, 2 open, 3 close of
 * an image of `height` rows of `width` pixels, rows as half-open span events in
 * CSR form (offs[height + 1] counts events). */
int vo_or_image_morph(int op, int width, int height, const int32_t *offs, const int32_t *events, double radius,
                      int32_t **out_offs, int32_t **out_events);
/* The FP64 twin (DoubleCompressedImage): rows of closed spans with FP64 events;
 * dilate scales the radius by the row count, erode does not. */
int vo_or_image_morph_f64(int op, int width, int height, const int32_t *offs, const double *events, double radius,
                          int32_t **out_offs, double **out_events);
/* Xor volume (Voronoi.cpp:91-111). */
double vo_or_xor_volume(const vo_or_grid *g, const vo_or_csr *a, const vo_or_csr *b);
double vo_or_get_volume(const vo_or_grid *g, const vo_or_csr *a);

/* Pass-1 intermediate statistics for one radius: total pieces over all columns. */
int64_t vo_or_pass1_pieces(const vo_or_grid *g, const vo_or_csr *in, double radius, int nthreads);

/* Mesh -> dexels (Dexelize.cpp:56-274). verts[3*nv], tris[3*nt].
 * num_dexels > 0 sets spacing = max_extent / num_dexels; otherwise *spacing is used.
 * Fills g (grid) and out. */
int vo_or_dexelize(const double *verts, int nv, const int32_t *tris, int nt, double *spacing,
                   int padding, int num_dexels, vo_or_grid *g, vo_or_csr *out);

void vo_or_free(void *p);

#ifdef __cplusplus
}
#endif
#endif
