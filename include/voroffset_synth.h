/*
 * voroffset_synth.h -- seeded synthetic inputs for the dexel morphology path.
 *
 * Host-only C library (libvoroffset_synth.so), kept apart from the GPU
 * library: it makes the benchmark's and the tests' input volumes and meshes
 * and has no reference counterpart. The random stream is splitmix64, so every
 * input is reproducible from its seed on any machine. Status codes are the
 * VO_* codes of voroffset_gpu.h.
 */
#ifndef VOROFFSET_SYNTH_H
#define VOROFFSET_SYNTH_H
#include <stdint.h>

#include "voroffset_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Seeded synthetic volume: union of spheres and flat-capped cylinders
 * evaluated at dexel centres, clipped to [0, zmax], merged per column. */
typedef struct {
  int32_t nx, ny;
  double zmax;
  int32_t n_spheres;
  int32_t sphere_dist; /* 0: radius uniform in [s_rmin, s_rmax]; 1: lognormal(s_median, s_sigma) clipped */
  double s_rmin, s_rmax, s_median, s_sigma;
  int32_t n_cyl; /* endpoints uniform in the box, radius uniform in [c_rmin, c_rmax] */
  double c_rmin, c_rmax;
  uint64_t seed;
} vo_synth_params;
/* offs: caller array of nx*ny+1; *z is allocated (free with vo_host_free). */
int vo_synth_volume(const vo_synth_params *p, int32_t *offs, double **z, int64_t *nseg);
/* Watertight torus centred at (0.5,0.5,0.5), nu x nv quads split in triangles,
 * vertices displaced along the normal by uniform noise in [-noise, noise]. */
int vo_synth_torus(int nu, int nv, double major, double minor, double noise, uint64_t seed,
                   double **verts, int *nverts, int32_t **tris, int *ntris);
void vo_host_free(void *p);

#ifdef __cplusplus
}
#endif
#endif
