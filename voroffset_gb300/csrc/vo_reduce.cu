// Xor volume of two volumes on the device (replaces the return value of
// VoronoiMorpho::calculateXor, src/vor3d/Voronoi.cpp:91-111, with
// calculate_ray_xor + removepoint, MorphologyOperators.cpp:334-374).
//
// Per column, a merge sweep over the endpoints of both (sorted, disjoint)
// lists yields the maximal runs where exactly one volume covers z; runs that
// meet at a point are one run (the reference's closed-interval union merges
// touching pieces), and runs shorter than 1e-10 are dropped like removepoint.
// Column lengths are summed per block and the block partials are added in a
// fixed order, so the result is deterministic.
#include "vo_internal.cuh"

namespace vo {
namespace {

constexpr int kThreads = 256;

__device__ double column_xor(const double2 *a, int na, const double2 *b, int nb) {
  int ina = 0, inb = 0;  // coverage state just above the current position
  bool run = false;
  double start = 0, len = 0;
  // Boundaries flip the coverage state; all boundaries at the same z are
  // processed together, so pieces meeting at a point form one run.
  int ia = 0, ib = 0;  // boundary index within each list (2 per segment)
  while (ia < 2 * na || ib < 2 * nb) {
    const double za = ia < 2 * na ? ((ia & 1) ? a[ia >> 1].y : a[ia >> 1].x) : INFINITY;
    const double zb = ib < 2 * nb ? ((ib & 1) ? b[ib >> 1].y : b[ib >> 1].x) : INFINITY;
    const double zc = za < zb ? za : zb;
    while (ia < 2 * na && ((ia & 1) ? a[ia >> 1].y : a[ia >> 1].x) == zc) {
      ina ^= 1;
      ++ia;
    }
    while (ib < 2 * nb && ((ib & 1) ? b[ib >> 1].y : b[ib >> 1].x) == zc) {
      inb ^= 1;
      ++ib;
    }
    const bool x = (ina ^ inb) != 0;
    if (x && !run) {
      run = true;
      start = zc;
    } else if (!x && run) {
      run = false;
      const double l = zc - start;
      if (!(l < 1e-10)) len += l;
    }
  }
  return len;
}

__global__ void k_xor(int ncols, const int32_t *__restrict__ oa, const double2 *__restrict__ za,
                      const int32_t *__restrict__ ob, const double2 *__restrict__ zb,
                      double *__restrict__ partial) {
  __shared__ double s[kThreads];
  const int c = blockIdx.x * kThreads + threadIdx.x;
  double v = 0;
  if (c < ncols) v = column_xor(za + oa[c], oa[c + 1] - oa[c], zb + ob[c], ob[c + 1] - ob[c]);
  s[threadIdx.x] = v;
  __syncthreads();
  for (int o = kThreads / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = s[0];
}

__global__ void k_sum(const double *partial, int n, double *out) {
  __shared__ double s[kThreads];
  double v = 0;
  for (int i = threadIdx.x; i < n; i += kThreads) v += partial[i];
  s[threadIdx.x] = v;
  __syncthreads();
  for (int o = kThreads / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = s[0];
}

}  // namespace
}  // namespace vo

using namespace vo;

extern "C" int vo_xor_volume(vo_ctx *ctx, const vo_volume *a, const vo_volume *b, double *volume) {
  if (!ctx) return VO_EINVAL;
  if (!a || !b || !volume) return set_error(ctx, VO_EINVAL, "xor: NULL argument");
  if (a->grid.nx != b->grid.nx || a->grid.ny != b->grid.ny)
    return set_error(ctx, VO_EINVAL, "xor: grids differ");
  cudaSetDevice(ctx->device);
  const int ncols = a->grid.nx * a->grid.ny;
  const int nblk = (ncols + kThreads - 1) / kThreads;
  double *partial = nullptr, *d_out = nullptr;
  int rc = dalloc(ctx, &partial, (size_t)nblk);
  if (!rc) rc = dalloc(ctx, &d_out, 1);
  if (rc) {
    dfree(ctx, partial);
    return rc;
  }
  k_xor<<<nblk, kThreads, 0, ctx->stream>>>(ncols, a->offs, a->z, b->offs, b->z, partial);
  k_sum<<<1, kThreads, 0, ctx->stream>>>(partial, nblk, d_out);
  double h = 0;
  cudaMemcpyAsync(&h, d_out, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
  dfree(ctx, partial);
  dfree(ctx, d_out);
  VO_CK(ctx, cudaStreamSynchronize(ctx->stream));
  const double sp = a->grid.spacing;
  *volume = sp * sp * sp * h;
  return VO_OK;
}
