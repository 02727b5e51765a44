// Mesh -> dexels by vertical ray casting on sm_103a (replaces create_dexels +
// compute_sign, src/vor3d/Dexelize.cpp:166-274).
//
//  1. host: bounding box, spacing and grid exactly as create_dexels
//     (Dexelize.cpp:254-271) and the CompressedVolume constructor
//     (CompressedVolume.cpp:11-23);
//  2. k_bin_count / scan / k_bin_fill: every facet is binned into the columns
//     whose centre may lie in its xy bounding box (a conservative superset;
//     the exact inclusive box test is repeated per column, so the candidate
//     set equals geogram's AABB box query);
//  3. k_cast<FILL>: per column, the SOS-robust inside test and barycentric z
//     of Dexelize.cpp:56-162, hits divided by the spacing, sorted, counted
//     then written (count -> scan -> fill).
// All FP64 products/sums use explicit round-to-nearest intrinsics so nothing
// is contracted into FMA: results equal the reference's x86 FP64 arithmetic.
#include <algorithm>
#include <cmath>
#include <vector>

#include "vo_internal.cuh"

namespace vo {
namespace {

constexpr int kHitCap = 64;       // hits per column in the fast kernel
constexpr int kHitCapBig = 4096;  // hits per column in the overflow re-run

__device__ __forceinline__ double mul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double sub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double add(double a, double b) { return __dadd_rn(a, b); }

// orientation (Dexelize.cpp:56-67)
__device__ int orientation(double x1, double y1, double x2, double y2, double &tsa) {
  tsa = sub(mul(y1, x2), mul(x1, y2));
  if (tsa > 0) return 1;
  if (tsa < 0) return -1;
  if (y2 > y1) return 1;
  if (y2 < y1) return -1;
  if (x1 > x2) return 1;
  if (x1 < x2) return -1;
  return 0;
}

// point_in_triangle_2d (Dexelize.cpp:73-92) + intersect_ray_z (:137-162).
__device__ bool ray_hit(double qx, double qy, double3 p1, double3 p2, double3 p3, double &z) {
  const double x1 = sub(p1.x, qx), x2 = sub(p2.x, qx), x3 = sub(p3.x, qx);
  const double y1 = sub(p1.y, qy), y2 = sub(p2.y, qy), y3 = sub(p3.y, qy);
  double a, b, c;
  const int sa = orientation(x2, y2, x3, y3, a);
  if (sa == 0) return false;
  const int sb = orientation(x3, y3, x1, y1, b);
  if (sb != sa) return false;
  const int sc = orientation(x1, y1, x2, y2, c);
  if (sc != sa) return false;
  const double sum = add(add(a, b), c);
  a = __ddiv_rn(a, sum);
  b = __ddiv_rn(b, sum);
  c = __ddiv_rn(c, sum);
  z = add(add(mul(a, p1.z), mul(b, p2.z)), mul(c, p3.z));
  // orient_2d_inexact (Dexelize.cpp:107-121): a hit counts only for a
  // non-degenerate projected triangle.
  const double a11 = sub(p2.x, p1.x), a12 = sub(p2.y, p1.y);
  const double a21 = sub(p3.x, p1.x), a22 = sub(p3.y, p1.y);
  const double delta = sub(mul(a11, a22), mul(a12, a21));
  return delta != 0;
}

struct Mesh {
  const double3 *v;
  const int3 *f;
  int nt;
};

struct GridView {
  int nx, ny;
  double ox, oy, h;
};

__device__ void facet_range(const Mesh &m, const GridView &g, int f, int &x0, int &x1, int &y0,
                            int &y1) {
  const int3 t = m.f[f];
  const double3 a = m.v[t.x], b = m.v[t.y], c = m.v[t.z];
  const double lx = fmin(a.x, fmin(b.x, c.x)), hx = fmax(a.x, fmax(b.x, c.x));
  const double ly = fmin(a.y, fmin(b.y, c.y)), hy = fmax(a.y, fmax(b.y, c.y));
  x0 = (int)floor((lx - g.ox) / g.h - 0.5) - 1;
  x1 = (int)ceil((hx - g.ox) / g.h - 0.5) + 1;
  y0 = (int)floor((ly - g.oy) / g.h - 0.5) - 1;
  y1 = (int)ceil((hy - g.oy) / g.h - 0.5) + 1;
  x0 = max(x0, 0);
  y0 = max(y0, 0);
  x1 = min(x1, g.nx - 1);
  y1 = min(y1, g.ny - 1);
}

__global__ void k_bin_count(Mesh m, GridView g, int32_t *cnt) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= m.nt) return;
  int x0, x1, y0, y1;
  facet_range(m, g, f, x0, x1, y0, y1);
  for (int y = y0; y <= y1; ++y)
    for (int x = x0; x <= x1; ++x) atomicAdd(&cnt[x + g.nx * y], 1);
}

__global__ void k_bin_fill(Mesh m, GridView g, const int32_t *boffs, int32_t *cursor, int32_t *bins) {
  const int f = blockIdx.x * blockDim.x + threadIdx.x;
  if (f >= m.nt) return;
  int x0, x1, y0, y1;
  facet_range(m, g, f, x0, x1, y0, y1);
  for (int y = y0; y <= y1; ++y)
    for (int x = x0; x <= x1; ++x) {
      const int c = x + g.nx * y;
      bins[boffs[c] + atomicAdd(&cursor[c], 1)] = f;
    }
}

// Returns the number of hits of column c (the FILL pass writes the first
// 2 * (hits / 2) of them: an unpaired trailing hit is dropped), or -1 on overflow.
template <bool FILL>
__device__ int cast_column(const Mesh &m, const GridView &g, const int32_t *boffs, const int32_t *bins,
                           int c, double *hits, int cap, double *out) {
  const int x = c % g.nx, y = c / g.nx;
  // dexelCenter (CompressedVolumeBase.cpp:5-11)
  const double cx = add(mul(x + 0.5, g.h), g.ox);
  const double cy = add(mul(y + 0.5, g.h), g.oy);
  int nh = 0;
  for (int k = boffs[c]; k < boffs[c + 1]; ++k) {
    const int3 t = m.f[bins[k]];
    const double3 a = m.v[t.x], b = m.v[t.y], cc = m.v[t.z];
    const double lx = fmin(a.x, fmin(b.x, cc.x)), hx = fmax(a.x, fmax(b.x, cc.x));
    const double ly = fmin(a.y, fmin(b.y, cc.y)), hy = fmax(a.y, fmax(b.y, cc.y));
    if (cx < lx || cx > hx || cy < ly || cy > hy) continue;
    double z;
    if (ray_hit(cx, cy, a, b, cc, z)) {
      if (nh >= cap) return -1;
      // insertion into a sorted list (std::sort of the hits, Dexelize.cpp:208)
      const double v = __ddiv_rn(z, g.h);
      int i = nh++;
      while (i > 0 && hits[i - 1] > v) {
        hits[i] = hits[i - 1];
        --i;
      }
      hits[i] = v;
    }
  }
  const int raw = nh;
  nh &= ~1;  // an unpaired trailing hit is ignored (values are consumed in pairs)
  if (FILL)
    for (int i = 0; i < nh; ++i) out[i] = hits[i];
  return raw;
}

template <bool FILL>
__global__ void k_cast(Mesh m, GridView g, const int32_t *boffs, const int32_t *bins, int32_t *counts,
                       const int32_t *ooffs, double *oz, int *ovf_count, int *ovf_cols) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= g.nx * g.ny) return;
  double hits[kHitCap];
  const int n = cast_column<FILL>(m, g, boffs, bins, c, hits, kHitCap,
                                  FILL ? oz + 2 * (size_t)ooffs[c] : nullptr);
  if (!FILL) {
    if (n < 0) {
      ovf_cols[atomicAdd(ovf_count, 1)] = c;
      counts[c] = 0;
    } else {
      counts[c] = n / 2;
      if (n & 1) atomicAdd(ovf_count + 2, 1);  // odd columns (the flag word after the two status words)
    }
  }
}

template <bool FILL>
__global__ void k_cast_big(Mesh m, GridView g, const int32_t *boffs, const int32_t *bins,
                           int32_t *counts, const int32_t *ooffs, double *oz, const int *ovf_count,
                           const int *ovf_cols, double *scratch, int *fatal) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;
  double *hits = scratch + (size_t)tid * kHitCapBig;
  for (int i = tid; i < *ovf_count; i += nth) {
    const int c = ovf_cols[i];
    const int n = cast_column<FILL>(m, g, boffs, bins, c, hits, kHitCapBig,
                                    FILL ? oz + 2 * (size_t)ooffs[c] : nullptr);
    if (n < 0) *fatal = 1;
    if (!FILL) {
      counts[c] = n < 0 ? 0 : n / 2;
      if (n > 0 && (n & 1)) atomicAdd(fatal + 1, 1);  // odd columns, as in k_cast
    }
  }
}

}  // namespace
}  // namespace vo

using namespace vo;

extern "C" int vo_dexelize_odd_columns(vo_ctx *ctx, int64_t *count) {
  if (!ctx || !count) return VO_EINVAL;
  if (ctx->dexel_odd_columns < 0) return set_error(ctx, VO_EINVAL, "no successful vo_dexelize on this context");
  *count = ctx->dexel_odd_columns;
  return VO_OK;
}

extern "C" int vo_dexelize(vo_ctx *ctx, const double *verts, int nv, const int32_t *tris, int nt,
                           double *spacing, int padding, int num_dexels, vo_volume **out) {
  if (!ctx) return VO_EINVAL;
  if (!verts || nv <= 0 || nt < 0 || (nt > 0 && !tris) || !spacing || !out || padding < 0)
    return set_error(ctx, VO_EINVAL, "dexelize: bad arguments");
  for (int64_t i = 0; i < 3 * (int64_t)nt; ++i)
    if (tris[i] < 0 || tris[i] >= nv) return set_error(ctx, VO_EINVAL, "dexelize: vertex index out of range");
  cudaSetDevice(ctx->device);
  ctx->err.clear();
  ctx->dexel_odd_columns = -1;
  *out = nullptr;
  // create_dexels (Dexelize.cpp:254-271)
  double mn[3], mx[3];
  for (int k = 0; k < 3; ++k) mn[k] = mx[k] = verts[k];
  for (int i = 1; i < nv; ++i)
    for (int k = 0; k < 3; ++k) {
      mn[k] = std::min(mn[k], verts[3 * i + k]);
      mx[k] = std::max(mx[k], verts[3 * i + k]);
    }
  const double ext[3] = {mx[0] - mn[0], mx[1] - mn[1], mx[2] - mn[2]};
  if (num_dexels > 0) *spacing = std::max(ext[0], std::max(ext[1], ext[2])) / num_dexels;
  const double h = *spacing;
  if (!(h > 0) || !std::isfinite(h)) return set_error(ctx, VO_EINVAL, "dexelize: spacing must be > 0");
  vo_grid g;
  g.spacing = h;
  g.padding = padding;
  for (int k = 0; k < 3; ++k) {
    g.origin[k] = mn[k] - padding * h;
    g.extent[k] = ext[k];
  }
  const double fnx = std::ceil(ext[0] / h) + 2 * padding, fny = std::ceil(ext[1] / h) + 2 * padding;
  if (fnx * fny > 2e9) return set_error(ctx, VO_ERANGE, "dexelize: grid too large");
  g.nx = (int)fnx;
  g.ny = (int)fny;
  const int ncols = g.nx * g.ny;

  double3 *dv = nullptr;
  int3 *df = nullptr;
  int32_t *cnt = nullptr, *boffs = nullptr, *cursor = nullptr, *bins = nullptr, *ovf_cols = nullptr;
  double *big = nullptr;
  vo_volume *res = nullptr;
  long long nb = 0, total = 0;
  int rc = dalloc(ctx, &dv, (size_t)nv);
  if (!rc) rc = dalloc(ctx, &df, (size_t)std::max(nt, 1));
  if (!rc) rc = dalloc(ctx, &cnt, (size_t)ncols);
  if (!rc) rc = dalloc(ctx, &boffs, (size_t)ncols + 1);
  if (!rc) rc = dalloc(ctx, &cursor, (size_t)ncols);
  if (!rc) rc = dalloc(ctx, &ovf_cols, (size_t)ncols);
  const int gbig = 148 * 4;
  if (!rc) rc = dalloc(ctx, &big, (size_t)gbig * 32 * kHitCapBig);
  Mesh m{dv, df, nt};
  GridView gv{g.nx, g.ny, g.origin[0], g.origin[1], h};
  if (!rc) {
    cudaMemcpyAsync(dv, verts, sizeof(double) * 3 * (size_t)nv, cudaMemcpyHostToDevice, ctx->stream);
    if (nt) cudaMemcpyAsync(df, tris, sizeof(int32_t) * 3 * (size_t)nt, cudaMemcpyHostToDevice, ctx->stream);
    cudaMemsetAsync(cnt, 0, sizeof(int32_t) * ncols, ctx->stream);
    cudaMemsetAsync(cursor, 0, sizeof(int32_t) * ncols, ctx->stream);
    cudaMemsetAsync(ctx->d_flags, 0, 3 * sizeof(int), ctx->stream);  // overflow count, fatal, odd columns
    if (nt) k_bin_count<<<(nt + 127) / 128, 128, 0, ctx->stream>>>(m, gv, cnt);
    rc = scan_counts(ctx, cnt, boffs, ncols, &nb);
  }
  if (!rc) rc = dalloc(ctx, &bins, (size_t)nb);
  if (!rc) {
    if (nt) k_bin_fill<<<(nt + 127) / 128, 128, 0, ctx->stream>>>(m, gv, boffs, cursor, bins);
    k_cast<false><<<(ncols + 127) / 128, 128, 0, ctx->stream>>>(m, gv, boffs, bins, cnt, nullptr, nullptr,
                                                                ctx->d_flags, ovf_cols);
    k_cast_big<false><<<gbig, 32, 0, ctx->stream>>>(m, gv, boffs, bins, cnt, nullptr, nullptr,
                                                    ctx->d_flags, ovf_cols, big, ctx->d_flags + 1);
    rc = volume_alloc(ctx, g, 0, &res);
  }
  if (!rc) rc = scan_counts(ctx, cnt, res->offs, ncols, &total);
  if (!rc) {
    res->nseg = total;
    rc = dalloc(ctx, &res->z, (size_t)total);
  }
  if (!rc) {
    k_cast<true><<<(ncols + 127) / 128, 128, 0, ctx->stream>>>(m, gv, boffs, bins, nullptr, res->offs,
                                                               (double *)res->z, ctx->d_flags, ovf_cols);
    k_cast_big<true><<<gbig, 32, 0, ctx->stream>>>(m, gv, boffs, bins, nullptr, res->offs, (double *)res->z,
                                                   ctx->d_flags, ovf_cols, big, ctx->d_flags + 1);
    int hf[3] = {0, 0, 0};
    cudaMemcpyAsync(hf, ctx->d_flags, sizeof(hf), cudaMemcpyDeviceToHost, ctx->stream);
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess)
      rc = cuda_error(ctx, e, "dexelize");
    else if (hf[1])
      rc = set_error(ctx, VO_EINTERNAL, "dexelize: a column has more than 4096 hits");
    else
      ctx->dexel_odd_columns = hf[2];
  }
  dfree(ctx, dv);
  dfree(ctx, df);
  dfree(ctx, cnt);
  dfree(ctx, boffs);
  dfree(ctx, cursor);
  dfree(ctx, bins);
  dfree(ctx, ovf_cols);
  dfree(ctx, big);
  if (rc) {
    if (res) vo_volume_free(ctx, res);
    return rc;
  }
  cudaError_t e = cudaStreamSynchronize(ctx->stream);
  if (e != cudaSuccess) {
    vo_volume_free(ctx, res);
    return cuda_error(ctx, e, "dexelize");
  }
  *out = res;
  return VO_OK;
}
