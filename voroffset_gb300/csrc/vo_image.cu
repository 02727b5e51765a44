// 2D morphology of pixel images (the reference's src/vor2d CompressedImage:
// dilate, erode, open, close, CompressedImage.cpp:608-647).
//
// An image is `height` rows of `width` pixels; row i is a sorted list of
// half-open pixel spans given as events [a0, b0, a1, b1, ...]. The reference
// sweeps the rows with a Voronoi diagram of segments (Voronoi.cpp); its result
// is the lattice union below, which is what the kernels compute:
//
// * dilate: row i is the union over rows i0 with t = |i - i0| <= floor(r) of the
//   spans [a, b) of row i0 widened to [max(a - dy, 0), min(b + dy, width)),
//   dy = floor(sqrt(r*r - t*t)) in the reference's FP64 expression
//   (VoronoiMorpho::getLine, Voronoi.cpp:749-759); touching spans merge.
// * erode: the complement, within [0, width), of the same union taken over the
//   complement spans of every row with one border pixel on each side and a
//   full extra row before the first and after the last row (voronoi_half_erode,
//   Voronoi.h:126-150, then negate, CompressedImage.cpp:366-397).
//
// One block per output row: each candidate span adds +1 / -1 at its ends in a
// shared-memory difference array, a block prefix sum gives the coverage, and a
// block scan of the coverage changes places the output events. A count launch
// sizes the CSR output, a fill launch writes it.
#include <algorithm>
#include <cmath>
#include <vector>

#include "vo_internal.cuh"

namespace vo {
namespace {

constexpr int kImgThreads = 256;
constexpr int kImgMaxWidth = 50000;  // the difference array lives in shared memory

__device__ __forceinline__ void img_add(int32_t *diff, int w, long long lo, long long hi) {
  if (lo < 0) lo = 0;
  if (hi > w) hi = w;
  if (lo >= hi) return;
  atomicAdd(&diff[lo], 1);
  atomicAdd(&diff[hi], -1);
}

template <bool FILL>
__global__ void __launch_bounds__(kImgThreads) k_image(int w, int h, const int32_t *__restrict__ offs,
                                                       const int32_t *__restrict__ ev, double r, int D, int erode,
                                                       int32_t *__restrict__ counts, const int32_t *__restrict__ ooffs,
                                                       int32_t *__restrict__ oev) {
  extern __shared__ int32_t diff[];  // [w + 1]
  __shared__ int wsum[kImgThreads / 32];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  for (int i = blockIdx.x; i < h; i += gridDim.x) {
    for (int p = tid; p <= w; p += kImgThreads) diff[p] = 0;
    __syncthreads();
    // rows beyond the image and its two border rows contribute nothing
    for (int i0 = max(i - D, -1); i0 <= min(i + D, h); ++i0) {
      const int t = i0 < i ? i - i0 : i0 - i;
      if (erode && (i0 == -1 || i0 == h)) {  // the extra full row
        if (tid == 0) img_add(diff, w, 0, w);
        continue;
      }
      if (i0 < 0 || i0 >= h) continue;
      const long long dy = (long long)floor(sqrt(r * r - (double)((long long)t * t)));
      const int32_t *e = ev + offs[i0];
      const int n = offs[i0 + 1] - offs[i0];
      if (!erode) {
        for (int k = 2 * tid; k + 1 < n; k += 2 * kImgThreads) img_add(diff, w, e[k] - dy, e[k + 1] + dy);
      } else {
        // complement spans [-1, a0 - 1], [b0, a1 - 1], ..., [b_last, w] (inclusive), widened
        for (int q = tid; q <= n / 2; q += kImgThreads) {
          const long long y1 = q == 0 ? -1 : e[2 * q - 1];
          const long long y2e = q == n / 2 ? (long long)w + 1 : e[2 * q];  // one past the span's last pixel
          img_add(diff, w, y1 - dy, y2e + dy);
        }
      }
    }
    __syncthreads();
    // coverage: prefix sums of diff over contiguous chunks of [0, w]
    const int L = (w + 1 + kImgThreads - 1) / kImgThreads;
    const int p0 = min(w + 1, tid * L), p1 = min(w + 1, p0 + L);
    int local = 0;
    for (int p = p0; p < p1; ++p) local += diff[p];
    int x = local;
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) wsum[warp] = x;
    __syncthreads();
    int pre = 0;
    for (int k = 0; k < warp; ++k) pre += wsum[k];
    __syncthreads();
    // events: positions p in [0, w] where the output flag changes (flag(-1) = flag(w) = 0)
    auto flag = [&](int p, int cov) -> int { return p < w ? (erode ? (cov <= 0) : (cov > 0)) : 0; };
    int cov = pre + x - local;  // coverage just before p0
    int prevf = p0 > 0 ? flag(p0 - 1, cov) : 0;
    int nev = 0;
    {
      int c2 = cov, pf = prevf;
      for (int p = p0; p < p1; ++p) {
        c2 += diff[p];
        const int f = flag(p, c2);
        nev += f != pf;
        pf = f;
      }
    }
    // exclusive sum of event counts over the threads
    int y = nev;
    for (int o = 1; o < 32; o <<= 1) {
      const int v = __shfl_up_sync(0xffffffffu, y, o);
      if (lane >= o) y += v;
    }
    if (lane == 31) wsum[warp] = y;
    __syncthreads();
    int base = 0, total = 0;
    for (int k = 0; k < kImgThreads / 32; ++k) {
      if (k < warp) base += wsum[k];
      total += wsum[k];
    }
    base += y - nev;
    if (!FILL) {
      if (tid == 0) counts[i] = total;
    } else {
      int c2 = cov, pf = prevf, o = ooffs[i] + base;
      for (int p = p0; p < p1; ++p) {
        c2 += diff[p];
        const int f = flag(p, c2);
        if (f != pf) oev[o++] = p;
        pf = f;
      }
    }
    __syncthreads();
  }
}

int image_op(vo_ctx *ctx, int erode, double r, int w, int h, const int32_t *offs, const int32_t *ev, int32_t **ooffs,
             int32_t **oev, long long *total) {
  const int D = (int)std::floor(r);
  int32_t *counts = nullptr;
  *ooffs = nullptr;
  *oev = nullptr;
  int rc = dalloc(ctx, &counts, (size_t)h + 1);
  if (!rc) rc = dalloc(ctx, ooffs, (size_t)h + 1);
  const size_t sh = sizeof(int32_t) * ((size_t)w + 1);
  const int grid = std::min(h, 152 * 8);
  if (!rc) {
    cudaFuncSetAttribute(k_image<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sh);
    cudaFuncSetAttribute(k_image<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sh);
    if (h > 0)
      k_image<false><<<grid, kImgThreads, sh, ctx->stream>>>(w, h, offs, ev, r, D, erode, counts, nullptr, nullptr);
    ctx->launches += 1;
    rc = scan_counts(ctx, counts, *ooffs, h, total);
  }
  if (!rc) rc = dalloc(ctx, oev, (size_t)std::max<long long>(*total, 1));
  if (!rc && h > 0) {
    k_image<true><<<grid, kImgThreads, sh, ctx->stream>>>(w, h, offs, ev, r, D, erode, nullptr, *ooffs, *oev);
    ctx->launches += 1;
  }
  dfree(ctx, counts);
  if (!rc) {
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) rc = cuda_error(ctx, e, "image kernels");
  }
  if (rc) {
    dfree(ctx, *ooffs);
    dfree(ctx, *oev);
    *ooffs = nullptr;
    *oev = nullptr;
  }
  return rc;
}

}  // namespace
}  // namespace vo

using namespace vo;

extern "C" int vo_image_morph(vo_ctx *ctx, int op, double radius, int width, int height, const int32_t *row_offs,
                              const int32_t *events, int32_t *out_row_offs, int32_t *out_events,
                              int64_t out_capacity) {
  if (!ctx) return VO_EINVAL;
  if (op < VO_DILATION || op > VO_CLOSING || !(radius >= 0) || !std::isfinite(radius) || width < 1 ||
      height < 0 || !row_offs || !out_row_offs || (row_offs[height] > 0 && !events) || out_capacity < 0 ||
      (out_capacity > 0 && !out_events))
    return set_error(ctx, VO_EINVAL, "image: bad arguments");
  if (width > kImgMaxWidth) return set_error(ctx, VO_EINVAL, "image: width beyond 50000 pixels");
  if (radius > 1e6) return set_error(ctx, VO_EINVAL, "image: radius beyond 1e6 pixels");
  // rows: even event counts, events strictly increasing within [0, width]
  if (row_offs[0] != 0) return set_error(ctx, VO_EINVAL, "image: row_offs[0] must be 0");
  for (int i = 0; i < height; ++i) {
    const int a = row_offs[i], b = row_offs[i + 1];
    if (b < a || ((b - a) & 1)) return set_error(ctx, VO_EINVAL, "image: a row needs an even event count");
    for (int k = a; k < b; ++k)
      if (events[k] < 0 || events[k] > width || (k > a && events[k] <= events[k - 1]))
        return set_error(ctx, VO_EINVAL, "image: events must increase strictly within [0, width]");
  }
  // a radius within rounding below an integer would make the reference's row reach,
  // floor(i0 + r), depend on the row index
  const int D = (int)std::floor(radius);
  for (int i0 = -1; i0 <= height; ++i0)
    if ((int)std::floor((double)i0 + radius) != i0 + D)
      return set_error(ctx, VO_ERADIUS, "image: radius within rounding of an integer");
  cudaSetDevice(ctx->device);
  ctx->err.clear();
  ctx->launches = 0;
  const long long nev = row_offs[height];
  int32_t *d_offs = nullptr, *d_ev = nullptr;
  int rc = dalloc(ctx, &d_offs, (size_t)height + 1);
  if (!rc) rc = dalloc(ctx, &d_ev, (size_t)std::max<long long>(nev, 1));
  if (!rc) {
    cudaMemcpyAsync(d_offs, row_offs, sizeof(int32_t) * ((size_t)height + 1), cudaMemcpyHostToDevice, ctx->stream);
    if (nev) cudaMemcpyAsync(d_ev, events, sizeof(int32_t) * nev, cudaMemcpyHostToDevice, ctx->stream);
  }
  // the op's steps: dilate 0 / erode 1; opening = erode, dilate; closing = dilate, erode
  std::vector<int> steps;
  if (op == VO_DILATION) steps = {0};
  else if (op == VO_EROSION) steps = {1};
  else if (op == VO_OPENING) steps = {1, 0};
  else steps = {0, 1};
  long long total = nev;
  for (size_t s = 0; !rc && s < steps.size(); ++s) {
    int32_t *o2 = nullptr, *e2 = nullptr;
    rc = image_op(ctx, steps[s], radius, width, height, d_offs, d_ev, &o2, &e2, &total);
    dfree(ctx, d_offs);
    dfree(ctx, d_ev);
    d_offs = o2;
    d_ev = e2;
  }
  if (!rc) {
    VO_CK(ctx, cudaMemcpyAsync(out_row_offs, d_offs, sizeof(int32_t) * ((size_t)height + 1), cudaMemcpyDeviceToHost,
                               ctx->stream));
    VO_CK(ctx, cudaStreamSynchronize(ctx->stream));
    if (total > out_capacity) {
      rc = set_error(ctx, VO_ERANGE, "image: out_capacity below the result's event count (in out_row_offs[height])");
    } else if (total > 0) {
      VO_CK(ctx, cudaMemcpyAsync(out_events, d_ev, sizeof(int32_t) * total, cudaMemcpyDeviceToHost, ctx->stream));
      VO_CK(ctx, cudaStreamSynchronize(ctx->stream));
    }
  }
  dfree(ctx, d_offs);
  dfree(ctx, d_ev);
  if (!rc) VO_CK(ctx, cudaStreamSynchronize(ctx->stream));
  return rc;
}

// ============================================================ the FP64 twin
//
// DoubleCompressedImage (DoubleCompressedImage.cpp:680-720): rows of closed
// spans with FP64 events in [0, width]. Its dilation of row i is the union over
// rows i0 with |i - i0| <= floor(R) of [y1 - dy, y2 + dy], dy = sqrt(R*R - t*t)
// (VoronoiMorphoF::getLine, DoubleVoronoi.cpp:713-726): the 3D dilation of a
// grid of one row of columns, computed here by the FP32-guarded kernels, then
// clamped to [0, width] with intervals wholly outside dropped. Dilation scales
// its radius by the row count (R = r * height) and erosion does not, as in the
// reference. Erosion dilates the complement spans [-1, a0], [b0, a1], ...,
// [b_last, width] of every row plus a full row [-1, width] before the first
// and after the last (voronoiF_half_erode, DoubleVoronoi.h:124-148), clamps,
// and negates (DoubleCompressedImage.cpp:438-470).

namespace vo {
namespace {

__global__ void k_half_offsets(int n, const int32_t *__restrict__ ev_offs, int32_t *__restrict__ seg_offs) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i <= n) seg_offs[i] = ev_offs[i] / 2;
}

// Complement rows (h + 2 of them, the first and last full) as a one-row-of-columns volume.
template <bool FILL>
__global__ void k_img64_complement(int h, double w, const int32_t *__restrict__ ev_offs, const double *__restrict__ ev,
                                   int32_t *__restrict__ counts, const int32_t *__restrict__ ooffs,
                                   double2 *__restrict__ oz) {
  const int r = blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= h + 2) return;
  if (r == 0 || r == h + 1) {
    if (FILL) oz[ooffs[r]] = make_double2(-1.0, w);
    else counts[r] = 1;
    return;
  }
  const int i = r - 1, a = ev_offs[i], b = ev_offs[i + 1];
  if (!FILL) {
    counts[r] = (b - a) / 2 + 1;
    return;
  }
  double2 *o = oz + ooffs[r];
  double y1 = -1.0;
  for (int k = a; k + 1 < b; k += 2) {
    *o++ = make_double2(y1, ev[k]);
    y1 = ev[k + 1];
  }
  *o = make_double2(y1, w);
}

// Rows row0 .. row0 + h - 1 of a dilated volume, clamped to [0, w] with
// intervals wholly outside dropped, and (negate) complemented the way
// DoubleCompressedImage::negate does: an empty row becomes [0, w]; a leading 0
// is dropped, else 0 is prepended; a trailing w is dropped, else w is appended.
// An interval clamped to end at w is its row's last (the union's intervals are
// disjoint), so under negation that end is never written.
template <bool FILL>
__global__ void k_img64_clip(int h, int row0, double w, int negate, const int32_t *__restrict__ soffs,
                             const double2 *__restrict__ z, int32_t *__restrict__ counts,
                             const int32_t *__restrict__ ooffs, double *__restrict__ oev) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= h) return;
  const int s0 = soffs[row0 + i], s1 = soffs[row0 + i + 1];
  double *o = FILL ? oev + ooffs[i] : nullptr;
  int n = 0, kept = 0;
  bool last_w = false;
#define EMIT(v)            \
  {                        \
    if (FILL) o[n] = (v);  \
    ++n;                   \
  }
  for (int s = s0; s < s1; ++s) {
    const double2 v = z[s];
    if (v.y < 0 || v.x > w) continue;
    const double lo = v.x > 0 ? v.x : 0.0, hi = v.y < w ? v.y : w;
    if (kept == 0 && negate) {
      if (lo != 0.0) {
        EMIT(0.0)
        EMIT(lo)
      }
    } else {
      EMIT(lo)
    }
    if (negate && hi == w) last_w = true;
    else EMIT(hi)
    ++kept;
  }
  if (negate) {
    if (kept == 0) {
      EMIT(0.0)
      EMIT(w)
    } else if (!last_w) {
      EMIT(w)
    }
  }
#undef EMIT
  if (!FILL) counts[i] = n;
}

struct Rows64 {
  int32_t *offs = nullptr;  // events per row, CSR [h + 1]
  double *ev = nullptr;
  long long total = 0;
};

void rows_free(vo_ctx *ctx, Rows64 &r) {
  dfree(ctx, r.offs);
  dfree(ctx, r.ev);
  r = Rows64();
}

// One dilation (erode = 0, radius R) or erosion (erode = 1) of device rows.
int image64_step(vo_ctx *ctx, int erode, double R, int w, int h, const Rows64 &in, Rows64 &out) {
  const int nr = erode ? h + 2 : h;
  vo_grid g;
  g.nx = nr;
  g.ny = 1;
  for (int k = 0; k < 3; ++k) g.origin[k] = 0.0;
  g.extent[0] = nr;
  g.extent[1] = 1;
  g.extent[2] = w;
  g.spacing = 1.0;
  g.padding = 0;
  int32_t *counts = nullptr;
  int rc = dalloc(ctx, &counts, (size_t)nr + 2);
  vo_volume src;  // a view (no ownership) or the complement volume below
  src.grid = g;
  src.owns = false;
  vo_volume *comp = nullptr;
  if (!rc && !erode) {
    rc = dalloc(ctx, &src.offs, (size_t)h + 1);
    if (!rc) {
      k_half_offsets<<<(h + 1 + 255) / 256, 256, 0, ctx->stream>>>(h, in.offs, src.offs);
      ctx->launches += 1;
      src.z = reinterpret_cast<double2 *>(in.ev);
      src.nseg = in.total / 2;
    }
  } else if (!rc) {
    long long tot = 0;
    rc = volume_alloc(ctx, g, 0, &comp);
    if (!rc) {
      k_img64_complement<false><<<(nr + 255) / 256, 256, 0, ctx->stream>>>(h, (double)w, in.offs, in.ev, counts,
                                                                          nullptr, nullptr);
      ctx->launches += 1;
      rc = scan_counts(ctx, counts, comp->offs, nr, &tot);
    }
    if (!rc) {
      comp->nseg = tot;
      rc = dalloc(ctx, &comp->z, (size_t)std::max<long long>(tot, 1));
    }
    if (!rc) {
      k_img64_complement<true><<<(nr + 255) / 256, 256, 0, ctx->stream>>>(h, (double)w, in.offs, in.ev, nullptr,
                                                                         comp->offs, comp->z);
      ctx->launches += 1;
    }
  }
  vo_volume *dil = nullptr;
  if (!rc) rc = dilate(ctx, VO_METHOD_FAST, R, erode ? comp : &src, &dil, nullptr);
  if (!rc) rc = dalloc(ctx, &out.offs, (size_t)h + 1);
  if (!rc) {
    k_img64_clip<false><<<(h + 255) / 256, 256, 0, ctx->stream>>>(h, erode ? 1 : 0, (double)w, erode, dil->offs,
                                                                  dil->z, counts, nullptr, nullptr);
    ctx->launches += 1;
    rc = scan_counts(ctx, counts, out.offs, h, &out.total);
  }
  if (!rc) rc = dalloc(ctx, &out.ev, (size_t)std::max<long long>(out.total, 1));
  if (!rc) {
    k_img64_clip<true><<<(h + 255) / 256, 256, 0, ctx->stream>>>(h, erode ? 1 : 0, (double)w, erode, dil->offs,
                                                                 dil->z, nullptr, out.offs, out.ev);
    ctx->launches += 1;
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) rc = cuda_error(ctx, e, "image kernels");
  }
  if (!erode) dfree(ctx, src.offs);
  if (comp) vo_volume_free(ctx, comp);
  if (dil) vo_volume_free(ctx, dil);
  dfree(ctx, counts);
  if (rc) rows_free(ctx, out);
  return rc;
}

}  // namespace
}  // namespace vo

extern "C" int vo_image_morph_f64(vo_ctx *ctx, int op, double radius, int width, int height,
                                  const int32_t *row_offs, const double *events, int32_t *out_row_offs,
                                  double *out_events, int64_t out_capacity) {
  if (!ctx) return VO_EINVAL;
  if (op < VO_DILATION || op > VO_CLOSING || !(radius >= 0) || !std::isfinite(radius) || width < 1 ||
      height < 0 || !row_offs || !out_row_offs || (row_offs[height] > 0 && !events) || out_capacity < 0 ||
      (out_capacity > 0 && !out_events))
    return set_error(ctx, VO_EINVAL, "image: bad arguments");
  if (row_offs[0] != 0) return set_error(ctx, VO_EINVAL, "image: row_offs[0] must be 0");
  for (int i = 0; i < height; ++i) {
    const int a = row_offs[i], b = row_offs[i + 1];
    if (b < a || ((b - a) & 1)) return set_error(ctx, VO_EINVAL, "image: a row needs an even event count");
    for (int k = a; k < b; ++k)
      if (!(events[k] >= 0 && events[k] <= width) || (k > a && events[k] < events[k - 1]))
        return set_error(ctx, VO_EINVAL, "image: events must be sorted within [0, width]");
  }
  cudaSetDevice(ctx->device);
  ctx->err.clear();
  ctx->launches = 0;
  if (height == 0) {
    out_row_offs[0] = 0;
    return VO_OK;
  }
  Rows64 cur;
  cur.total = row_offs[height];
  int rc = dalloc(ctx, &cur.offs, (size_t)height + 1);
  if (!rc) rc = dalloc(ctx, &cur.ev, (size_t)std::max<long long>(cur.total, 1));
  if (!rc) {
    cudaMemcpyAsync(cur.offs, row_offs, sizeof(int32_t) * ((size_t)height + 1), cudaMemcpyHostToDevice, ctx->stream);
    if (cur.total)
      cudaMemcpyAsync(cur.ev, events, sizeof(double) * cur.total, cudaMemcpyHostToDevice, ctx->stream);
  }
  std::vector<int> steps;
  if (op == VO_DILATION) steps = {0};
  else if (op == VO_EROSION) steps = {1};
  else if (op == VO_OPENING) steps = {1, 0};
  else steps = {0, 1};
  for (size_t s = 0; !rc && s < steps.size(); ++s) {
    Rows64 nxt;
    // dilation: radius scaled by the row count (radius * m_Rays.size(), DoubleCompressedImage.cpp:685)
    const double R = steps[s] ? radius : radius * (double)height;
    rc = image64_step(ctx, steps[s], R, width, height, cur, nxt);
    rows_free(ctx, cur);
    cur = nxt;
  }
  if (!rc) {
    VO_CK(ctx, cudaMemcpyAsync(out_row_offs, cur.offs, sizeof(int32_t) * ((size_t)height + 1),
                               cudaMemcpyDeviceToHost, ctx->stream));
    VO_CK(ctx, cudaStreamSynchronize(ctx->stream));
    if (cur.total > out_capacity) {
      rc = set_error(ctx, VO_ERANGE, "image: out_capacity below the result's event count (in out_row_offs[height])");
    } else if (cur.total > 0) {
      VO_CK(ctx, cudaMemcpyAsync(out_events, cur.ev, sizeof(double) * cur.total, cudaMemcpyDeviceToHost,
                                 ctx->stream));
      VO_CK(ctx, cudaStreamSynchronize(ctx->stream));
    }
  }
  rows_free(ctx, cur);
  return rc;
}
