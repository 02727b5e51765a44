// Exact separable dilation with FP32 envelope arithmetic and an FP64 guard
// (VO_METHOD_FAST, and the engine behind VO_METHOD_SEPARABLE on large inputs).
//
// The separable scheme of the reference (VoronoiVorPower.cpp:24-96: a y-pass
// giving each z the nearest covering row distance d with radius
// r(d) = sqrt(R^2 - d^2), then an x-pass dilating by sqrt(r(d)^2 - dx^2))
// produces, per output column (x, y), the union of the candidate intervals
//     [z1 - H[|dy|][|dx|], z2 + H[|dy|][|dx|]]
// over the input segments [z1, z2] of every column (x+dx, y+dy) with
// |dx| <= Dx[|dy|], where H[d][a] = sqrt(r(d)*r(d) - a*a) is the reference's
// own FP64 value (pass-1 pieces are sub-intervals of these segments whose
// candidates tile them, so both unions are the same set, bit for bit).
//
// One thread per output column walks the (|dx|, |dy|) pairs in decreasing H
// and merges each source column's dilated segments into a small sorted union
// kept in local memory. Candidate endpoints are formed in FP32 (FP32 copies of
// the inputs and of H); every comparison is decided in FP32 when the values
// differ by more than a guard band E bounding the FP32 error, and otherwise
// re-evaluated exactly in FP64 from the candidate's identity (input value
// index, d, a). Output endpoints are always recomputed in FP64 from their
// identities, so results are bit-identical to the FP64 oracle.
// Columns whose union outgrows the local capacity are re-run by an FP64
// kernel with a large global working list.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#include "vo_internal.cuh"

namespace vo {
namespace {

constexpr int kKA = 32;          // union capacity per thread
constexpr int kFB = 32, kFBY = 4;  // block shape: x-major
constexpr int kBigCap = 8192;    // fallback working list (intervals)
constexpr int kBigThreads = 32;

struct FastArgs {
  int nx, ny, W;
  // Column c's segments are [beg[c], end[c]); for CSR input beg = offs and
  // end = offs + 1, for a fixed-capacity slot layout beg[c] = c * cap.
  const int32_t *beg, *end;
  const double *zd;     // FP64 values, 2 per segment
  const float *zf;      // FP32 copies
  const float *Hf;      // [(Dy+1) * W]
  const double *H64;    // [(Dy+1) * W]
  const int2 *pairs;    // (a, d) sorted by decreasing H
  int npairs;
  const float *E;       // guard band (device scalar)
};

// Identities of union endpoints, kept in local memory and read only when an
// FP32 comparison falls inside the guard band or the output is written.
struct UnionIds {
  int li[kKA], hi_i[kKA];  // input value index of the lower / upper endpoint
  int lda[kKA], hda[kKA];  // d | a << 8 of the lower / upper endpoint
};

__device__ __forceinline__ double exact_val(const FastArgs &A, int idx, int da, bool plus) {
  const double h = A.H64[(da & 255) * A.W + (da >> 8)];
  const double z = A.zd[idx];
  return plus ? __dadd_rn(z, h) : __dsub_rn(z, h);
}

// Exact comparisons, out of line: identities are loaded only here.
// Union endpoint (j, hi?) < candidate endpoint (idx, da, plus)?
__device__ __noinline__ bool ex_u_lt_c(const FastArgs &A, const UnionIds &U, int j, bool jhi, int idx, int da,
                                       bool plus) {
  const double u = jhi ? exact_val(A, U.hi_i[j], U.hda[j], true) : exact_val(A, U.li[j], U.lda[j], false);
  return u < exact_val(A, idx, da, plus);
}
// Candidate endpoint < union endpoint?
__device__ __noinline__ bool ex_c_lt_u(const FastArgs &A, const UnionIds &U, int idx, int da, bool plus, int j,
                                       bool jhi) {
  const double u = jhi ? exact_val(A, U.hi_i[j], U.hda[j], true) : exact_val(A, U.li[j], U.lda[j], false);
  return exact_val(A, idx, da, plus) < u;
}
// Union endpoint (i, ihi) < union endpoint (j, jhi)?
__device__ __noinline__ bool ex_u_lt_u(const FastArgs &A, const UnionIds &U, int i, bool ihi, int j, bool jhi) {
  const double a = ihi ? exact_val(A, U.hi_i[i], U.hda[i], true) : exact_val(A, U.li[i], U.lda[i], false);
  const double b = jhi ? exact_val(A, U.hi_i[j], U.hda[j], true) : exact_val(A, U.li[j], U.lda[j], false);
  return a < b;
}

// FP32 difference t = y - x decides x < y outside the guard band [-E, E].
#define GUARD(t, E, exact) ((t) > (E) ? true : ((t) < -(E) ? false : (exact)))

// Returns the number of intervals, or -1 when more than kKA are needed.
// Writes the exact FP64 union to out[0..n).
//
// `mask` holds the lanes of the warp running this function together. For each
// (|dx|, |dy|) pair the four source columns' segments form one list per lane;
// every lane of the warp iterates to the warp's longest list with a predicate,
// and the loop body has no early exits, so the lanes reconverge after every
// candidate instead of drifting apart over the source transitions.
__device__ int fast_column(const FastArgs &A, float E, int x, int y, float2 *sv, int stride, UnionIds &U,
                           double2 *out, unsigned mask) {
  int n = 0;
  bool overflow = false;
#define SV(k) sv[(k) * stride]
  for (int p = 0; p < A.npairs; ++p) {
    const int2 ad = A.pairs[p];
    const int a = ad.x, d = ad.y;
    const float h = A.Hf[d * A.W + a];
    const int da = d | (a << 8);
    int kb0, ke0, kb1, ke1, kb2, ke2, kb3, ke3;
#define SRC(S, KB, KE)                                                                                  \
  {                                                                                                     \
    const int xs = ((S) & 1) ? x + a : x - a;                                                           \
    const int ys = ((S) & 2) ? y + d : y - d;                                                           \
    const bool ok = !(((S) & 1) && a == 0) && !(((S) & 2) && d == 0) && xs >= 0 && xs < A.nx && ys >= 0 && \
                    ys < A.ny;                                                                          \
    const int c = ok ? xs + A.nx * ys : 0;                                                              \
    KB = ok ? A.beg[c] : 0;                                                                             \
    KE = ok ? A.end[c] : 0;                                                                             \
  }
    SRC(0, kb0, ke0)
    SRC(1, kb1, ke1)
    SRC(2, kb2, ke2)
    SRC(3, kb3, ke3)
#undef SRC
    const int total = (ke0 - kb0) + (ke1 - kb1) + (ke2 - kb2) + (ke3 - kb3);
    const int iters = __reduce_max_sync(mask, total);
    int s = 0, k = kb0, kend = ke0;
    int cur = 0;
    float2 cv = n > 0 ? SV(0) : make_float2(0.f, 0.f);
    for (int it = 0; it < iters; ++it) {
      if (it < total && !overflow) {
        while (k >= kend) {  // next non-empty source column: restart the cursor
          ++s;
          k = s == 1 ? kb1 : (s == 2 ? kb2 : kb3);
          kend = s == 1 ? ke1 : (s == 2 ? ke2 : ke3);
          cur = 0;
          if (n > 0) cv = SV(0);
        }
        const float2 zf = *reinterpret_cast<const float2 *>(A.zf + 2 * k);
        const float lo = zf.x - h, hi = zf.y + h;
        const int il = 2 * k, ih = 2 * k + 1;
        ++k;
        // skip union intervals that end strictly below the candidate: U.hi[cur] < lo
        while (cur < n && GUARD(lo - cv.y, E, ex_u_lt_c(A, U, cur, true, il, da, false))) {
          ++cur;
          if (cur < n) cv = SV(cur);
        }
        bool covered = false;
        if (cur < n) {
          if (lo - cv.x > E && cv.y - hi > E) {
            covered = true;  // inside U[cur] by more than the guard band
          } else {
            const bool lo_in = !GUARD(cv.x - lo, E, ex_c_lt_u(A, U, il, da, false, cur, false));
            covered = lo_in && !GUARD(hi - cv.y, E, ex_u_lt_c(A, U, cur, true, ih, da, true));
          }
        }
        if (!covered) {
          if (cur == n || GUARD(cv.x - hi, E, ex_c_lt_u(A, U, ih, da, true, cur, false))) {
            // disjoint: insert before cur
            if (n >= kKA) {
              overflow = true;
            } else {
              for (int j = n; j > cur; --j) {
                SV(j) = SV(j - 1);
                U.li[j] = U.li[j - 1];
                U.hi_i[j] = U.hi_i[j - 1];
                U.lda[j] = U.lda[j - 1];
                U.hda[j] = U.hda[j - 1];
              }
              cv = make_float2(lo, hi);
              SV(cur) = cv;
              U.li[cur] = il;
              U.hi_i[cur] = ih;
              U.lda[cur] = da;
              U.hda[cur] = da;
              ++n;
            }
          } else {
            // overlapping or touching U[cur]: extend it
            if (GUARD(cv.x - lo, E, ex_c_lt_u(A, U, il, da, false, cur, false))) {
              cv.x = lo;
              U.li[cur] = il;
              U.lda[cur] = da;
            }
            if (GUARD(hi - cv.y, E, ex_u_lt_c(A, U, cur, true, ih, da, true))) {
              cv.y = hi;
              U.hi_i[cur] = ih;
              U.hda[cur] = da;
              // absorb following intervals that now start at or below the new end
              int j = cur + 1;
              while (j < n) {
                const float2 nv = SV(j);
                if (GUARD(nv.x - cv.y, E, ex_u_lt_u(A, U, cur, true, j, false))) break;  // U.hi[cur] < U.lo[j]
                if (GUARD(nv.y - cv.y, E, ex_u_lt_u(A, U, cur, true, j, true))) {       // U.hi[cur] < U.hi[j]
                  cv.y = nv.y;
                  U.hi_i[cur] = U.hi_i[j];
                  U.hda[cur] = U.hda[j];
                }
                ++j;
              }
              const int gone = j - cur - 1;
              if (gone > 0) {
                for (int m = cur + 1; m + gone < n; ++m) {
                  SV(m) = SV(m + gone);
                  U.li[m] = U.li[m + gone];
                  U.hi_i[m] = U.hi_i[m + gone];
                  U.lda[m] = U.lda[m + gone];
                  U.hda[m] = U.hda[m + gone];
                }
                n -= gone;
              }
            }
            SV(cur) = cv;
          }
        }
      }
    }
  }
#undef SV
  if (overflow) return -1;
  for (int k = 0; k < n; ++k)
    out[k] = make_double2(exact_val(A, U.li[k], U.lda[k], false), exact_val(A, U.hi_i[k], U.hda[k], true));
  return n;
}

// One pass: the exact union of every output column goes to its fixed-capacity
// staging slot (kKA intervals) with its count; columns that need more are
// listed for the FP64 re-run. A compaction pass then packs the slots.
__global__ void __launch_bounds__(kFB *kFBY) k_fast(FastArgs A, int32_t *counts, double2 *staging,
                                                    int *ovf_count, int *ovf_cols) {
  __shared__ float2 sv[kKA * kFB * kFBY];
  const int tid = threadIdx.x + kFB * threadIdx.y;
  const int x = blockIdx.x * kFB + threadIdx.x;
  const int y = blockIdx.y * kFBY + threadIdx.y;
  if (x >= A.nx || y >= A.ny) return;
  const int c = x + A.nx * y;
  const float E = *A.E;
  UnionIds U;
  const unsigned mask = __activemask();
  const int n = fast_column(A, E, x, y, sv + tid, kFB * kFBY, U, staging + (size_t)c * kKA, mask);
  if (n < 0) {
    ovf_cols[atomicAdd(ovf_count, 1)] = c;
    counts[c] = 0;
  } else {
    counts[c] = n;
  }
}

// Packs the staging slots of non-overflowing columns into the CSR output.
__global__ void k_compact(int ncols, const int32_t *__restrict__ counts, const double2 *__restrict__ staging,
                          const int32_t *__restrict__ ooffs, double2 *__restrict__ oz) {
  // one warp per column, lanes over intervals
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (w >= ncols) return;
  const int n = ooffs[w + 1] - ooffs[w];
  if (n > kKA) return;  // written by the FP64 re-run
  for (int k = lane; k < n; k += 32) oz[ooffs[w] + k] = staging[(size_t)w * kKA + k];
}

// FP64 re-run of columns whose union outgrew kKA: same candidate set, exact
// arithmetic, insertion into a large sorted list in global scratch.
__device__ bool big_insert(double2 *L, int &n, int cap, double lo, double hi) {
  int l = 0, r = n;
  while (l < r) {
    const int m = (l + r) >> 1;
    if (L[m].y >= lo)
      r = m;
    else
      l = m + 1;
  }
  const int i = l;
  if (i == n || L[i].x > hi) {
    if (n >= cap) return false;
    for (int k = n; k > i; --k) L[k] = L[k - 1];
    L[i] = make_double2(lo, hi);
    ++n;
    return true;
  }
  int j = i;
  while (j + 1 < n && L[j + 1].x <= hi) ++j;
  L[i] = make_double2(L[i].x < lo ? L[i].x : lo, L[j].y > hi ? L[j].y : hi);
  if (j > i) {
    const int sh = j - i;
    for (int k = i + 1; k + sh < n; ++k) L[k] = L[k + sh];
    n -= sh;
  }
  return true;
}

template <bool FILL>
__global__ void __launch_bounds__(kBigThreads) k_fast_big(FastArgs A, int32_t *counts, const int32_t *ooffs,
                                                         double2 *oz, const int *ovf_count, const int *ovf_cols,
                                                         double2 *scratch, int *fatal) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;
  double2 *L = scratch + (size_t)tid * kBigCap;
  for (int i = tid; i < *ovf_count; i += nth) {
    const int c = ovf_cols[i];
    const int x = c % A.nx, y = c / A.nx;
    int n = 0;
    bool ok = true;
    for (int p = 0; p < A.npairs && ok; ++p) {
      const int2 ad = A.pairs[p];
      const int a = ad.x, d = ad.y;
      const double h = A.H64[d * A.W + a];
      for (int s = 0; s < 4 && ok; ++s) {
        const int xs = (s & 1) ? x + a : x - a;
        const int ys = (s & 2) ? y + d : y - d;
        if ((s & 1) && a == 0) continue;
        if ((s & 2) && d == 0) continue;
        if (xs < 0 || xs >= A.nx || ys < 0 || ys >= A.ny) continue;
        const int cs = xs + A.nx * ys;
        for (int k = A.beg[cs]; k < A.end[cs] && ok; ++k)
          ok = big_insert(L, n, kBigCap, __dsub_rn(A.zd[2 * k], h), __dadd_rn(A.zd[2 * k + 1], h));
      }
    }
    if (!ok) {
      *fatal = 1;
      n = 0;
    }
    if (FILL) {
      double2 *o = oz + ooffs[c];
      for (int k = 0; k < n; ++k) o[k] = L[k];
    } else {
      counts[c] = n;
    }
  }
}

// ---------------------------------------------------------------- helpers

// FP32 copies of the input values and max |z| (as float bits, for the guard).
__global__ void k_to_f32(const double *zd, int64_t nval, float *zf, unsigned int *maxabs_bits) {
  unsigned int m = 0;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nval; i += (int64_t)gridDim.x * blockDim.x) {
    const float f = __double2float_rn(zd[i]);
    zf[i] = f;
    const unsigned int b = __float_as_uint(fabsf(f));
    m = b > m ? b : m;
  }
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned int t = __shfl_xor_sync(0xffffffffu, m, o);
    m = t > m ? t : m;
  }
  if ((threadIdx.x & 31) == 0) atomicMax(maxabs_bits, m);
}

// Guard band: E bounds the error of an FP32 comparison t = y - x of two
// candidate endpoints (each within 1.5 ulp of its FP64 value: rounding of z,
// of H and of the sum), plus the rounding of t itself: 4 ulp32(U) for
// magnitudes up to U; E = 2^-20 * U leaves a factor two of margin.
__global__ void k_guard(const unsigned int *maxabs_bits, float R, float *E) {
  const float U = __uint_as_float(*maxabs_bits) + R + 1.0f;
  *E = U * 9.5367431640625e-07f;  // 2^-20
}

// FP32 copies of the values of columns [beg, end) (slot layouts leave unused
// slots, which are skipped) and max |z| for the guard band.
__global__ void k_to_f32_cols(int ncols, const int32_t *beg, const int32_t *end, const double *zd, float *zf,
                              unsigned int *maxabs_bits) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  unsigned int m = 0;
  if (c < ncols)
    for (int k = 2 * beg[c]; k < 2 * end[c]; ++k) {
      const float f = __double2float_rn(zd[k]);
      zf[k] = f;
      const unsigned int b = __float_as_uint(fabsf(f));
      m = b > m ? b : m;
    }
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned int t = __shfl_xor_sync(0xffffffffu, m, o);
    m = t > m ? t : m;
  }
  if ((threadIdx.x & 31) == 0) atomicMax(maxabs_bits, m);
}

// One dilation of a batch: its tables, input view, and outputs.
struct BatchVol {
  FastArgs A;
  int32_t *counts;   // per column
  double2 *staging;  // ncols * kKA slots
  int *ovf;          // set when some column needs more than kKA intervals
  int tiles_x;
};

// Persistent kernel over the tiles (kFB x kFBY output columns) of every
// dilation of a batch: blocks pull (volume, tile) items from a queue ordered
// by decreasing estimated work, so uneven volumes balance across the SMs.
__global__ void __launch_bounds__(kFB *kFBY) k_fast_batched(const BatchVol *vols, const int2 *queue, int nq,
                                                            int *next) {
  __shared__ float2 sv[kKA * kFB * kFBY];
  __shared__ int s_item;
  const int tid = threadIdx.x + kFB * threadIdx.y;
  for (;;) {
    if (tid == 0) s_item = atomicAdd(next, 1);
    __syncthreads();
    const int item = s_item;
    __syncthreads();
    if (item >= nq) return;
    const int2 q = queue[item];
    const BatchVol V = vols[q.x];
    const int x = (q.y % V.tiles_x) * kFB + threadIdx.x;
    const int y = (q.y / V.tiles_x) * kFBY + threadIdx.y;
    if (x < V.A.nx && y < V.A.ny) {
      const int c = x + V.A.nx * y;
      UnionIds U;
      const unsigned mask = __activemask();
      const int n = fast_column(V.A, *V.A.E, x, y, sv + tid, kFB * kFBY, U, V.staging + (size_t)c * kKA, mask);
      V.counts[c] = n < 0 ? 0 : n;
      if (n < 0) atomicOr(V.ovf, 1);
    }
  }
}

}  // namespace

// ================================================================ host side

namespace {

struct FastTables {
  double R = -1;
  int kmax = 0;
  int2 *pairs = nullptr;
  int npairs = 0;
};

int big_grid_fast() {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms > 0 ? sms : 148;
}

}  // namespace

int dilate_fast(vo_ctx *ctx, double R, const vo_volume *in, vo_volume **out, vo_timings *tm) {
  const vo_grid g = in->grid;
  const int nx = g.nx, ny = g.ny, ncols = nx * ny;
  const DeviceTables *T = nullptr;
  int rc = get_tables(ctx, R, std::max(nx, ny), &T);
  if (rc) return rc;
  const Tables &h = T->host;
  // (a, d) pairs alive (a <= Dx[d]) sorted by decreasing H
  std::vector<int2> pairs;
  for (int d = 0; d <= h.Dy; ++d)
    for (int a = 0; a <= h.Dx[d]; ++a) pairs.push_back(make_int2(a, d));
  std::stable_sort(pairs.begin(), pairs.end(), [&](const int2 &p, const int2 &q) {
    return h.H[(size_t)p.y * h.W + p.x] > h.H[(size_t)q.y * h.W + q.x];
  });
  const int64_t nval = 2 * in->nseg;
  float *zf = nullptr, *dE = nullptr;
  unsigned int *dmax = nullptr;
  int2 *dpairs = nullptr;
  int32_t *counts = nullptr;
  int *ovf_cols = nullptr;
  double2 *big = nullptr;
  vo_volume *res = nullptr;
  long long total = 0;
  const int gbig = big_grid_fast();
  rc = dalloc(ctx, &zf, (size_t)std::max<int64_t>(nval, 2));
  if (!rc) rc = dalloc(ctx, &dE, 1);
  if (!rc) rc = dalloc(ctx, &dmax, 1);
  if (!rc) rc = dalloc(ctx, &dpairs, pairs.size());
  if (!rc) rc = dalloc(ctx, &counts, (size_t)ncols);
  if (!rc) rc = dalloc(ctx, &ovf_cols, (size_t)ncols);
  if (!rc) rc = dalloc(ctx, &big, (size_t)gbig * kBigThreads * kBigCap);
  if (!rc) {
    cudaMemcpyAsync(dpairs, pairs.data(), sizeof(int2) * pairs.size(), cudaMemcpyHostToDevice, ctx->stream);
    cudaMemsetAsync(dmax, 0, sizeof(unsigned int), ctx->stream);
    cudaMemsetAsync(ctx->d_flags, 0, 2 * sizeof(int), ctx->stream);
    cudaEventRecord(ctx->ev[0], ctx->stream);
    if (nval > 0) {
      const int grid = (int)std::min<int64_t>((nval + 255) / 256, 152 * 32);
      k_to_f32<<<grid, 256, 0, ctx->stream>>>((const double *)in->z, nval, zf, dmax);
      ctx->launches += 1;
    }
    k_guard<<<1, 1, 0, ctx->stream>>>(dmax, (float)R, dE);
    ctx->launches += 1;
    cudaEventRecord(ctx->ev[1], ctx->stream);
  }
  FastArgs A{nx, ny, h.W, in->offs, in->offs + 1, (const double *)in->z, zf, T->Hf, T->H, dpairs,
             (int)pairs.size(), dE};
  const dim3 blk(kFB, kFBY), grd((nx + kFB - 1) / kFB, (ny + kFBY - 1) / kFBY);
  double2 *staging = nullptr;
  if (!rc) rc = dalloc(ctx, &staging, (size_t)ncols * kKA);
  if (!rc) {
    cudaEventRecord(ctx->ev[4], ctx->stream);
    k_fast<<<grd, blk, 0, ctx->stream>>>(A, counts, staging, ctx->d_flags, ovf_cols);
    k_fast_big<false><<<gbig, kBigThreads, 0, ctx->stream>>>(A, counts, nullptr, nullptr, ctx->d_flags, ovf_cols,
                                                             big, ctx->d_flags + 1);
    ctx->launches += 2;
    cudaEventRecord(ctx->ev[5], ctx->stream);
    rc = volume_alloc(ctx, g, 0, &res);
  }
  if (!rc) rc = scan_counts(ctx, counts, res->offs, ncols, &total);
  if (!rc) {
    res->nseg = total;
    rc = dalloc(ctx, &res->z, (size_t)total);
  }
  if (!rc) {
    cudaEventRecord(ctx->ev[6], ctx->stream);
    k_compact<<<(int)(((int64_t)ncols * 32 + 255) / 256), 256, 0, ctx->stream>>>(ncols, counts, staging, res->offs,
                                                                                 res->z);
    k_fast_big<true><<<gbig, kBigThreads, 0, ctx->stream>>>(A, nullptr, res->offs, res->z, ctx->d_flags, ovf_cols,
                                                            big, ctx->d_flags + 1);
    ctx->launches += 2;
    cudaEventRecord(ctx->ev[7], ctx->stream);
    int hf[2] = {0, 0};
    cudaMemcpyAsync(hf, ctx->d_flags, sizeof(hf), cudaMemcpyDeviceToHost, ctx->stream);
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess)
      rc = cuda_error(ctx, e, "dilate_fast");
    else if (hf[1])
      rc = set_error(ctx, VO_EINTERNAL, "a column exceeds the fallback union capacity");
    else
      ctx->ovf_cols += hf[0];
  }
  dfree(ctx, staging);
  if (!rc && tm) {
    float e0 = 0, e1 = 0, e2 = 0;
    cudaEventElapsedTime(&e0, ctx->ev[0], ctx->ev[1]);
    cudaEventElapsedTime(&e1, ctx->ev[4], ctx->ev[5]);
    cudaEventElapsedTime(&e2, ctx->ev[6], ctx->ev[7]);
    tm->pass1_ms += e0;
    tm->pass2_ms += e1 + e2;
    tm->kernel_ms[0] += e0;
    tm->kernel_ms[2] += e1;
    tm->kernel_ms[3] += e2;
  }
  dfree(ctx, zf);
  dfree(ctx, dE);
  dfree(ctx, dmax);
  dfree(ctx, dpairs);
  dfree(ctx, counts);
  dfree(ctx, ovf_cols);
  dfree(ctx, big);
  if (rc) {
    if (res) vo_volume_free(ctx, res);
    return rc;
  }
  *out = res;
  return VO_OK;
}

// ================================================================ batched executor

namespace {

enum StepKind { kDil, kNeg, kNorm, kNegInv };

// Operation chains (Voronoi.cpp:8-17 erosion; offset3d.cpp:124-133 opening/closing).
std::vector<StepKind> steps_of(int op) {
  switch (op) {
    case VO_DILATION:
      return {kDil};
    case VO_EROSION:
      return {kNeg, kNorm, kDil, kNegInv};
    case VO_OPENING:
      return {kNeg, kNorm, kDil, kNegInv, kDil};
    default:
      return {kDil, kNeg, kNorm, kDil, kNegInv};
  }
}

struct DilPlan {
  int vol;
  SlotVol in, out;
  float *zf = nullptr;
  float *E = nullptr;
  unsigned int *maxbits = nullptr;
  int32_t *counts = nullptr;
  int2 *pairs = nullptr;
  int npairs = 0;
  const DeviceTables *T = nullptr;
  double cost = 0;
};

}  // namespace

int morph_batched_fast(vo_ctx *ctx, int n, const int *ops, const double *radii, const vo_volume *const *ins,
                       vo_volume **outs, vo_timings *tm) {
  const auto t0 = std::chrono::steady_clock::now();
  std::vector<std::vector<StepKind>> plan(n);
  for (int v = 0; v < n; ++v) plan[v] = steps_of(ops[v]);
  // ---- setup (host synchronisation allowed): tables, input capacities
  int *d_max = nullptr, *d_flags = nullptr;
  int rc = dalloc(ctx, &d_max, (size_t)std::max(n, 1));
  if (!rc) rc = dalloc(ctx, &d_flags, (size_t)std::max(n, 1) + 1);  // [v]: per volume overflow, [n]: slot overflow
  if (rc) return rc;
  cudaMemsetAsync(d_max, 0, sizeof(int) * std::max(n, 1), ctx->stream);
  cudaMemsetAsync(d_flags, 0, sizeof(int) * (std::max(n, 1) + 1), ctx->stream);
  std::vector<SlotVol> cur(n);
  for (int v = 0; v < n; ++v) {
    cur[v] = slot_view(ins[v], 0);
    slot_max_count(ctx, cur[v], d_max + v);
  }
  std::vector<int> hmax(std::max(n, 1), 0);
  cudaMemcpyAsync(hmax.data(), d_max, sizeof(int) * std::max(n, 1), cudaMemcpyDeviceToHost, ctx->stream);
  VO_CK(ctx, cudaStreamSynchronize(ctx->stream));
  for (int v = 0; v < n; ++v) cur[v].cap = hmax[v];
  std::vector<const DeviceTables *> tabs(n);
  for (int v = 0; v < n; ++v) {
    const vo_grid &g = ins[v]->grid;
    rc = get_tables(ctx, radii[v], std::max(g.nx, g.ny) + 2, &tabs[v]);
    if (rc) {
      dfree(ctx, d_max);
      dfree(ctx, d_flags);
      return rc;
    }
  }
  // ---- rounds: stage k of every volume; all dilations of a round in one launch
  std::vector<size_t> next_step(n, 0);
  std::vector<SlotVol> owned;  // intermediates to release at the end
  int launches0 = ctx->launches;
  cudaEventRecord(ctx->ev[0], ctx->stream);
  float dil_ms = 0;
  for (;;) {
    std::vector<DilPlan> dils;
    bool any = false;
    for (int v = 0; v < n && !rc; ++v) {
      if (next_step[v] >= plan[v].size()) continue;
      any = true;
      const StepKind k = plan[v][next_step[v]++];
      SlotVol nxt;
      if (k == kNeg) {
        rc = slot_negate(ctx, cur[v], nxt, d_flags + n);
      } else if (k == kNorm) {
        rc = slot_normalize(ctx, cur[v], nxt, d_flags + n);
      } else if (k == kNegInv) {
        rc = slot_negate_inv(ctx, cur[v], ins[v]->grid, nxt, d_flags + n);
      } else {
        DilPlan d;
        d.vol = v;
        d.in = cur[v];
        d.T = tabs[v];
        dils.push_back(d);
        continue;
      }
      if (!rc) {
        owned.push_back(nxt);
        cur[v] = nxt;
      }
    }
    if (rc || !any) break;
    if (dils.empty()) continue;
    // prepare every dilation of the round
    std::vector<BatchVol> hb(dils.size());
    std::vector<int2> queue;
    for (size_t i = 0; i < dils.size() && !rc; ++i) {
      DilPlan &d = dils[i];
      const Tables &h = d.T->host;
      const vo_grid &g = d.in.grid;
      const int ncols = g.nx * g.ny;
      std::vector<int2> pairs;
      for (int dd = 0; dd <= h.Dy; ++dd)
        for (int a = 0; a <= h.Dx[dd]; ++a) pairs.push_back(make_int2(a, dd));
      std::stable_sort(pairs.begin(), pairs.end(), [&](const int2 &p, const int2 &q) {
        return h.H[(size_t)p.y * h.W + p.x] > h.H[(size_t)q.y * h.W + q.x];
      });
      d.npairs = (int)pairs.size();
      const size_t nval = 2 * (size_t)ncols * (size_t)std::max(d.in.cap, 1);
      const size_t nvalz = d.in.owns ? nval : 2 * (size_t)std::max<int64_t>(ins[d.vol]->nseg, 1);
      rc = dalloc(ctx, &d.zf, d.in.owns ? nval : nvalz);
      if (!rc) rc = dalloc(ctx, &d.E, 1);
      if (!rc) rc = dalloc(ctx, &d.maxbits, 1);
      if (!rc) rc = dalloc(ctx, &d.counts, (size_t)ncols);
      if (!rc) rc = dalloc(ctx, &d.pairs, pairs.size());
      if (!rc) rc = slot_alloc(ctx, g, kKA, d.out);
      if (rc) break;
      cudaMemcpyAsync(d.pairs, pairs.data(), sizeof(int2) * pairs.size(), cudaMemcpyHostToDevice, ctx->stream);
      cudaMemsetAsync(d.maxbits, 0, sizeof(unsigned int), ctx->stream);
      k_to_f32_cols<<<(ncols + 255) / 256, 256, 0, ctx->stream>>>(ncols, d.in.beg, d.in.end, (const double *)d.in.z,
                                                                  d.zf, d.maxbits);
      k_guard<<<1, 1, 0, ctx->stream>>>(d.maxbits, (float)radii[d.vol], d.E);
      ctx->launches += 2;
      hb[i].A = FastArgs{g.nx, g.ny, h.W, d.in.beg, d.in.end, (const double *)d.in.z, d.zf, d.T->Hf, d.T->H,
                         d.pairs, d.npairs, d.E};
      hb[i].counts = d.counts;
      hb[i].staging = d.out.z;
      hb[i].ovf = d_flags + d.vol;
      hb[i].tiles_x = (g.nx + kFB - 1) / kFB;
      const int tiles = hb[i].tiles_x * ((g.ny + kFBY - 1) / kFBY);
      // estimated work per tile: candidates ~ pairs x mean segments per column
      const double segs = d.in.owns ? (double)std::max(d.in.cap, 1) * 0.5 : (double)ins[d.vol]->nseg / ncols;
      d.cost = (double)d.npairs * (segs + 0.5);
      for (int t = 0; t < tiles; ++t) queue.push_back(make_int2((int)i, t));
    }
    if (rc) break;
    std::stable_sort(queue.begin(), queue.end(),
                     [&](const int2 &p, const int2 &q) { return dils[p.x].cost > dils[q.x].cost; });
    BatchVol *dvols = nullptr;
    int2 *dqueue = nullptr;
    int *dnext = nullptr;
    rc = dalloc(ctx, &dvols, hb.size());
    if (!rc) rc = dalloc(ctx, &dqueue, queue.size());
    if (!rc) rc = dalloc(ctx, &dnext, 1);
    if (!rc) {
      cudaMemcpyAsync(dvols, hb.data(), sizeof(BatchVol) * hb.size(), cudaMemcpyHostToDevice, ctx->stream);
      cudaMemcpyAsync(dqueue, queue.data(), sizeof(int2) * queue.size(), cudaMemcpyHostToDevice, ctx->stream);
      cudaMemsetAsync(dnext, 0, sizeof(int), ctx->stream);
      int dev = 0, sms = 0, per_sm = 0;
      cudaGetDevice(&dev);
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_fast_batched, kFB * kFBY, 0);
      const int grid = std::max(1, std::min<int>((int)queue.size(), sms * std::max(per_sm, 1)));
      cudaEventRecord(ctx->ev[4], ctx->stream);
      k_fast_batched<<<grid, dim3(kFB, kFBY), 0, ctx->stream>>>(dvols, dqueue, (int)queue.size(), dnext);
      cudaEventRecord(ctx->ev[5], ctx->stream);
      ctx->launches += 1;
      for (auto &d : dils) {
        slot_end_from_counts(ctx, d.out, d.counts);
        owned.push_back(d.out);
        cur[d.vol] = d.out;
      }
      // the hb/queue host vectors must outlive the asynchronous copies
      VO_CK(ctx, cudaStreamSynchronize(ctx->stream));
      float ms = 0;
      cudaEventElapsedTime(&ms, ctx->ev[4], ctx->ev[5]);
      dil_ms += ms;
    }
    dfree(ctx, dvols);
    dfree(ctx, dqueue);
    dfree(ctx, dnext);
    for (auto &d : dils) {
      dfree(ctx, d.zf);
      dfree(ctx, d.E);
      dfree(ctx, d.maxbits);
      dfree(ctx, d.counts);
      dfree(ctx, d.pairs);
    }
  }
  // ---- outputs, then volumes whose columns overflowed a slot run the plain path
  std::vector<int> hflags(n + 1, 0);
  if (!rc) {
    cudaMemcpyAsync(hflags.data(), d_flags, sizeof(int) * (n + 1), cudaMemcpyDeviceToHost, ctx->stream);
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) rc = cuda_error(ctx, e, "batched morphology");
  }
  for (int v = 0; v < n && !rc; ++v) {
    outs[v] = nullptr;
    if (hflags[v] || hflags[n]) continue;
    rc = slot_to_volume(ctx, cur[v], &outs[v]);
  }
  for (auto &o : owned) slot_free(ctx, o);
  dfree(ctx, d_max);
  dfree(ctx, d_flags);
  int reruns = 0;
  for (int v = 0; v < n && !rc; ++v) {
    if (outs[v]) continue;
    ++reruns;
    vo_timings t;
    std::memset(&t, 0, sizeof t);
    vo_volume *o = nullptr;
    switch (ops[v]) {
      case VO_DILATION:
        rc = dilate(ctx, VO_METHOD_FAST, radii[v], ins[v], &o, &t);
        break;
      case VO_EROSION:
        rc = erode(ctx, VO_METHOD_FAST, radii[v], ins[v], &o, &t);
        break;
      default: {
        vo_volume *tmp = nullptr;
        rc = ops[v] == VO_OPENING ? erode(ctx, VO_METHOD_FAST, radii[v], ins[v], &tmp, &t)
                                  : dilate(ctx, VO_METHOD_FAST, radii[v], ins[v], &tmp, &t);
        if (!rc)
          rc = ops[v] == VO_OPENING ? dilate(ctx, VO_METHOD_FAST, radii[v], tmp, &o, &t)
                                    : erode(ctx, VO_METHOD_FAST, radii[v], tmp, &o, &t);
        if (tmp) vo_volume_free(ctx, tmp);
      }
    }
    outs[v] = o;
  }
  if (rc) {
    for (int v = 0; v < n; ++v)
      if (outs[v]) {
        vo_volume_free(ctx, outs[v]);
        outs[v] = nullptr;
      }
    return rc;
  }
  VO_CK(ctx, cudaStreamSynchronize(ctx->stream));
  if (tm) {
    std::memset(tm, 0, sizeof *tm);
    tm->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    tm->pass2_ms = dil_ms;
    tm->kernel_ms[3] = dil_ms;
    for (int v = 0; v < n; ++v) {
      tm->in_segments += ins[v]->nseg;
      tm->out_segments += outs[v]->nseg;
    }
    tm->kernel_launches = ctx->launches - launches0;
    tm->overflow_columns = reruns;
  }
  return VO_OK;
}

}  // namespace vo
