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
#include <cmath>
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
  const int32_t *offs;
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
// The interval under the cursor is cached in registers (values cv, identities
// cli/chi/clda/chda) and written back when the cursor moves or a source column
// ends, so extending it touches no memory. The four source columns of a
// (|dx|, |dy|) pair share one loop.
__device__ int fast_column(const FastArgs &A, float E, int x, int y, float2 *sv, int stride, UnionIds &U,
                           double2 *out) {
  int n = 0;
#define SV(k) sv[(k) * stride]
  for (int p = 0; p < A.npairs; ++p) {
    const int2 ad = A.pairs[p];
    const int a = ad.x, d = ad.y;
    const float h = A.Hf[d * A.W + a];
    const int da = d | (a << 8);
    // segment ranges of the (up to four) source columns of this pair
    int kb[4], ke[4];
#pragma unroll
    for (int s = 0; s < 4; ++s) {
      const int xs = (s & 1) ? x + a : x - a;
      const int ys = (s & 2) ? y + d : y - d;
      const bool ok = !((s & 1) && a == 0) && !((s & 2) && d == 0) && xs >= 0 && xs < A.nx && ys >= 0 &&
                      ys < A.ny;
      const int c = xs + A.nx * ys;
      kb[s] = ok ? A.offs[c] : 0;
      ke[s] = ok ? A.offs[c + 1] : 0;
    }
    int s = 0, k = kb[0], kend = ke[0];
    int cur = 0;
    float2 cv = n > 0 ? SV(0) : make_float2(0.f, 0.f);
    int cli = 0, chi = 0, clda = 0, chda = 0;  // identities of U[cur] (valid when cached)
    bool cached = false;                       // cached identities differ from U[cur] in memory
    bool loaded = false;                       // cli.. hold U[cur]'s identities
#define LOAD_IDS()                 \
  if (!loaded) {                   \
    cli = U.li[cur];               \
    chi = U.hi_i[cur];             \
    clda = U.lda[cur];             \
    chda = U.hda[cur];             \
    loaded = true;                 \
  }
#define FLUSH()                    \
  if (cached) {                    \
    U.li[cur] = cli;               \
    U.hi_i[cur] = chi;             \
    U.lda[cur] = clda;             \
    U.hda[cur] = chda;             \
    SV(cur) = cv;                  \
    cached = false;                \
  }
    for (;;) {
      while (k >= kend) {
        // next source column: write back the cached interval, restart the cursor
        FLUSH();
        if (++s >= 4) break;
        k = kb[s];
        kend = ke[s];
        cur = 0;
        loaded = false;
        if (n > 0) cv = SV(0);
      }
      if (s >= 4) break;
      const float2 zf = *reinterpret_cast<const float2 *>(A.zf + 2 * k);
      const float lo = zf.x - h, hi = zf.y + h;
      const int il = 2 * k, ih = 2 * k + 1;
      ++k;
      // skip union intervals that end strictly below the candidate: U.hi[cur] < lo
      while (cur < n) {
        const float t = lo - cv.y;
        bool below;
        if (t > E) {
          below = true;
        } else if (t < -E) {
          below = false;
        } else {
          FLUSH();
          below = ex_u_lt_c(A, U, cur, true, il, da, false);
        }
        if (!below) break;
        FLUSH();
        ++cur;
        loaded = false;
        if (cur < n) cv = SV(cur);
      }
      if (cur < n) {
        // covered: U.lo[cur] <= lo and hi <= U.hi[cur]
        if (lo - cv.x > E && cv.y - hi > E) continue;  // fast accept
        FLUSH();
        const bool lo_in = !GUARD(cv.x - lo, E, ex_c_lt_u(A, U, il, da, false, cur, false));
        if (lo_in && !GUARD(hi - cv.y, E, ex_u_lt_c(A, U, cur, true, ih, da, true))) continue;
      }
      FLUSH();
      if (cur == n || GUARD(cv.x - hi, E, ex_c_lt_u(A, U, ih, da, true, cur, false))) {
        // disjoint: insert before cur
        if (n >= kKA) return -1;
        for (int j = n; j > cur; --j) {
          SV(j) = SV(j - 1);
          U.li[j] = U.li[j - 1];
          U.hi_i[j] = U.hi_i[j - 1];
          U.lda[j] = U.lda[j - 1];
          U.hda[j] = U.hda[j - 1];
        }
        cv = make_float2(lo, hi);
        cli = il;
        chi = ih;
        clda = da;
        chda = da;
        loaded = true;
        cached = true;
        ++n;
        continue;
      }
      // overlapping or touching U[cur]: extend it (in registers)
      LOAD_IDS();
      if (GUARD(cv.x - lo, E, ex_c_lt_u(A, U, il, da, false, cur, false))) {
        cv.x = lo;
        cli = il;
        clda = da;
        cached = true;
      }
      if (GUARD(hi - cv.y, E, ex_u_lt_c(A, U, cur, true, ih, da, true))) {
        cv.y = hi;
        chi = ih;
        chda = da;
        cached = true;
        // absorb following intervals that now start at or below the new end
        FLUSH();
        int j = cur + 1;
        while (j < n) {
          const float2 nv = SV(j);
          if (GUARD(nv.x - cv.y, E, ex_u_lt_u(A, U, cur, true, j, false))) break;  // U.hi[cur] < U.lo[j]
          if (GUARD(nv.y - cv.y, E, ex_u_lt_u(A, U, cur, true, j, true))) {       // U.hi[cur] < U.hi[j]
            cv.y = nv.y;
            U.hi_i[cur] = U.hi_i[j];
            U.hda[cur] = U.hda[j];
            SV(cur) = cv;
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
        loaded = false;
      }
    }
#undef LOAD_IDS
#undef FLUSH
  }
#undef SV
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
  const int n = fast_column(A, E, x, y, sv + tid, kFB * kFBY, U, staging + (size_t)c * kKA);
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
        for (int k = A.offs[cs]; k < A.offs[cs + 1] && ok; ++k)
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
  FastArgs A{nx, ny, h.W, in->offs, (const double *)in->z, zf, T->Hf, T->H, dpairs, (int)pairs.size(), dE};
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

}  // namespace vo
