// Exact separable dilation with FP32 envelope arithmetic and an FP64 guard
// (VO_METHOD_FAST, and the engine of batch plans).
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
// (FP32 values in shared memory, endpoint identities in local memory).
// Candidate endpoints are formed in FP32 (FP32 copies of the inputs and of H);
// every comparison is decided in FP32 when the values differ by more than a
// guard band E bounding the FP32 error, and otherwise re-evaluated exactly in
// FP64 from the candidate's identity (input value index, d, a). Output
// endpoints are always recomputed in FP64 from their identities, so results
// are bit-identical to the FP64 oracle.
//
// Dominance: a source column whose segments all lie in segments of its
// neighbour one lattice step toward the output column, widened by at most the
// growth dH of H over that step, adds nothing that neighbour's candidates do
// not cover, and is skipped. Both bounds are computed with directed rounding,
// so skipping never changes the union.
//
// Capacities: the main kernels keep KA union slots per column (KA in
// {24, 32, 48, 64}, chosen per input density or by the batch autotuner; one
// slot holds the sentinel, so KA - 1 intervals); columns that need more are
// re-run by the same code with kUnionCapMid (128) slots (count, then fill),
// and beyond that by an FP64 kernel with a large working list in global
// scratch.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <vector>

#include <cuda_fp16.h>

#include "vo_internal.cuh"

namespace vo {
namespace {

constexpr int kKM = kUnionCapMid;  // union capacity of the second tier
// Block shape of k_fast: one warp (one patch of columns), at most 64
// registers so that 32 warps fit an SM; measured faster than four-warp blocks
// at 80 registers (305 vs 340 ms on the 2048^2 r=32 dilation).
constexpr int kFB = kFastCols, kFBY = 1;
constexpr int kBigCap = 8192;    // FP64 fallback working list (intervals)
constexpr int kBigThreads = 32;
constexpr int kMidThreads = 32;

// Identities of union endpoints, kept in local memory and read only when an
// FP32 comparison falls inside the guard band or the output is written.
template <int KA>
struct UnionIds {
  // (input value index, d | a << 8) of the lower / upper endpoint
  int2 lo[KA], hi[KA];
};

__device__ __forceinline__ double exact_val(const FastArgs &A, int idx, int da, bool plus) {
  const double h = A.H64[(da & 255) * A.W + (da >> 8)];
  const double z = A.zd[idx];
  return plus ? __dadd_rn(z, h) : __dsub_rn(z, h);
}

// Exact comparisons, out of line: identities are loaded only here.
// Union endpoint (j, hi?) < candidate endpoint (idx, da, plus)?
template <int KA>
__device__ __noinline__ bool ex_u_lt_c(const FastArgs &A, const UnionIds<KA> &U, int j, bool jhi, int idx, int da,
                                       bool plus) {
  const double u = jhi ? exact_val(A, U.hi[j].x, U.hi[j].y, true) : exact_val(A, U.lo[j].x, U.lo[j].y, false);
  return u < exact_val(A, idx, da, plus);
}
// Candidate endpoint < union endpoint?
template <int KA>
__device__ __noinline__ bool ex_c_lt_u(const FastArgs &A, const UnionIds<KA> &U, int idx, int da, bool plus, int j,
                                       bool jhi) {
  const double u = jhi ? exact_val(A, U.hi[j].x, U.hi[j].y, true) : exact_val(A, U.lo[j].x, U.lo[j].y, false);
  return exact_val(A, idx, da, plus) < u;
}
// Union endpoint (i, ihi) < union endpoint (j, jhi)?
template <int KA>
__device__ __noinline__ bool ex_u_lt_u(const FastArgs &A, const UnionIds<KA> &U, int i, bool ihi, int j, bool jhi) {
  const double a = ihi ? exact_val(A, U.hi[i].x, U.hi[i].y, true) : exact_val(A, U.lo[i].x, U.lo[i].y, false);
  const double b = jhi ? exact_val(A, U.hi[j].x, U.hi[j].y, true) : exact_val(A, U.lo[j].x, U.lo[j].y, false);
  return a < b;
}

// The FP16 in the low (lo != 0) or high half of v.
__device__ __forceinline__ __half half_of(unsigned v, int lo) {
  return __ushort_as_half((unsigned short)(lo ? (v & 0xffffu) : (v >> 16)));
}

// FP32 difference t = y - x decides x < y outside the guard band [-E, E].
#define GUARD(t, E, exact) ((t) > (E) ? true : ((t) < -(E) ? false : (exact)))

// Returns the number of intervals of the union (identities in U), or -1 when
// more than KA - 1 are needed (the last of the KA slots holds the sentinel).
//
// `mask` holds the lanes of the warp running this function together. For each
// (|dx|, |dy|) pair the four source columns' segments form one list per lane;
// every lane of the warp iterates to the warp's longest list with a predicate,
// and the loop body has no early exits, so the lanes reconverge after every
// candidate instead of drifting apart over the source transitions.
template <int KA>
__device__ int fast_column(const FastArgs &A, float E, int x, int y, float2 *sv, int stride, UnionIds<KA> &U,
                           unsigned mask) {
  int n = 0;
  bool overflow = false;
#define SV(k) sv[(k) * stride]
  // SV(n) holds a sentinel above every value, so the cursor walk stops at
  // the end of the union without a bounds test; the union holds up to KA - 1
  // intervals.
  const float2 kTop = make_float2(INFINITY, INFINITY);
  SV(0) = kTop;
  // Per pair: its four source columns' records and their segment dominance
  // masks at the pair's levels, loaded when the pair starts (only the pair's
  // own table entry is loaded one pair ahead: holding the source records
  // across the merge loop cost more in register spills than their load
  // latency, which the other resident warps hide).
  // Source S: x + a if S & 1 (its neighbour toward the output is at x - 1,
  // direction "x-" = 0), else x - a ("x+" = 1); likewise y with S & 2
  // ("y-" = 2, "y+" = 3).
  const int ncols = A.nx * A.ny;
  const int mbits = A.mask_bits;
#define MASK(DIR, LV, C)                                                                                \
  ((LV) < kDomLevels ? (mbits == 16 ? (unsigned)static_cast<const unsigned short *>(A.dmask)[((DIR) * kDomLevels + (LV)) * ncols + (C)] \
                                    : static_cast<const unsigned *>(A.dmask)[((DIR) * kDomLevels + (LV)) * ncols + (C)])        \
                     : 0u)
#define LOAD_ONE(OK, XS, YS, S, R, D)                                                                   \
  {                                                                                                     \
    const int c_ = (OK) ? (XS) + A.nx * (YS) : 0;                                                       \
    R = (OK) ? reinterpret_cast<const int2 *>(A.col)[2 * c_] : make_int2(0, 0);                          \
    D = (OK) ? (MASK((S) & 1 ? 0 : 1, lx_, c_) | MASK((S) & 2 ? 2 : 3, ly_, c_)) : 0u;                  \
  }
#define LOAD_SOURCES(PR)                                                                                \
  {                                                                                                     \
    const int ad_ = __float_as_int((PR).x), a_ = ad_ & 0xff, d_ = (ad_ >> 8) & 0xff;                    \
    const int lx_ = (ad_ >> 16) & 0xf, ly_ = (ad_ >> 20) & 0xf;                                         \
    const bool xm = x - a_ >= 0, xp = a_ > 0 && x + a_ < A.nx;                                          \
    const bool ym = y - d_ >= 0, yp = d_ > 0 && y + d_ < A.ny;                                          \
    LOAD_ONE(xm && ym, x - a_, y - d_, 0, c0, d0)                                                       \
    LOAD_ONE(xp && ym, x + a_, y - d_, 1, c1, d1)                                                       \
    LOAD_ONE(xm && yp, x - a_, y + d_, 2, c2, d2)                                                       \
    LOAD_ONE(xp && yp, x + a_, y + d_, 3, c3, d3)                                                       \
  }
  float4 pr = A.prec[0];
  for (int p = 0; p < A.npairs; ++p) {
    const float4 pc = pr;
    if (p + 1 < A.npairs) pr = A.prec[p + 1];
    int2 c0, c1, c2, c3;  // (beg, end) of each source column
    unsigned d0, d1, d2, d3;
    LOAD_SOURCES(pc)
    const int ad = __float_as_int(pc.x), a = ad & 0xff, d = (ad >> 8) & 0xff;
    const float h = pc.y;
    const int da = d | (a << 8);
    // growth of H over one step toward the output column (x step, y step),
    // against which the sources' dominance widths are tested
    const float dhx = pc.z, dhy = pc.w;
    // FP16 bounds of the pair's growths (rounded down) for the source tests
    const __half dhx_h = __float2half_rd(dhx), dhy_h = __float2half_rd(dhy);
    // Per source: [kb, ke) and the mask of its kept segments (bit j: segment
    // kb + j); a source of more than mbits segments keeps all (m = 0, dense).
    // A source of up to mbits segments that is dominated whole has an empty kept
    // mask; a source of more segments (no masks) is tested with its column
    // widths.
#define SRC(S, XS, YS, C, DM, KB, KE, M)                                                                \
  {                                                                                                     \
    KB = (C).x;                                                                                         \
    KE = (C).y;                                                                                         \
    const int ns_ = KE - KB;                                                                            \
    if (ns_ > mbits) {                                                                                  \
      const int4 cr_ = A.col[(XS) + A.nx * (YS)];                                                       \
      if (__hle(half_of((unsigned)cr_.z, (S) & 1), dhx_h) || __hle(half_of((unsigned)cr_.w, (S) & 2), dhy_h)) \
        KE = KB;                                                                                        \
    }                                                                                                   \
    M = ns_ <= mbits ? ~(DM) & (ns_ == 32 ? 0xffffffffu : ((1u << ns_) - 1u)) : 0u;                    \
  }
    int kb0, ke0, kb1, ke1, kb2, ke2, kb3, ke3;
    unsigned m0, m1, m2, m3;
    SRC(0, x - a, y - d, c0, d0, kb0, ke0, m0)
    SRC(1, x + a, y - d, c1, d1, kb1, ke1, m1)
    SRC(2, x - a, y + d, c2, d2, kb2, ke2, m2)
    SRC(3, x + a, y + d, c3, d3, kb3, ke3, m3)
#undef SRC
#define KEPT(KB, KE, M) ((KE) - (KB) > mbits ? (KE) - (KB) : __popc(M))
    const int t0 = KEPT(kb0, ke0, m0), t1 = KEPT(kb1, ke1, m1), t2 = KEPT(kb2, ke2, m2), t3 = KEPT(kb3, ke3, m3);
#undef KEPT
    const int total = t0 + t1 + t2 + t3;
    const int iters = __reduce_max_sync(mask, total);
    // Walk state: the sources still to visit that keep candidates (bit s),
    // the current source s, its remaining mask ms (sparse) or next index kc
    // (dense); NEXT yields the next kept candidate (KN, SN), or KN = -1. A
    // source is entered only when it keeps a candidate, so NEXT takes at most
    // one source switch and no loop.
    unsigned srcs = (t0 > 0 ? 1u : 0u) | (t1 > 0 ? 2u : 0u) | (t2 > 0 ? 4u : 0u) | (t3 > 0 ? 8u : 0u);
    int s = -1, kc = 0, kend = 0, kbs = 0;
    unsigned ms = 0;
    bool dense = false;
#define NEXT(KN, SN)                                                                                    \
  {                                                                                                     \
    if ((dense ? kc >= kend : ms == 0u) && srcs) {                                                      \
      s = __ffs(srcs) - 1;                                                                              \
      srcs &= srcs - 1;                                                                                 \
      kbs = s == 0 ? kb0 : s == 1 ? kb1 : s == 2 ? kb2 : kb3;                                           \
      kend = s == 0 ? ke0 : s == 1 ? ke1 : s == 2 ? ke2 : ke3;                                          \
      ms = s == 0 ? m0 : s == 1 ? m1 : s == 2 ? m2 : m3;                                                \
      dense = kend - kbs > mbits;                                                                       \
      kc = kbs;                                                                                         \
    }                                                                                                   \
    KN = -1;                                                                                            \
    if (dense) {                                                                                        \
      if (kc < kend) KN = kc++;                                                                         \
    } else if (ms) {                                                                                    \
      KN = kbs + __ffs(ms) - 1;                                                                         \
      ms &= ms - 1;                                                                                     \
    }                                                                                                   \
    SN = s;                                                                                             \
  }
    int cur = 0, cur_src = -1;
    float2 cv = make_float2(0.f, 0.f);
    int kn, sn;
    NEXT(kn, sn)
    float2 znext = kn >= 0 ? *reinterpret_cast<const float2 *>(A.zf + 2 * kn) : make_float2(0.f, 0.f);
    for (int it = 0; it < iters; ++it) {
      if (it < total && !overflow) {
        const int k = kn, src = sn;
        const float2 zf = znext;
        NEXT(kn, sn)
        if (kn >= 0) znext = *reinterpret_cast<const float2 *>(A.zf + 2 * kn);
        if (src != cur_src) {  // first candidate of a new source column: restart the cursor
          cur_src = src;
          cur = 0;
          cv = SV(0);
        }
        {
          const float lo = zf.x - h, hi = zf.y + h;
          const int il = 2 * k, ih = 2 * k + 1;
          // skip union intervals that end strictly below the candidate: U.hi[cur] < lo
          // (the next interval's values are loaded one step ahead)
          if (lo - cv.y > E) {  // two intervals per step: cur < n here, so cur + 1 <= n
            float2 c1 = SV(cur + 1), c2 = SV(min(cur + 2, n));
            for (;;) {
              if (!(lo - c1.y > E)) {
                cur += 1;
                cv = c1;
                break;
              }
              if (!(lo - c2.y > E)) {
                cur += 2;
                cv = c2;
                break;
              }
              cur += 2;
              c1 = SV(cur + 1);
              c2 = SV(min(cur + 2, n));
            }
          }
          while (cur < n && GUARD(lo - cv.y, E, ex_u_lt_c(A, U, cur, true, il, da, false))) {
            ++cur;
            cv = SV(cur);
          }
          // covered: inside U[cur]; else ext_lo / ext_hi: the candidate reaches
          // below / above U[cur] (both decided once, used again to extend it)
          bool covered = false, ext_lo = false, ext_hi = false;
          if (cur < n) {
            if (lo - cv.x > E && cv.y - hi > E) {
              covered = true;  // inside U[cur] by more than the guard band
            } else {
              ext_lo = GUARD(cv.x - lo, E, ex_c_lt_u(A, U, il, da, false, cur, false));
              ext_hi = GUARD(hi - cv.y, E, ex_u_lt_c(A, U, cur, true, ih, da, true));
              covered = !ext_lo && !ext_hi;
            }
          }
          if (!covered) {
            if (cur == n || GUARD(cv.x - hi, E, ex_c_lt_u(A, U, ih, da, true, cur, false))) {
              // disjoint: insert before cur
              if (n >= KA - 1) {
                overflow = true;
              } else {
                for (int j = n; j > cur; --j) {
                  SV(j) = SV(j - 1);
                  U.lo[j] = U.lo[j - 1];
                  U.hi[j] = U.hi[j - 1];
                }
                cv = make_float2(lo, hi);
                SV(cur) = cv;
                U.lo[cur] = make_int2(il, da);
                U.hi[cur] = make_int2(ih, da);
                ++n;
                SV(n) = kTop;
              }
            } else {
              // overlapping or touching U[cur]: extend it
              if (ext_lo) {
                cv.x = lo;
                U.lo[cur] = make_int2(il, da);
              }
              if (ext_hi) {
                cv.y = hi;
                U.hi[cur] = make_int2(ih, da);
                // absorb following intervals that now start at or below the new end
                int j = cur + 1;
                while (j < n) {
                  const float2 nv = SV(j);
                  if (GUARD(nv.x - cv.y, E, ex_u_lt_u(A, U, cur, true, j, false))) break;  // U.hi[cur] < U.lo[j]
                  if (GUARD(nv.y - cv.y, E, ex_u_lt_u(A, U, cur, true, j, true))) {       // U.hi[cur] < U.hi[j]
                    cv.y = nv.y;
                    U.hi[cur] = U.hi[j];
                  }
                  ++j;
                }
                const int gone = j - cur - 1;
                if (gone > 0) {
                  for (int m = cur + 1; m + gone < n; ++m) {
                    SV(m) = SV(m + gone);
                    U.lo[m] = U.lo[m + gone];
                    U.hi[m] = U.hi[m + gone];
                  }
                  n -= gone;
                  SV(n) = kTop;
                }
              }
              SV(cur) = cv;
            }
          }
        }
      }
    }
  }
#undef SV
#undef LOAD_SOURCES
#undef LOAD_ONE
#undef MASK
#undef NEXT
  return overflow ? -1 : n;
}

// Writes the exact FP64 union held by U (n intervals) to out[0..n).
template <int KA>
__device__ __forceinline__ void write_union(const FastArgs &A, const UnionIds<KA> &U, int n, double2 *out) {
  for (int k = 0; k < n; ++k)
    out[k] = make_double2(exact_val(A, U.lo[k].x, U.lo[k].y, false), exact_val(A, U.hi[k].x, U.hi[k].y, true));
}

// One pass: the exact union of every output column goes to its fixed-capacity
// staging slot (KA entries, at most KA - 1 used) with its count; columns that need more are
// listed for the second tier. A compaction pass then packs the slots.
template <int KA>
__global__ void __launch_bounds__(kFB *kFBY, 1024 / (kFB * kFBY)) k_fast(FastArgs A, int32_t *counts,
                                                                          double2 *staging,
                                                    int *ovf_count, int *ovf_cols) {
  extern __shared__ float2 sv_dyn[];
  const int tid = threadIdx.x + kFB * threadIdx.y;
  // blocks (patches) in bands of 512 columns, all rows of a band before the next: the blocks running
  // together cover a compact region, whose source columns stay in L2
  constexpr int kBand = 512 / kPatchX;
  const int tiles_x = (A.nx + kPatchX - 1) / kPatchX, tiles_y = (A.ny + kPatchY - 1) / kPatchY;
  const int band = (int)blockIdx.x / (kBand * tiles_y);
  const int rb = (int)blockIdx.x - band * kBand * tiles_y;
  const int bw = min(kBand, tiles_x - band * kBand);
  const int x = (band * kBand + rb % bw) * kPatchX + threadIdx.x % kPatchX;
  const int y = (rb / bw) * kPatchY + threadIdx.x / kPatchX;
  if (x >= A.nx || y >= A.ny) return;
  const int c = x + A.nx * y;
  const float E = *A.E;
  UnionIds<KA> U;
  const unsigned mask = __activemask();
  const int n = fast_column<KA>(A, E, x, y, sv_dyn + tid, kFB * kFBY, U, mask);
  if (n > 0) write_union(A, U, n, staging + (size_t)c * KA);
  if (n < 0) {
    ovf_cols[atomicAdd(ovf_count, 1)] = c;
    counts[c] = 0;
  } else {
    counts[c] = n;
  }
}

// Packs the staging slots (ka intervals each) of the columns that fit into
// the CSR output.
__global__ void k_compact(int ncols, int ka, const int32_t *__restrict__ counts,
                          const double2 *__restrict__ staging, const int32_t *__restrict__ ooffs,
                          double2 *__restrict__ oz) {
  // one warp per column, lanes over intervals
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (w >= ncols) return;
  const int n = ooffs[w + 1] - ooffs[w];
  if (n > ka) return;  // written by the second tier
  for (int k = lane; k < n; k += 32) oz[ooffs[w] + k] = staging[(size_t)w * ka + k];
}

// Second tier over the columns listed by k_fast (grid-stride): the same
// computation with kKM slots (kKM - 1 intervals). Count pass: counts[c], or the
// column goes to the FP64 list when even that is exceeded. Fill pass: writes the union at its
// CSR offset (columns of the FP64 list are left to it).
template <bool FILL>
__global__ void __launch_bounds__(kMidThreads) k_fast_mid(FastArgs A, int32_t *counts, const int32_t *ooffs,
                                                          double2 *oz, const int *list_count, const int *list,
                                                          int *big_count, int *big_list) {
  __shared__ float2 sv[kKM * kMidThreads];
  const float E = *A.E;
  const int m = *list_count;
  const int nth = gridDim.x * kMidThreads;
  for (int i = blockIdx.x * kMidThreads + threadIdx.x; i < m; i += nth) {
    const int c = list[i];
    const int x = c % A.nx, y = c / A.nx;
    UnionIds<kKM> U;
    const unsigned mask = __activemask();
    const int n = fast_column<kKM>(A, E, x, y, sv + threadIdx.x, kMidThreads, U, mask);
    if (FILL) {
      if (n >= 0) write_union(A, U, n, oz + ooffs[c]);
    } else if (n < 0) {
      big_list[atomicAdd(big_count, 1)] = c;
      counts[c] = 0;
    } else {
      counts[c] = n;
    }
  }
}

// FP64 re-run of columns whose union outgrew kKM: same candidate set, exact
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

// Guard band: E bounds the error of an FP32 comparison t = y - x of two
// candidate endpoints (each within 1.5 ulp of its FP64 value: rounding of z,
// of H and of the sum), plus the rounding of t itself: 4 ulp32(U) for
// magnitudes up to U; E = 2^-20 * U leaves a factor two of margin.
__global__ void k_guard(const unsigned int *maxabs_bits, float R, float *E) {
  const float U = __uint_as_float(*maxabs_bits) + R + 1.0f;
  *E = U * 9.5367431640625e-07f;  // 2^-20
}

// Lower bounds of the growth of H per lattice step toward the centre.
__global__ void k_dh_tables(int Dy, int W, const double *__restrict__ H, const int *__restrict__ Dx,
                            float *__restrict__ dH) {
  const int n = (Dy + 1) * W;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const int d = i / W, a = i % W;
  float fx = -INFINITY, fy = -INFINITY;
  if (a <= Dx[d]) {
    if (a >= 1) fx = __double2float_rd(__dsub_rd(H[d * W + a - 1], H[i]));
    if (d >= 1) fy = __double2float_rd(__dsub_rd(H[(d - 1) * W + a], H[i]));
  }
  dH[i] = fx;
  dH[n + i] = fy;
}

// Dominance widths, one thread per column. For segment i and direction k
// (neighbour (x-1, y), (x+1, y), (x, y-1), (x, y+1)):
//   w_i = min over the neighbour's segments j of max(z1_j - z1_i, z2_i - z2_j),
// evaluated in FP32 on bounds of the FP64 values with every difference
// rounded up, so w bounds the exact value from above (+inf outside the grid
// or without a neighbour segment). The scan stops after the
// first neighbour segment starting above segment i: every later neighbour
// segment gives a larger value. The column's width per direction is the max
// over its segments (-inf for an empty column), stored as FP16 rounded up in
// the column record col[c] = (beg, end, x- | x+ << 16, y- | y+ << 16).
__global__ void k_dominance(int nx, int ny, const int32_t *__restrict__ beg, const int32_t *__restrict__ end,
                            const float2 *__restrict__ zf, int4 *__restrict__ col, void *__restrict__ dmask,
                            int mask_bits, const DomLevels L) {
  const int ncols = nx * ny;
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncols) return;
  const int x = c % nx, y = c / nx;
  const int k0 = beg[c], k1 = end[c];
  int nb0[4], nb1[4];
  for (int k = 0; k < 4; ++k) {
    const int xn = x + (k == 0 ? -1 : k == 1 ? 1 : 0), yn = y + (k == 2 ? -1 : k == 3 ? 1 : 0);
    const bool in = xn >= 0 && xn < nx && yn >= 0 && yn < ny;
    const int cn = in ? xn + nx * yn : 0;
    nb0[k] = in ? beg[cn] : 0;
    nb1[k] = in ? end[cn] : 0;
  }
  float cmax[4] = {-INFINITY, -INFINITY, -INFINITY, -INFINITY};
  unsigned bits[4][kDomLevels];
  for (int k = 0; k < 4; ++k)
    for (int l = 0; l < kDomLevels; ++l) bits[k][l] = 0u;
  const bool masked = k1 - k0 <= mask_bits;
  for (int i = k0; i < k1; ++i) {
    // bounds of the exact values: an FP32 copy is within half an ulp of its
    // FP64 value, so the neighbouring floats enclose it
    const float2 fi = zf[i];
    const float i1 = nextafterf(fi.x, -INFINITY), i2 = nextafterf(fi.y, INFINITY);
    for (int k = 0; k < 4; ++k) {
      float best = INFINITY;
      for (int j = nb0[k]; j < nb1[k]; ++j) {
        const float2 fj = zf[j];
        const float lo = __fsub_ru(nextafterf(fj.x, INFINITY), i1);
        const float hi = __fsub_ru(i2, nextafterf(fj.y, -INFINITY));
        const float m = lo > hi ? lo : hi;
        best = m < best ? m : best;
        if (fj.x > fi.y) break;  // any early stop only leaves the bound larger
      }
      cmax[k] = best > cmax[k] ? best : cmax[k];
      if (masked)
        for (int l = 0; l < kDomLevels; ++l)
          if (best <= L.t[l]) bits[k][l] |= 1u << (i - k0);
    }
  }
  if (dmask)
    for (int k = 0; k < 4; ++k)
      for (int l = 0; l < kDomLevels; ++l) {
        const size_t idx = (size_t)(k * kDomLevels + l) * ncols + c;
        if (mask_bits == 16) static_cast<unsigned short *>(dmask)[idx] = (unsigned short)bits[k][l];
        else static_cast<unsigned *>(dmask)[idx] = bits[k][l];
      }
  unsigned h[4];
  for (int k = 0; k < 4; ++k) h[k] = __half_as_ushort(__float2half_ru(cmax[k]));
  col[c] = make_int4(k0, k1, (int)(h[0] | (h[1] << 16)), (int)(h[2] | (h[3] << 16)));
}

static_assert(kDomLevels <= 15, "pair records hold a level in 4 bits, 15 meaning none");

// Largest dominance level whose threshold is <= dh (15: none).
__device__ __forceinline__ int dom_level_of(float dh, const DomLevels &L) {
  int lv = 15;
  for (int l = 0; l < kDomLevels; ++l)
    if (L.t[l] <= dh) lv = l;
  return lv;
}

// Pair records: (a | d << 8 | x-step level << 16 | y-step level << 20 as
// float bits, H in FP32, dH x step, dH y step).
__global__ void k_pair_records(const int2 *__restrict__ pairs, int npairs, const float *__restrict__ Hf,
                               const float *__restrict__ dH, int W, int dHy, float4 *__restrict__ prec,
                               const DomLevels L) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npairs) return;
  const int a = pairs[p].x, d = pairs[p].y;
  const float dx = dH[d * W + a], dy = dH[dHy + d * W + a];
  const int code = a | (d << 8) | (dom_level_of(dx, L) << 16) | (dom_level_of(dy, L) << 20);
  prec[p] = make_float4(__int_as_float(code), Hf[d * W + a], dx, dy);
}

// ---------------------------------------------------------------- batches

static_assert(sizeof(BatchVol) % sizeof(int) == 0, "BatchVol is copied as ints");

// Output slot of column (x, y) of a batch dilation for an n-interval union:
// the column's own slot when its tile capacity allows, else spill space, else
// -1 (the dilation's overflow flag is then set).
__device__ __forceinline__ int place_union(const BatchVol &V, int x, int y, int n) {
  const int nx = V.A.nx;
  int cap = V.cap, dst;
  if (V.tcap) {
    const int tx = x / kSizerTile, ty = y / kSizerTile, t = tx + V.tiles32_x * ty;
    const int w = min(kSizerTile, nx - tx * kSizerTile);
    cap = V.tcap[t];
    dst = V.toff[t] + ((x - tx * kSizerTile) + w * (y - ty * kSizerTile)) * cap;
  } else {
    dst = (x + nx * y) * cap;
  }
  if (n > cap) {
    const int off = atomicAdd(V.spill_used, n);
    if (off + n <= V.spill_cap) return V.spill_base + off;
    atomicOr(V.ovf, 4);  // spill region exhausted
    return -1;
  }
  return dst;
}

// Persistent kernel over the tiles (FBY patches of 8 x 4 output columns) of every
// dilation of a batch: blocks pull (dilation, tile) items from a queue ordered
// by decreasing estimated work, so uneven volumes balance across the SMs.
// Each column's union goes to its slot (place_union); a union of more than
// KA - 1 intervals is listed for k_fast_batched_mid.
// SINGLE: the round has one dilation, whose arguments come as the kernel
// parameter A1 (constant bank) instead of from memory.
// LBN / (kFB * FBY) blocks per SM bound the registers: LBN = 1024 gives 64
// per thread (32 warps per SM, some spills), 768 gives 85 (24 warps); the
// autotuner picks per round (the first wins on the 2048^2 r=32 dilation).
template <int KA, int FBY, bool SINGLE, int LBN>
__global__ void __launch_bounds__(kFB *FBY, LBN / (kFB * FBY)) k_fast_batched(const BatchVol *vols,
                                                                               const int2 *queue, int nq, int *next,
                                                                               const FastArgs A1) {
  extern __shared__ float2 sv_dyn[];
  __shared__ int s_item;
  __shared__ BatchVol s_vol;  // the item's arguments, read by every thread in the hot loop
  const int tid = threadIdx.x + kFB * threadIdx.y;
  int cur_vol = -1;
  for (;;) {
    if (tid == 0) s_item = atomicAdd(next, 1);
    __syncthreads();
    const int item = s_item;
    if (item >= nq) return;
    const int2 q = queue[item];
    if (q.x != cur_vol) {
      for (int i = tid; i < (int)(sizeof(BatchVol) / sizeof(int)); i += kFB * FBY)
        reinterpret_cast<int *>(&s_vol)[i] = reinterpret_cast<const int *>(&vols[q.x])[i];
      cur_vol = q.x;
    }
    __syncthreads();
    const BatchVol &V = s_vol;
    const int nx = V.A.nx, ny = V.A.ny;
    const int bw = kPatchX * FBY;  // the item's columns: bw x kPatchY, warp w at x offset w * kPatchX
    const int tiles_x = (nx + bw - 1) / bw;
    const int x = (q.y % tiles_x) * bw + threadIdx.y * kPatchX + threadIdx.x % kPatchX;
    const int y = (q.y / tiles_x) * kPatchY + threadIdx.x / kPatchX;
    if (x < nx && y < ny) {
      const int c = x + nx * y;
      UnionIds<KA> U;
      const unsigned mask = __activemask();
      const FastArgs &A = SINGLE ? A1 : V.A;
      int n = fast_column<KA>(A, *A.E, x, y, sv_dyn + tid, kFB * FBY, U, mask);
      int dst = 0;
      if (n < 0) {
        V.mid_list[atomicAdd(V.mid_count, 1)] = c;
        n = 0;
      } else {
        dst = place_union(V, x, y, n);
        if (dst < 0) {
          dst = 0;
          n = 0;
        } else {
          write_union(A, U, n, V.oz + dst);
        }
      }
      V.obeg[c] = dst;
      V.oend[c] = dst + n;
    }
  }
}

// Second tier of a batch round: the listed columns of every dilation with
// kKM slots, placed like the first tier; a union of more than kKM - 1
// intervals sets the dilation's overflow flag.
__global__ void __launch_bounds__(kMidThreads) k_fast_batched_mid(const BatchVol *vols, int nv) {
  __shared__ float2 sv[kKM * kMidThreads];
  const int nth = gridDim.x * kMidThreads;
  for (int v = 0; v < nv; ++v) {
    const BatchVol &V = vols[v];
    const int m = *V.mid_count;
    for (int i = blockIdx.x * kMidThreads + threadIdx.x; i < m; i += nth) {
      const int c = V.mid_list[i];
      const int x = c % V.A.nx, y = c / V.A.nx;
      UnionIds<kKM> U;
      const unsigned mask = __activemask();
      int n = fast_column<kKM>(V.A, *V.A.E, x, y, sv + threadIdx.x, kMidThreads, U, mask);
      int dst = -1;
      if (n < 0) {
        V.big_list[atomicAdd(V.big_count, 1)] = c;  // third tier
        n = 0;
        dst = 0;
      } else {
        dst = place_union(V, x, y, n);
      }
      if (dst < 0) {
        dst = 0;
        n = 0;
      } else if (n > 0) {
        write_union(V.A, U, n, V.oz + dst);
      }
      V.obeg[c] = dst;
      V.oend[c] = dst + n;
    }
  }
}

// Third tier of a batch round (FP64, grid-stride): the columns whose union
// exceeds kKM, each built in a kBigCap-interval list in global scratch and
// placed like the other tiers; a union beyond kBigCap sets the overflow flag.
__global__ void __launch_bounds__(kBigThreads) k_fast_batched_big(const BatchVol *vols, int nv, double2 *scratch) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;
  double2 *L = scratch + (size_t)tid * kBigCap;
  for (int v = 0; v < nv; ++v) {
    const BatchVol &V = vols[v];
    const FastArgs &A = V.A;
    const int m = *V.big_count;
    for (int i = tid; i < m; i += nth) {
      const int c = V.big_list[i];
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
      int dst = -1;
      if (!ok)
        atomicOr(V.ovf, 1);
      else
        dst = place_union(V, x, y, n);
      if (dst < 0) {
        dst = 0;
        n = 0;
      } else {
        for (int k = 0; k < n; ++k) V.oz[dst + k] = L[k];
      }
      V.obeg[c] = dst;
      V.oend[c] = dst + n;
    }
  }
}

}  // namespace

// ================================================================ host side

namespace {

int sm_count_fast() {
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
  const std::vector<int2> pairs = fast_pairs(h);
  float *zf = nullptr, *dE = nullptr;
  int4 *col = nullptr;
  float4 *prec = nullptr;
  unsigned *dmask = nullptr;
  unsigned int *dmax = nullptr;
  int2 *dpairs = nullptr;
  int32_t *counts = nullptr;
  int *ovf_cols = nullptr, *big_cols = nullptr;
  double2 *big = nullptr;
  vo_volume *res = nullptr;
  long long total = 0;
  const int sms = sm_count_fast();
  const int gbig = sms, gmid = sms * 16;
  rc = dalloc(ctx, &zf, (size_t)std::max<int64_t>(2 * in->nseg, 2));
  if (!rc) rc = dalloc(ctx, &dE, 1);
  if (!rc) rc = dalloc(ctx, &col, (size_t)ncols);
  const int mbits = mask_bits_for((double)in->nseg / std::max(ncols, 1));
  if (!rc) rc = dalloc(ctx, &dmask, mask_words((size_t)ncols, mbits));
  if (!rc) rc = dalloc(ctx, &prec, pairs.size());
  if (!rc) rc = dalloc(ctx, &dmax, 1);
  if (!rc) rc = dalloc(ctx, &dpairs, pairs.size());
  if (!rc) rc = dalloc(ctx, &counts, (size_t)ncols);
  if (!rc) rc = dalloc(ctx, &ovf_cols, (size_t)ncols);
  if (!rc) rc = dalloc(ctx, &big_cols, (size_t)ncols);
  if (!rc) rc = dalloc(ctx, &big, (size_t)gbig * kBigThreads * kBigCap);
  if (!rc) {
    cudaMemcpyAsync(dpairs, pairs.data(), sizeof(int2) * pairs.size(), cudaMemcpyHostToDevice, ctx->stream);
    cudaMemsetAsync(ctx->d_flags, 0, 3 * sizeof(int), ctx->stream);  // [0] tier-2 list, [1] fatal, [2] FP64 list
    cudaEventRecord(ctx->ev[0], ctx->stream);
    fast_prepare(ctx->stream, nx, ny, in->offs, in->offs + 1, in->z, zf, dmax, (float)R, dE, col, dmask, mbits,
                 T->host.dom);
    fast_pair_records(ctx->stream, dpairs, (int)pairs.size(), *T, prec);
    ctx->launches += 4;
    cudaEventRecord(ctx->ev[1], ctx->stream);
  }
  FastArgs A{nx, ny, h.W, in->offs, in->offs + 1, (const double *)in->z, zf, T->Hf, T->H, dpairs,
             (int)pairs.size(), dE, col, prec, dmask, mbits};
  const dim3 blk(kFB, kFBY), grd(((nx + kPatchX - 1) / kPatchX) * ((ny + kPatchY - 1) / kPatchY));
  // union capacity from the input's mean segment count per column (24, 32,
  // 48 or 64; dense inputs take 48 up to 24 segments per column, which keeps
  // more warps per SM than 64, the rest going to the second tier)
  const double mean_segs = (double)in->nseg / std::max(ncols, 1);
  const int ka = fast_union_cap(mean_segs) == 64 ? (mean_segs > 24.0 ? 64 : 48) : fast_union_cap(mean_segs);
  const size_t smem = sizeof(float2) * ka * kFB * kFBY;
  double2 *staging = nullptr;
  if (!rc) rc = dalloc(ctx, &staging, (size_t)ncols * ka);
  if (!rc && ka == 64 &&
      cudaFuncSetAttribute(reinterpret_cast<const void *>(&k_fast<64>), cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem) != cudaSuccess)
    rc = cuda_error(ctx, cudaGetLastError(), "k_fast shared memory");
  if (!rc) {
    cudaEventRecord(ctx->ev[4], ctx->stream);
    if (ka == 64)
      k_fast<64><<<grd, blk, smem, ctx->stream>>>(A, counts, staging, ctx->d_flags, ovf_cols);
    else if (ka == 48)
      k_fast<48><<<grd, blk, smem, ctx->stream>>>(A, counts, staging, ctx->d_flags, ovf_cols);
    else if (ka == 32)
      k_fast<32><<<grd, blk, smem, ctx->stream>>>(A, counts, staging, ctx->d_flags, ovf_cols);
    else
      k_fast<24><<<grd, blk, smem, ctx->stream>>>(A, counts, staging, ctx->d_flags, ovf_cols);
    k_fast_mid<false><<<gmid, kMidThreads, 0, ctx->stream>>>(A, counts, nullptr, nullptr, ctx->d_flags, ovf_cols,
                                                               ctx->d_flags + 2, big_cols);
    k_fast_big<false><<<gbig, kBigThreads, 0, ctx->stream>>>(A, counts, nullptr, nullptr, ctx->d_flags + 2,
                                                             big_cols, big, ctx->d_flags + 1);
    ctx->launches += 3;
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
    k_compact<<<(int)(((int64_t)ncols * 32 + 255) / 256), 256, 0, ctx->stream>>>(ncols, ka, counts, staging,
                                                                                 res->offs, res->z);
    k_fast_mid<true><<<gmid, kMidThreads, 0, ctx->stream>>>(A, nullptr, res->offs, res->z, ctx->d_flags, ovf_cols,
                                                              nullptr, nullptr);
    k_fast_big<true><<<gbig, kBigThreads, 0, ctx->stream>>>(A, nullptr, res->offs, res->z, ctx->d_flags + 2,
                                                            big_cols, big, ctx->d_flags + 1);
    ctx->launches += 3;
    cudaEventRecord(ctx->ev[7], ctx->stream);
    int hf[3] = {0, 0, 0};
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
  dfree(ctx, col);
  dfree(ctx, dmask);
  dfree(ctx, prec);
  dfree(ctx, dmax);
  dfree(ctx, dpairs);
  dfree(ctx, counts);
  dfree(ctx, ovf_cols);
  dfree(ctx, big_cols);
  dfree(ctx, big);
  if (rc) {
    if (res) vo_volume_free(ctx, res);
    return rc;
  }
  *out = res;
  return VO_OK;
}

// ================================================================ batch launch helpers

std::vector<int2> fast_pairs(const Tables &h) {
  std::vector<int2> pairs;
  for (int d = 0; d <= h.Dy; ++d)
    for (int a = 0; a <= h.Dx[d]; ++a) pairs.push_back(make_int2(a, d));
  std::stable_sort(pairs.begin(), pairs.end(), [&](const int2 &p, const int2 &q) {
    return h.H[(size_t)p.y * h.W + p.x] > h.H[(size_t)q.y * h.W + q.x];
  });
  return pairs;
}

void fast_prepare(cudaStream_t st, int nx, int ny, const int32_t *beg, const int32_t *end, const double2 *z,
                  float *zf, unsigned int *maxbits, float R, float *E, int4 *col, void *dmask, int mask_bits,
                  const DomLevels &L) {
  const int ncols = nx * ny;
  cudaMemsetAsync(maxbits, 0, sizeof(unsigned int), st);
  k_to_f32_cols<<<(ncols + 255) / 256, 256, 0, st>>>(ncols, beg, end, (const double *)z, zf, maxbits);
  k_guard<<<1, 1, 0, st>>>(maxbits, R, E);
  k_dominance<<<(ncols + 127) / 128, 128, 0, st>>>(nx, ny, beg, end, reinterpret_cast<const float2 *>(zf), col,
                                                    dmask, mask_bits, L);
}

void fast_pair_records(cudaStream_t st, const int2 *pairs, int npairs, const DeviceTables &T, float4 *prec) {
  const int W = T.host.W;
  k_pair_records<<<(npairs + 127) / 128, 128, 0, st>>>(pairs, npairs, T.Hf, T.dH, W, (T.host.Dy + 1) * W, prec,
                                                       T.host.dom);
}

void launch_dh_tables(cudaStream_t st, int Dy, int W, const double *H, const int *Dx, float *dH) {
  const int n = (Dy + 1) * W;
  k_dh_tables<<<(n + 127) / 128, 128, 0, st>>>(Dy, W, H, Dx, dH);
}

int fast_union_cap(double mean_segments_per_column) {
  return mean_segments_per_column > 10.0 ? 64 : mean_segments_per_column > 6.0 ? 32 : 24;
}

namespace {
using BatchedFn = void (*)(const BatchVol *, const int2 *, int, int *, const FastArgs);

template <int KA, int FBY, bool SINGLE>
BatchedFn batched_fn_regs(int regs) {
  return regs == 64 ? &k_fast_batched<KA, FBY, SINGLE, 1024> : &k_fast_batched<KA, FBY, SINGLE, 768>;
}
template <int KA, int FBY>
BatchedFn batched_fn_single(bool single, int regs) {
  return single ? batched_fn_regs<KA, FBY, true>(regs) : batched_fn_regs<KA, FBY, false>(regs);
}
template <int KA>
BatchedFn batched_fn_fby(int fby, bool single, int regs) {
  switch (fby) {
    case 1:
      return batched_fn_single<KA, 1>(single, regs);
    case 2:
      return batched_fn_single<KA, 2>(single, regs);
    case 4:
      return batched_fn_single<KA, 4>(single, regs);
  }
  return nullptr;
}
BatchedFn batched_fn(int ka, int fby, bool single, int regs) {
  if (regs != 64 && regs != 80) return nullptr;
  switch (ka) {
    case 24:
      return batched_fn_fby<24>(fby, single, regs);
    case 32:
      return batched_fn_fby<32>(fby, single, regs);
    case 48:
      return batched_fn_fby<48>(fby, single, regs);
    case 64:
      return batched_fn_fby<64>(fby, single, regs);
  }
  return nullptr;
}
}  // namespace

int fast_batched_blocks_per_sm(int ka, int fby, bool single, int regs) {
  const BatchedFn f = batched_fn(ka, fby, single, regs);
  if (!f) return 0;
  const size_t smem = sizeof(float2) * ka * kFB * fby;
  if (smem > 227 * 1024 ||
      cudaFuncSetAttribute(reinterpret_cast<const void *>(f), cudaFuncAttributeMaxDynamicSharedMemorySize,
                           (int)smem) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, reinterpret_cast<const void *>(f), kFB * fby, smem) !=
      cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return per_sm;
}

int fast_batched_launch(int ka, int fby, int regs, int grid, cudaStream_t st, const BatchVol *vols,
                        const int2 *queue, int nq, int *next, const FastArgs *single) {
  const BatchedFn f = batched_fn(ka, fby, single != nullptr, regs);
  if (!f) return VO_EINVAL;
  const size_t smem = sizeof(float2) * ka * kFB * fby;
  FastArgs none;
  std::memset(&none, 0, sizeof none);
  f<<<grid, dim3(kFB, fby), smem, st>>>(vols, queue, nq, next, single ? *single : none);
  return VO_OK;
}

void fast_batched_mid_launch(cudaStream_t st, const BatchVol *vols, int nv, int grid) {
  k_fast_batched_mid<<<grid, kMidThreads, 0, st>>>(vols, nv);
}

size_t fast_batched_big_scratch_elems(int grid) { return (size_t)grid * kBigThreads * kBigCap; }

void fast_batched_big_launch(cudaStream_t st, const BatchVol *vols, int nv, int grid, double2 *scratch) {
  k_fast_batched_big<<<grid, kBigThreads, 0, st>>>(vols, nv, scratch);
}

}  // namespace vo
