// The separable "ours" scheme in its envelope form (VO_METHOD_ENVELOPE), FP64:
// the plain GPU method, two sweeping kernels.
//
// Pass 1 (k_env1, VoronoiMorpho2D along y, Voronoi2D.cpp:591-723): one warp
// per x-line sweeps the line's columns forward and backward. Its state is the
// half-space Voronoi envelope of the segments seen so far: for every z, the
// most recent row that covers it (disjoint labelled pieces, sorted by z), the
// lower envelope of the distance to the sweep line from one side. A step
// repaints the envelope with the new column's segments (each old piece keeps
// only its parts outside them), drops pieces whose row lies beyond floor(R)
// (the reference's expiry floor(y_s + R) + 1, Voronoi2D.cpp:619), and emits
// the envelope's pieces with their distance d to the column. The column's
// segments are staged into shared memory by a TMA bulk copy
// (cp.async.bulk + mbarrier), one column ahead; warp ballots and shuffles
// compact the surviving pieces and place them. The forward pieces of a column
// and its backward pieces with d >= 1 together give, for every z, the nearest
// covering row (their union with labels is the pass-1 intermediate of
// VoronoiVorPower.cpp:24-66: each piece dilates by r(d) = sqrt(R^2 - d^2)).
//
// Pass 2 (k_env2, SeparatePowerMorpho2D along x, SeparatePower2D.cpp:228-541):
// one block per row sweeps the row's columns forward, then backward. Its state
// is the set of live stadiums, the pass-1 pieces of the columns within reach
// (a piece of column x0 with label d reaches |x - x0| <= Dx[d], the
// reference's floor(x_s + r) + 1 expiry, SeparatePower2D.cpp:258-293), kept
// sorted by the start of their cores. A stadium's chord on the sweep line is
// [z1 - H[d][|x - x0|], z2 + H[d][|x - x0|]] with H the reference's FP64
// sqrt(r(d)^2 - dx^2) (getLine, SeparatePower2D.cpp:295-341). Their union is
// taken without sorting the chords: with the items in core order, a point g
// between two chords is uncovered exactly when the prefix maximum of the upper
// ends stops below the suffix minimum of the lower ends (every item whose core
// lies below an uncovered point precedes every item whose core lies above
// it), so two block scans give the union's intervals. The forward sweep stores
// its half-union per column; the backward sweep merges its half-union with it
// (the reference's unionMap, HalfDilationOperator.hpp:5-15) by a warp
// merge-path and the same scan. The result is the union of the same candidate
// intervals as the reference's, computed with its FP64 expressions, so it is
// bit-identical to the oracle. Pass 2 also drops stadiums that a newer piece
// holds for the rest of their lives (covers_for_life): exact, and the state
// shrinks about threefold.
//
// Capacities: pass 1's first launch keeps each line's state in shared memory,
// and lines whose state outgrows it re-run with it in global memory. Pass 2
// does the same for bands of few rows; bands of at least two rows per SM, or
// whose state is estimated beyond shared memory, sweep with global-memory
// state from the start (five rows per SM against one). A column whose union
// outgrows its output slot, or a state beyond the global capacity, sends the
// whole volume to the painter form of the method (VO_METHOD_SEPARABLE), which
// has no such limits.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <vector>

#include "vo_internal.cuh"

namespace vo {
namespace {

constexpr int kE1Warps = 4;          // lines (one warp each) per pass-1 block
constexpr int kE1Stage = 128;        // staged segments per column (more: read from global memory)
constexpr int kE1Cap = 448;          // shared-memory envelope capacity per line (pieces)
constexpr int kE1CapBig = 16384;     // global-memory capacity of the re-run
constexpr int kE2Threads = 256;      // threads of a pass-2 block (one row)
constexpr int kE2Stage = 768;        // staged pieces per column
constexpr int kE2CapSmall = 4864;    // shared-memory stadium capacity of the first launch (227 KB in all)
constexpr int kE2CapBig = 65536;     // global-memory stadium capacity of the re-run
constexpr int kE2Out = 64;           // union intervals per column (output slot)
constexpr int kWaitIters = 1 << 22;  // bounded mbarrier waits

// status words (flags[]): 0 fatal (a state beyond the global capacity, an
// output slot overflow or a timed-out wait), 1 lines / rows listed for the
// re-run, 2 timed-out waits
enum { kFlagFatal = 0, kFlagListed = 1, kFlagTimeout = 2 };

// ------------------------------------------------------------ TMA bulk copies

__device__ __forceinline__ uint32_t smem_u32(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t *bar) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(bar)) : "memory");
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// One thread: the buffer's previous contents were read through the generic
// proxy (ordered before this by the caller's __syncwarp / __syncthreads);
// order those reads before the asynchronous write, then arm the barrier with
// the byte count and start the copy. src and dst are 16-byte aligned and
// bytes is a positive multiple of 16.
__device__ __forceinline__ void bulk_load(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}

// Waits (bounded) for the phase with the given parity; false on time-out.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity) {
  for (int it = 0; it < kWaitIters; ++it) {
    uint32_t ok;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  return false;
}

// ------------------------------------------------------------ small searches

// Pieces and stadiums are ordered by (start, end): a zero-length piece [s, s]
// precedes [s, b]. Ordered by start alone, splitting [s, b] could move its
// later part past the point piece; with ends breaking ties the order survives
// every split, since a point piece only ever sits at another piece's end.
__device__ __forceinline__ bool lex_less(double2 a, double2 b) { return a.x < b.x || (a.x == b.x && a.y < b.y); }
// number of entries of v[0..n) (sorted by (start, end)) before / not after key
__device__ __forceinline__ int count_lex_less(const double2 *v, int n, double2 key) {
  int l = 0, r = n;
  while (l < r) {
    const int m = (l + r) >> 1;
    if (lex_less(v[m], key)) l = m + 1; else r = m;
  }
  return l;
}
__device__ __forceinline__ int count_lex_leq(const double2 *v, int n, double2 key) {
  int l = 0, r = n;
  while (l < r) {
    const int m = (l + r) >> 1;
    if (!lex_less(key, v[m])) l = m + 1; else r = m;
  }
  return l;
}
// number of entries of v[0..n) (sorted by .x) with .x < key / <= key
__device__ __forceinline__ int count_less(const double2 *v, int n, double key) {
  int l = 0, r = n;
  while (l < r) {
    const int m = (l + r) >> 1;
    if (v[m].x < key) l = m + 1; else r = m;
  }
  return l;
}
__device__ __forceinline__ int count_leq(const double2 *v, int n, double key) {
  int l = 0, r = n;
  while (l < r) {
    const int m = (l + r) >> 1;
    if (v[m].x <= key) l = m + 1; else r = m;
  }
  return l;
}
// first entry of v[0..n) (sorted, disjoint) whose end .y is >= key
__device__ __forceinline__ int first_ending_at_or_after(const double2 *v, int n, double key) {
  int l = 0, r = n;
  while (l < r) {
    const int m = (l + r) >> 1;
    if (v[m].y < key) l = m + 1; else r = m;
  }
  return l;
}

// ============================================================ pass 1

// Parts of piece [a, b] outside the sorted, disjoint segments N[j0..m): the
// count, and with OUT != nullptr the parts themselves. A part [a, s1] ends
// where a segment starts, a part [s2, b] starts where one ends (closed
// intervals: a shared endpoint is covered by the segment, whose own label is
// nearer); a point piece covered by a segment has no part.
template <bool WRITE>
__device__ __forceinline__ int piece_parts(double a, double b, const double2 *N, int m, int j, double2 *out) {
  int k = 0;
  while (a <= b) {
    if (j >= m || N[j].x > b) {
      if (WRITE) out[k] = make_double2(a, b);
      ++k;
      break;
    }
    if (N[j].x > a) {
      if (WRITE) out[k] = make_double2(a, N[j].x);
      ++k;
    }
    a = N[j].y;
    if (a >= b) break;
    ++j;
  }
  return k;
}

__device__ __forceinline__ int warp_excl_sum(int v, int lane, int &total) {
  int x = v;
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  total = __shfl_sync(0xffffffffu, x, 31);
  return x - v;
}

struct E1Args {
  int nx, ny, yb0, yb1, Dy;
  const int32_t *offs;
  const double2 *z;
  int32_t *nF, *nB;           // COUNT: forward / backward (d >= 1) pieces per column
  const int32_t *poff;        // FILL: piece offsets of the band's columns (index c - yb0 * nx)
  double2 *pz;                // FILL: piece cores
  uint8_t *pd;                // FILL: piece labels d
  int *flags;
  int *list;                  // lines whose envelope outgrew the shared capacity (first launch)
  double2 *gz;                // re-run: global envelope storage, 2 * kE1CapBig pieces per warp
  int *gl;                    // re-run: labels, 2 * kE1CapBig per warp
};

// One warp per x-line (first launch: x = global warp index; re-run: the
// listed lines). FILL writes the pieces of the band's rows [yb0, yb1); COUNT
// counts them for every row of [yb0, yb1).
template <bool FILL, bool BIG>
__global__ void __launch_bounds__(32 * kE1Warps) k_env1(E1Args A) {
  extern __shared__ __align__(16) unsigned char e1_smem[];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  // shared layout per warp: 2 staging buffers, 2 mbarriers, envelope A and T (z, label)
  const int cap = BIG ? kE1CapBig : kE1Cap;
  const size_t per_warp = 2 * kE1Stage * sizeof(double2) + 16 + (BIG ? 0 : 2 * (size_t)kE1Cap * (sizeof(double2) + 4));
  unsigned char *base = e1_smem + warp * per_warp;
  double2 *stage = reinterpret_cast<double2 *>(base);
  uint64_t *bar = reinterpret_cast<uint64_t *>(base + 2 * kE1Stage * sizeof(double2));
  double2 *Az, *Tz;
  int *Al, *Tl;
  const int gw = blockIdx.x * kE1Warps + warp;
  if (BIG) {
    Az = A.gz + (size_t)gw * 2 * kE1CapBig;
    Tz = Az + kE1CapBig;
    Al = A.gl + (size_t)gw * 2 * kE1CapBig;
    Tl = Al + kE1CapBig;
  } else {
    unsigned char *e = base + 2 * kE1Stage * sizeof(double2) + 16;
    Az = reinterpret_cast<double2 *>(e);
    Tz = Az + kE1Cap;
    Al = reinterpret_cast<int *>(Tz + kE1Cap);
    Tl = Al + kE1Cap;
  }
  int x;
  if (BIG) {
    if (gw >= A.flags[kFlagListed]) return;
    x = A.list[gw];
  } else {
    x = gw;
    if (x >= A.nx) return;
  }
  if (lane == 0) {
    mbar_init(&bar[0]);
    mbar_init(&bar[1]);
  }
  __syncwarp();
  uint32_t phase[2] = {0u, 0u};
  const int nx = A.nx;
  for (int dir = 0; dir < 2; ++dir) {
    // forward: rows from yb0 - Dy (to build the envelope) to yb1 - 1; backward: from yb1 - 1 + Dy down to yb0
    const int ys = dir == 0 ? max(0, A.yb0 - A.Dy) : min(A.ny - 1, A.yb1 - 1 + A.Dy);
    const int ye = dir == 0 ? A.yb1 : A.yb0 - 1;
    const int step = dir == 0 ? 1 : -1;
    int n = 0;  // envelope size (in Az, Al)
    // stage the first column
    auto issue = [&](int y, int b) -> bool {
      const int c = x + nx * y;
      const int kb = A.offs[c], m = A.offs[c + 1] - kb;
      if (m <= 0 || m > kE1Stage) return false;
      if (lane == 0) bulk_load(stage + b * kE1Stage, A.z + kb, (uint32_t)m * 16u, &bar[b]);
      return true;
    };
    bool staged_cur = issue(ys, 0);
    int buf = 0;
    for (int y = ys; y != ye; y += step) {
      const int c = x + nx * y;
      const int kb = A.offs[c], m = A.offs[c + 1] - kb;
      const double2 *N = A.z + kb;
      if (staged_cur) {
        if (!mbar_wait(&bar[buf], phase[buf])) {
          if (lane == 0) {
            atomicExch(&A.flags[kFlagTimeout], 1);
            atomicExch(&A.flags[kFlagFatal], 1);
          }
          // wait (bounded) for the other buffer's copy if one is in flight, then leave
          return;
        }
        phase[buf] ^= 1u;
        N = stage + buf * kE1Stage;
      }
      // prefetch the next column into the other buffer (its last reader finished at the previous step)
      const int yn = y + step;
      bool staged_next = false;
      if (yn != ye) staged_next = issue(yn, buf ^ 1);
      // 1. parts of the live pieces outside the new segments, compacted into T
      int r = 0;
      bool ovf = false;
      for (int i0 = 0; i0 < n; i0 += 32) {
        const int i = i0 + lane;
        int cnt = 0, j0 = 0;
        double pa = 0, pb = 0;
        if (i < n) {
          const int age = dir == 0 ? y - Al[i] : Al[i] - y;
          if (age <= A.Dy) {
            pa = Az[i].x;
            pb = Az[i].y;
            j0 = first_ending_at_or_after(N, m, pa);
            cnt = piece_parts<false>(pa, pb, N, m, j0, nullptr);
          }
        }
        int tot;
        const int off = warp_excl_sum(cnt, lane, tot);
        if (r + tot > cap) {
          ovf = true;
          break;
        }
        if (cnt) {
          piece_parts<true>(pa, pb, N, m, j0, Tz + r + off);
          for (int k = 0; k < cnt; ++k) Tl[r + off + k] = Al[i];
        }
        r += tot;
      }
      if (!ovf && r + m > cap) ovf = true;
      if (ovf) {
        if (lane == 0) {
          if (BIG) {
            atomicExch(&A.flags[kFlagFatal], 1);
          } else {
            A.list[atomicAdd(&A.flags[kFlagListed], 1)] = x;
          }
        }
        // leave the line: drain the copy in flight, if any, before the block's shared memory is released
        if (staged_next) mbar_wait(&bar[buf ^ 1], phase[buf ^ 1]);
        return;
      }
      __syncwarp();
      // 2. merge the parts (T) and the new segments (label y) into A in (start, end) order; ties:
      // parts first
      for (int k = lane; k < r; k += 32) {
        const int pos = k + count_lex_less(N, m, Tz[k]);
        Az[pos] = Tz[k];
        Al[pos] = Tl[k];
      }
      for (int j = lane; j < m; j += 32) {
        const double2 s = N[j];
        const int pos = j + count_lex_leq(Tz, r, s);
        Az[pos] = s;
        Al[pos] = y;
      }
      n = r + m;
      __syncwarp();
      // 3. emit the envelope's pieces for this column (backward: without the column's own segments)
      if (y >= A.yb0 && y < A.yb1) {
        if (!FILL) {
          if (lane == 0) {
            if (dir == 0) A.nF[c] = n;
            else A.nB[c] = n - m;
          }
        } else {
          const int bc = c - A.yb0 * nx;
          int outb = A.poff[bc] + (dir == 0 ? 0 : A.nF[c]);
          for (int i0 = 0; i0 < n; i0 += 32) {
            const int i = i0 + lane;
            const int lab = i < n ? Al[i] : y;
            const int d = dir == 0 ? y - lab : lab - y;
            const bool keep = i < n && (dir == 0 || d > 0);
            const unsigned bal = __ballot_sync(0xffffffffu, keep);
            if (keep) {
              const int o = outb + __popc(bal & ((1u << lane) - 1u));
              A.pz[o] = Az[i];
              A.pd[o] = (uint8_t)d;
            }
            outb += __popc(bal);
          }
        }
      }
      __syncwarp();
      staged_cur = staged_next;
      buf ^= 1;
    }
  }
}

// ============================================================ pass 2

struct E2Args {
  int nx, yb0, Dy, W;
  const double *H;       // [(Dy + 1) * W], NaN beyond Dx
  const int *Dx;         // [Dy + 1]
  const int32_t *poff;   // piece offsets of the band's columns (index c - yb0 * nx)
  const int32_t *nF;     // forward pieces per column (the first ones of its run)
  const double2 *pz;
  const uint8_t *pd;
  double2 *slots;        // kE2Out intervals per column (index c)
  int32_t *counts;       // intervals per column
  int *flags;
  int *list;             // rows (band-relative) whose stadium set outgrew the shared capacity
  double2 *gz;           // re-run: 2 * kE2CapBig per block
  uint32_t *gk;          // re-run: keys, 2 * kE2CapBig per block
  double prune_eps;      // margin of the dominance test (a bound on the H tables' rounding)
  int cap_small;         // stadium capacity of the first launch (<= kE2CapSmall)
  int *ghist;            // placement counts of columns with more than kE2Stage pieces (per block)
  int ghist_stride;      // ints per block of ghist (the band's most pieces per column + 2)
};

// Key of a stadium found dominated for the rest of its life: kept in place for
// the column where it was found (no chord, no gap), dropped at the next one.
constexpr uint32_t kDeadKey = 0xffffffffu;

// A stadium (key: x0 | d << 24) reaches column x: d is a pass-1 label (<= Dy)
// and the column lies within Dx[d] of x0 on the swept side.
__device__ __forceinline__ bool live(uint32_t k, int x, int dir, const E2Args &A) {
  if (k == kDeadKey) return false;
  const int d = (int)(k >> 24);
  const int age = dir == 0 ? x - (int)(k & 0xffffffu) : (int)(k & 0xffffffu) - x;
  return d <= A.Dy && age >= 0 && age <= __ldg(&A.Dx[d]);
}

// Whether the new piece p (label dp, entering at column x) holds the chord of
// the live stadium v (key k) at every column the stadium still reaches, so
// that the stadium can leave the state without changing any union.
// With h_d(t) = sqrt(c_d - t^2), c_d = fl(r(d)^2), the tables hold
// H[d][t] = fl(sqrt(fl(c_d - t^2))) within 1.6 * 2^-53 * R of h_d(t). For the
// stadium (column xi, label di) and the piece, g(x') = h_dp(|x' - x|) -
// h_di(|x' - xi|) has g' > 0 wherever g >= 0 (the piece is the younger one),
// so g >= M' at x keeps g >= M' at every later column the piece outlives. With
// M the larger of the core overhangs a_p - a_v, b_v - b_p (at least 0) and
// M' = M + 4 table errors, the tables' chords at every later column satisfy
// [a_v - H_v, b_v + H_v] inside [a_p - H_p, b_p + H_p] in exact arithmetic on
// the FP64 values, hence also after each endpoint's rounding. The test takes M
// rounded up, the table difference rounded down and prune_eps >= 2^-50 * R.
__device__ __forceinline__ bool covers_for_life(double2 p, int dp, double2 v, uint32_t k, int x, int dir,
                                                const E2Args &A) {
  const int di = (int)(k >> 24), xi = (int)(k & 0xffffffu);
  const int li = __ldg(&A.Dx[di]), lj = __ldg(&A.Dx[dp]);
  if (dir == 0 ? x + lj < xi + li : x - lj > xi - li) return false;  // the piece expires first
  const int age = dir == 0 ? x - xi : xi - x;
  const double hv = __ldg(&A.H[di * A.W + age]), hp = __ldg(&A.H[dp * A.W]);
  const double m = fmax(fmax(__dsub_ru(p.x, v.x), __dsub_ru(v.y, p.y)), 0.0);
  return __dsub_rd(hp, hv) >= __dadd_ru(m, A.prune_eps);
}

// Block scans over kE2Threads threads (8 warps): exclusive sum, and the
// exclusive prefix maximum with the exclusive suffix minimum.
struct BlockScratch {
  int isum[kE2Threads / 32];
  double dmax[kE2Threads / 32], dmin[kE2Threads / 32];
  int tot;
};

__device__ __forceinline__ int block_excl_sum(int v, BlockScratch &s, int &total) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  int x = v;
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) s.isum[w] = x;
  __syncthreads();
  int pre = 0;
  total = 0;
  for (int k = 0; k < kE2Threads / 32; ++k) {
    if (k < w) pre += s.isum[k];
    total += s.isum[k];
  }
  __syncthreads();
  return pre + x - v;
}

// Exclusive prefix maximum of vmax (thread order) and exclusive suffix
// minimum of vmin (reverse order), with one pair of barriers.
__device__ __forceinline__ void block_excl_max_min(double vmax, double vmin, BlockScratch &s, double &pmax,
                                                   double &smin) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  double x = vmax, y = vmin;
  for (int o = 1; o < 32; o <<= 1) {
    const double a = __shfl_up_sync(0xffffffffu, x, o);
    const double b = __shfl_down_sync(0xffffffffu, y, o);
    if (lane >= o) x = fmax(x, a);
    if (lane + o < 32) y = fmin(y, b);
  }
  if (lane == 31) s.dmax[w] = x;
  if (lane == 0) s.dmin[w] = y;
  double ex = __shfl_up_sync(0xffffffffu, x, 1), ey = __shfl_down_sync(0xffffffffu, y, 1);
  if (lane == 0) ex = -INFINITY;
  if (lane == 31) ey = INFINITY;
  __syncthreads();
  double pre = -INFINITY, suf = INFINITY;
  for (int k = 0; k < w; ++k) pre = fmax(pre, s.dmax[k]);
  for (int k = w + 1; k < kE2Threads / 32; ++k) suf = fmin(suf, s.dmin[k]);
  __syncthreads();
  pmax = fmax(pre, ex);
  smin = fmin(suf, ey);
}

// Union of the sorted (by lower end) interval lists U1[0..n1) and U2[0..n2)
// into out[0..), touching intervals merged; one warp; returns the count or -1
// beyond `cap`. M is scratch for n1 + n2 entries.
__device__ int warp_union_two(const double2 *U1, int n1, const double2 *U2, int n2, double2 *M, double2 *out,
                              int cap) {
  const int lane = threadIdx.x & 31;
  for (int i = lane; i < n1; i += 32) M[i + count_less(U2, n2, U1[i].x)] = U1[i];
  for (int j = lane; j < n2; j += 32) M[j + count_leq(U1, n1, U2[j].x)] = U2[j];
  __syncwarp();
  const int n = n1 + n2;
  // sorted by lower end: a gap follows item i exactly when max(hi[0..i]) < lo[i + 1]
  double carry = -INFINITY;
  int outn = 0;
  double start = n > 0 ? M[0].x : 0.0;
  for (int i0 = 0; i0 < n; i0 += 32) {
    const int i = i0 + lane;
    double h = i < n ? M[i].y : -INFINITY;
    for (int o = 1; o < 32; o <<= 1) {
      const double y = __shfl_up_sync(0xffffffffu, h, o);
      if (lane >= o) h = fmax(h, y);
    }
    h = fmax(h, carry);
    const double nlo = i + 1 < n ? M[i + 1].x : INFINITY;
    const bool gap = i < n && h < nlo;
    const unsigned bal = __ballot_sync(0xffffffffu, gap);
    // interval k ends at the k-th gap: [lo after the previous gap, h]
    const int k = outn + __popc(bal & ((1u << lane) - 1u));
    if (gap && k < cap) out[k].y = h;
    if (gap && k + 1 < cap && i + 1 < n) out[k + 1].x = nlo;
    outn += __popc(bal);
    carry = __shfl_sync(0xffffffffu, h, 31);
  }
  __syncwarp();
  if (lane == 0 && n > 0 && cap > 0) out[0].x = start;
  __syncwarp();
  return outn > cap ? -1 : outn;
}

template <bool BIG>
__global__ void __launch_bounds__(kE2Threads, BIG ? 5 : 1) k_env2(E2Args A, int nrows_or_list) {
  extern __shared__ __align__(16) unsigned char e2_smem[];
  __shared__ uint64_t bar[2];
  __shared__ BlockScratch bs;
  __shared__ double2 U[kE2Out], U1[kE2Out], Mrg[2 * kE2Out];
  __shared__ int s_hist[2 * kE2Stage + 2];
  const int tid = threadIdx.x;
  const int cap = BIG ? kE2CapBig : A.cap_small;
  // shared layout: staging (2 buffers), then (first launch) stadiums S and T
  double2 *stage = reinterpret_cast<double2 *>(e2_smem);
  double2 *Sz, *Tz;
  uint32_t *Sk, *Tk;
  if (BIG) {
    Sz = A.gz + (size_t)blockIdx.x * 2 * kE2CapBig;
    Tz = Sz + kE2CapBig;
    Sk = A.gk + (size_t)blockIdx.x * 2 * kE2CapBig;
    Tk = Sk + kE2CapBig;
  } else {
    unsigned char *p = e2_smem + 2 * kE2Stage * sizeof(double2);
    Sz = reinterpret_cast<double2 *>(p);
    Tz = Sz + A.cap_small;
    Sk = reinterpret_cast<uint32_t *>(Tz + A.cap_small);
    Tk = Sk + A.cap_small;
  }
  int yrel;
  if (BIG) {
    if ((int)blockIdx.x >= nrows_or_list) return;
    yrel = A.list[blockIdx.x];
  } else {
    yrel = blockIdx.x;
    if (yrel >= nrows_or_list) return;
  }
  const int nx = A.nx, y = A.yb0 + yrel;
  if (tid == 0) {
    mbar_init(&bar[0]);
    mbar_init(&bar[1]);
  }
  __syncthreads();
  uint32_t phase[2] = {0u, 0u};
  for (int dir = 0; dir < 2; ++dir) {
    const int xs = dir == 0 ? 0 : nx - 1, xe = dir == 0 ? nx : -1, step = dir == 0 ? 1 : -1;
    int n = 0;
    auto issue = [&](int x, int b) -> bool {
      const int bc = x + nx * yrel;
      const int kb = A.poff[bc], m = A.poff[bc + 1] - kb;
      if (m <= 0 || m > kE2Stage) return false;
      if (tid == 0) bulk_load(stage + b * kE2Stage, A.pz + kb, (uint32_t)m * 16u, &bar[b]);
      return true;
    };
    bool staged_cur = issue(xs, 0);
    int buf = 0;
    int keep = 0;  // this thread's items live at x (counted by the previous column's chord loop)
    for (int x = xs; x != xe; x += step) {
      const int c = x + nx * y, bc = x + nx * yrel;
      const int kb = A.poff[bc], m = A.poff[bc + 1] - kb, f = A.nF[c], b = m - f;
      const double2 *P = A.pz + kb;
      if (staged_cur) {
        if (!mbar_wait(&bar[buf], phase[buf])) {
          if (tid == 0) {
            atomicExch(&A.flags[kFlagTimeout], 1);
            atomicExch(&A.flags[kFlagFatal], 1);
          }
          return;
        }
        phase[buf] ^= 1u;
        P = stage + buf * kE2Stage;
      }
      const int xn = x + step;
      bool staged_next = false;
      if (xn != xe) staged_next = issue(xn, buf ^ 1);
      const double2 *F = P, *B = P + f;  // the column's forward and backward pieces, each sorted
      const uint8_t *Fd = A.pd + kb, *Bd = A.pd + kb + f;
      // placement counts: bin c of F (0 <= c <= f) and bin f + 1 + c of B
      const int nbins = f + b + 2;
      int *hist = m <= kE2Stage ? s_hist : (A.ghist ? A.ghist + (size_t)blockIdx.x * A.ghist_stride : nullptr);
      if (hist == nullptr || (m > kE2Stage && nbins > A.ghist_stride)) {
        if (tid == 0) atomicExch(&A.flags[kFlagFatal], 1);
        if (staged_next && tid == 0) mbar_wait(&bar[buf ^ 1], phase[buf ^ 1]);
        return;
      }
      for (int h = tid; h < nbins; h += kE2Threads) hist[h] = 0;
      // ---- 1. survivors (within reach at x): each thread's first rank
      const int L = (n + kE2Threads - 1) / kE2Threads;
      const int r0 = min(n, tid * L), r1 = min(n, r0 + L);
      int nkeep;
      const int rk0 = block_excl_sum(keep, bs, nkeep);
      const int nn = nkeep + m;
      if (nn > cap) {
        if (tid == 0) {
          if (BIG) atomicExch(&A.flags[kFlagFatal], 1);
          else A.list[atomicAdd(&A.flags[kFlagListed], 1)] = yrel;
        }
        if (staged_next && tid == 0) mbar_wait(&bar[buf ^ 1], phase[buf ^ 1]);
        return;
      }
      __syncthreads();
      // ---- 2. merge survivors, forward pieces and backward pieces into T in (start, end) order
      // (ties: survivors, F, B)
      // A survivor that one of the new pieces beside it (in core order) holds
      // for the rest of its life is marked dead (covers_for_life). Its counts
      // cF, cB of smaller pieces also place the pieces: F[j] follows exactly
      // the survivors v with cF(v) <= j (v <= F[j], survivors first on ties),
      // so bin cF of a count over the survivors, summed up to j, is the number
      // of survivors before F[j]; likewise for B. No search over the state.
      {
        // the thread's items are in core order, so their counts of smaller pieces only grow: one
        // binary search for the first survivor, then steps forward
        int rk = rk0, cF = -1, cB = -1;
        for (int i = r0; i < r1; ++i) {
          const uint32_t k = Sk[i];
          if (live(k, x, dir, A)) {
            const double2 v = Sz[i];
            if (cF < 0) {
              cF = count_lex_less(F, f, v);
              cB = count_lex_less(B, b, v);
            } else {
              while (cF < f && lex_less(F[cF], v)) ++cF;
              while (cB < b && lex_less(B[cB], v)) ++cB;
            }
            const int pos = rk++ + cF + cB;
            // tested on every other column: a stadium the pieces of one column hold is mostly held by
            // the next column's as well (2048^2 spheres + cylinders, r = 32: 3.86 s testing every
            // column, 3.34 s every other one, 3.41 s every fourth; two candidates instead of four: 3.55 s)
            bool dom = false;
            if ((x & 1) == 0) {
              dom = cF > 0 && covers_for_life(F[cF - 1], Fd[cF - 1], v, k, x, dir, A);
              dom = dom || (cF < f && covers_for_life(F[cF], Fd[cF], v, k, x, dir, A));
              dom = dom || (cB > 0 && covers_for_life(B[cB - 1], Bd[cB - 1], v, k, x, dir, A));
              dom = dom || (cB < b && covers_for_life(B[cB], Bd[cB], v, k, x, dir, A));
            }
            Tz[pos] = v;
            Tk[pos] = dom ? kDeadKey : k;
            atomicAdd(&hist[cF], 1);
            atomicAdd(&hist[f + 1 + cB], 1);
          }
        }
      }
      __syncthreads();
      {  // inclusive prefix sums of the bins (F's, then B's on top of all survivors)
        const int K = (nbins + kE2Threads - 1) / kE2Threads;
        const int h0 = min(nbins, tid * K), h1 = min(nbins, h0 + K);
        int part = 0;
        for (int h = h0; h < h1; ++h) part += hist[h];
        int tot;
        int run = block_excl_sum(part, bs, tot);
        for (int h = h0; h < h1; ++h) {
          run += hist[h];
          hist[h] = run;
        }
      }
      __syncthreads();
      for (int j = tid; j < m; j += kE2Threads) {
        const bool isF = j < f;
        const int jj = isF ? j : j - f;
        const double2 p = isF ? F[jj] : B[jj];
        const int d = isF ? Fd[jj] : Bd[jj];
        const int before = isF ? hist[jj] : hist[f + 1 + jj] - hist[f];  // survivors before the piece
        const int pos = jj + before + (isF ? count_lex_less(B, b, p) : count_lex_leq(F, f, p));
        Tz[pos] = p;
        Tk[pos] = (uint32_t)x | ((uint32_t)d << 24);
      }
      __syncthreads();
      {
        double2 *t = Sz;
        Sz = Tz;
        Tz = t;
        uint32_t *u = Sk;
        Sk = Tk;
        Tk = u;
      }
      n = nn;
      // ---- 3. chords at x and their union (sort-free: prefix max of hi vs suffix min of lo); the
      // buffer T is free after the swap and holds (lo, hi), then (min lo over the later items, hi)
      // (the same split of the items over the threads as step 1 of the next column, which takes
      // its survivor counts from here)
      const int L2 = (n + kE2Threads - 1) / kE2Threads;
      const int q0 = min(n, tid * L2), q1 = min(n, q0 + L2);
      double run_max = -INFINITY, run_min = INFINITY;
      keep = 0;
      for (int i = q0; i < q1; ++i) {
        const uint32_t k = Sk[i];
        keep += live(k, x + step, dir, A) ? 1 : 0;
        if (k == kDeadKey) {  // held by a new piece's chord: no chord of its own
          Tz[i] = make_double2(INFINITY, -INFINITY);
          continue;
        }
        // every other item here is live (d <= Dy, 0 <= age <= Dx[d] < W); the clamps only keep the
        // table reads in bounds whatever the key holds
        const int d = min((int)(k >> 24), A.Dy);
        const int age = max(0, min(A.W - 1, dir == 0 ? x - (int)(k & 0xffffffu) : (int)(k & 0xffffffu) - x));
        const double h = __ldg(&A.H[d * A.W + age]);
        const double2 zz = Sz[i];
        const double lo = __dsub_rn(zz.x, h), hi = __dadd_rn(zz.y, h);
        Tz[i] = make_double2(lo, hi);
        run_max = fmax(run_max, hi);
        run_min = fmin(run_min, lo);
      }
      double pmax0, smin_after;
      block_excl_max_min(run_max, run_min, bs, pmax0, smin_after);
      double start0 = INFINITY;
      {
        double sm = smin_after;
        for (int i = q1 - 1; i >= q0; --i) {
          const double lo = Tz[i].x;
          Tz[i].x = sm;  // min lo over items i + 1 .. n - 1
          sm = fmin(sm, lo);
        }
        if (q0 == 0 && q1 > 0) start0 = sm;  // min lo over all items
      }
      // a gap follows item i when the items up to i end below every later start; dead items (no chord)
      // and the live items after which only dead ones follow (no later start) have none
      int gaps = 0;
      {
        double pm = pmax0;
        for (int i = q0; i < q1; ++i) {
          const double2 t = Tz[i];
          pm = fmax(pm, t.y);
          if (i + 1 < n && t.y != -INFINITY && t.x != INFINITY && pm < t.x) ++gaps;
        }
      }
      int G;
      const int gbase = block_excl_sum(gaps, bs, G);
      const int nu = n > 0 ? G + 1 : 0;
      if (nu > kE2Out) {
        if (tid == 0) atomicExch(&A.flags[kFlagFatal], 1);
        if (staged_next && tid == 0) mbar_wait(&bar[buf ^ 1], phase[buf ^ 1]);
        return;
      }
      {
        double pm = pmax0;
        int g = gbase;
        if (q0 == 0 && q1 > 0) U[0].x = start0;
        for (int i = q0; i < q1; ++i) {
          const double2 t = Tz[i];
          pm = fmax(pm, t.y);
          if (i + 1 < n && t.y != -INFINITY && t.x != INFINITY && pm < t.x) {
            U[g].y = pm;
            U[g + 1].x = t.x;
            ++g;
          }
          if (i == n - 1) U[G].y = pm;
        }
      }
      __syncthreads();
      // ---- 4. output: the forward half-union to the column's slot; backward: merged with it
      double2 *slot = A.slots + (size_t)c * kE2Out;
      if (dir == 0) {
        for (int k = tid; k < nu; k += kE2Threads) slot[k] = U[k];
        if (tid == 0) A.counts[c] = nu;
      } else if (tid < 32) {
        const int n1 = A.counts[c];
        for (int k = tid; k < n1; k += 32) U1[k] = slot[k];
        __syncwarp();
        const int nf = warp_union_two(U1, n1, U, nu, Mrg, slot, kE2Out);
        if (tid == 0) {
          if (nf < 0) atomicExch(&A.flags[kFlagFatal], 1);
          else A.counts[c] = nf;
        }
      }
      __syncthreads();
      staged_cur = staged_next;
      buf ^= 1;
    }
  }
}

// Compaction of the slots into the CSR output: one warp per column.
__global__ void k_env_compact(int ncols, const double2 *__restrict__ slots, const int32_t *__restrict__ ooffs,
                              double2 *__restrict__ oz) {
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (w >= ncols) return;
  const int n = ooffs[w + 1] - ooffs[w];
  for (int k = lane; k < n; k += 32) oz[ooffs[w] + k] = slots[(size_t)w * kE2Out + k];
}

// Pieces per row of the band (for the band split): one thread per row.
__global__ void k_row_pieces(int nx, int ny, const int32_t *nF, const int32_t *nB, long long *rows) {
  const int y = blockIdx.x * blockDim.x + threadIdx.x;
  if (y >= ny) return;
  long long s = 0;
  for (int x = 0; x < nx; ++x) s += nF[x + nx * y] + nB[x + nx * y];
  rows[y] = s;
}

// Lists every row of a band for the global-memory sweep.
__global__ void k_list_rows(int n, int *list, int *flags) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) list[i] = i;
  if (i == 0) flags[kFlagListed] = n;
}

// Pieces per column of a band, and their maximum (atomicMax into *maxc).
__global__ void k_band_counts(int n, const int32_t *nF, const int32_t *nB, int32_t *cnt, int *maxc) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const int v = i < n ? nF[i] + nB[i] : 0;
  if (i < n) cnt[i] = v;
  const int w = __reduce_max_sync(0xffffffffu, v);
  if ((threadIdx.x & 31) == 0) atomicMax(maxc, w);
}

size_t e1_smem_bytes(bool big) {
  const size_t per_warp = 2 * kE1Stage * sizeof(double2) + 16 + (big ? 0 : 2 * (size_t)kE1Cap * (sizeof(double2) + 4));
  return kE1Warps * per_warp;
}

size_t e2_smem_bytes(bool big) {
  const size_t stage = 2 * (size_t)kE2Stage * sizeof(double2);
  if (big) return stage;
  const size_t cap = (size_t)kE2CapSmall;
  return stage + 2 * cap * (sizeof(double2) + sizeof(uint32_t));
}

}  // namespace

// Host driver. Returns VO_OK, an error, or 1 when the volume must take the
// painter form (a capacity beyond the envelope kernels' limits).
int dilate_envelope(vo_ctx *ctx, double R, const vo_volume *in, vo_volume **out, vo_timings *tm) {
  const vo_grid g = in->grid;
  const int nx = g.nx, ny = g.ny, ncols = nx * ny;
  if (nx >= (1 << 24)) return 1;
  const DeviceTables *T = nullptr;
  int rc = get_tables(ctx, R, std::max(nx, ny), &T);
  if (rc) return rc;
  const int Dy = T->host.Dy, W = T->host.W;
  // first-tier stadium capacity of pass 2; VO_ENVELOPE_STATE_CAP lowers it (tests use it to send
  // rows to the global-memory re-run)
  int cap2 = kE2CapSmall;
  if (const char *sc = std::getenv("VO_ENVELOPE_STATE_CAP")) {
    const int v = std::atoi(sc);
    if (v > 0) cap2 = std::min(cap2, v);
  }
  cudaFuncSetAttribute(k_env1<false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)e1_smem_bytes(false));
  cudaFuncSetAttribute(k_env1<true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)e1_smem_bytes(false));
  cudaFuncSetAttribute(k_env2<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)e2_smem_bytes(false));
  int32_t *nF = nullptr, *nB = nullptr, *counts = nullptr, *bcnt = nullptr, *list = nullptr;
  long long *rowp = nullptr;
  double2 *slots = nullptr;
  rc = dalloc(ctx, &nF, (size_t)ncols);
  if (!rc) rc = dalloc(ctx, &nB, (size_t)ncols);
  if (!rc) rc = dalloc(ctx, &counts, (size_t)ncols + 1);
  if (!rc) rc = dalloc(ctx, &bcnt, (size_t)ncols + 1);
  if (!rc) rc = dalloc(ctx, &list, (size_t)std::max(nx, ny));
  if (!rc) rc = dalloc(ctx, &rowp, (size_t)ny);
  if (!rc) rc = dalloc(ctx, &slots, (size_t)ncols * kE2Out);
  double2 *gz1 = nullptr, *gz2 = nullptr;
  int gz1_lines = 0;
  int *gl1 = nullptr, *ghist = nullptr;
  uint32_t *gk2 = nullptr;
  int32_t *poff = nullptr;
  double2 *pz = nullptr;
  uint8_t *pd = nullptr;
  vo_volume *res = nullptr;
  int fallback = 0;
  int hflags[4] = {0, 0, 0, 0};  // status words, then (slot 3) the band's most pieces per column
  auto flags_now = [&]() -> int {
    VO_CK(ctx, cudaMemcpyAsync(hflags, ctx->d_flags, sizeof(hflags), cudaMemcpyDeviceToHost, ctx->stream));
    VO_CK(ctx, cudaStreamSynchronize(ctx->stream));
    return VO_OK;
  };
  E1Args a1{nx, ny, 0, ny, Dy, in->offs, in->z, nF, nB, nullptr, nullptr, nullptr, ctx->d_flags, list, nullptr,
            nullptr};
  const int e1_blocks = (nx + kE1Warps - 1) / kE1Warps;
  float ms1 = 0, ms2 = 0;
  // ---- pass 1, count (every row)
  if (!rc) {
    cudaMemsetAsync(ctx->d_flags, 0, 3 * sizeof(int), ctx->stream);
    cudaEventRecord(ctx->ev[0], ctx->stream);
    k_env1<false, false><<<e1_blocks, 32 * kE1Warps, e1_smem_bytes(false), ctx->stream>>>(a1);
    ctx->launches += 1;
    rc = flags_now();
  }
  auto run_big1 = [&](E1Args a) -> int {
    // lines listed by the first launch run again with their envelope in global memory
    const int nl = hflags[kFlagListed];
    if (nl == 0 || hflags[kFlagFatal]) return VO_OK;
    if (!a.pz) ctx->ovf_cols += nl;  // counted once, in the count pass
    if (nl > gz1_lines) {
      dfree(ctx, gz1);
      dfree(ctx, gl1);
      gz1 = nullptr;
      gl1 = nullptr;
      int r2 = dalloc(ctx, &gz1, (size_t)2 * kE1CapBig * nl);
      if (!r2) r2 = dalloc(ctx, &gl1, (size_t)2 * kE1CapBig * nl);
      if (r2) return r2;
      gz1_lines = nl;
    }
    a.gz = gz1;
    a.gl = gl1;
    const int blocks = (nl + kE1Warps - 1) / kE1Warps;
    if (a.pz) k_env1<true, true><<<blocks, 32 * kE1Warps, e1_smem_bytes(true), ctx->stream>>>(a);
    else k_env1<false, true><<<blocks, 32 * kE1Warps, e1_smem_bytes(true), ctx->stream>>>(a);
    ctx->launches += 1;
    return flags_now();
  };
  if (!rc) rc = run_big1(a1);
  if (!rc) {
    cudaEventRecord(ctx->ev[1], ctx->stream);
    if (hflags[kFlagFatal]) fallback = 1;
  }
  // ---- bands of rows whose pieces fit the piece budget
  std::vector<int> bands{0};
  if (!rc && !fallback) {
    k_row_pieces<<<(ny + 127) / 128, 128, 0, ctx->stream>>>(nx, ny, nF, nB, rowp);
    ctx->launches += 1;
    std::vector<long long> h(ny);
    VO_CK(ctx, cudaMemcpyAsync(h.data(), rowp, sizeof(long long) * ny, cudaMemcpyDeviceToHost, ctx->stream));
    VO_CK(ctx, cudaStreamSynchronize(ctx->stream));
    size_t freeb = 0, totb = 0;
    cudaMemGetInfo(&freeb, &totb);
    // pieces per band: a quarter of the free device memory (17 bytes per piece), at most int32
    // offsets; VO_ENVELOPE_BAND_PIECES lowers it for callers that share the device's memory
    long long budget = std::min<long long>(2000000000LL, (long long)(freeb / 4 / 17));
    if (const char *cap = std::getenv("VO_ENVELOPE_BAND_PIECES")) {
      const long long v = std::atoll(cap);
      if (v > 0) budget = std::min(budget, v);
    }
    long long acc = 0;
    for (int y = 0; y < ny; ++y) {
      if (h[y] > budget) {
        fallback = 1;
        break;
      }
      if (acc + h[y] > budget) {
        bands.push_back(y);
        acc = 0;
      }
      acc += h[y];
    }
    bands.push_back(ny);
  }
  // ---- per band: pass-1 fill, pass 2
  int64_t mid = 0;
  for (size_t bi = 0; !rc && !fallback && bi + 1 < bands.size(); ++bi) {
    const int yb0 = bands[bi], yb1 = bands[bi + 1];
    const int bcols = nx * (yb1 - yb0);
    long long ptotal = 0;
    rc = dalloc(ctx, &poff, (size_t)bcols + 1);
    if (!rc) {
      cudaMemsetAsync(ctx->d_flags + 3, 0, sizeof(int), ctx->stream);
      k_band_counts<<<(bcols + 255) / 256, 256, 0, ctx->stream>>>(bcols, nF + (size_t)yb0 * nx,
                                                                  nB + (size_t)yb0 * nx, bcnt, ctx->d_flags + 3);
      ctx->launches += 1;
      rc = scan_counts(ctx, bcnt, poff, bcols, &ptotal);
    }
    if (!rc) rc = flags_now();
    // placement counts of columns beyond the staging buffer live in global memory, one range per block
    const int max_pieces = hflags[3];
    const int hstride = max_pieces > kE2Stage ? max_pieces + 2 : 0;
    if (!rc && hstride > 0) rc = dalloc(ctx, &ghist, (size_t)hstride * (yb1 - yb0));
    if (!rc) rc = dalloc(ctx, &pz, (size_t)ptotal);
    if (!rc) rc = dalloc(ctx, &pd, (size_t)ptotal);
    if (rc) break;
    mid += ptotal;
    E1Args f1 = a1;
    f1.yb0 = yb0;
    f1.yb1 = yb1;
    f1.poff = poff;
    f1.pz = pz;
    f1.pd = pd;
    cudaEvent_t e0, e1, e2;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    cudaEventCreate(&e2);
    cudaMemsetAsync(ctx->d_flags, 0, 3 * sizeof(int), ctx->stream);
    cudaEventRecord(e0, ctx->stream);
    k_env1<true, false><<<e1_blocks, 32 * kE1Warps, e1_smem_bytes(false), ctx->stream>>>(f1);
    ctx->launches += 1;
    rc = flags_now();
    if (!rc) rc = run_big1(f1);
    if (!rc && hflags[kFlagFatal]) fallback = 1;
    cudaEventRecord(e1, ctx->stream);
    if (!rc && !fallback) {
      E2Args a2{nx,    yb0,    Dy,      W,  T->H, T->Dx, poff, nF, pz, pd, slots, counts, ctx->d_flags, list,
                nullptr, nullptr, std::ldexp(std::max(R, 1.0), -46), cap2, ghist, hstride};
      cudaMemsetAsync(ctx->d_flags, 0, 3 * sizeof(int), ctx->stream);
      // The global-memory sweep runs five rows per SM against one in shared memory (227 KB per
      // block); with at least two rows per SM to run it is the faster one (1024^2 spheres, r = 16:
      // 389 against 467 ms), and so it is for rows whose live-stadium state would mostly outgrow
      // shared memory, estimated as a third of the pieces of the floor(R) + 1 columns within reach
      // (what the pruning leaves on the 2048^2 and 1024^2 sphere workloads at r = 32).
      const double mean_pieces = bcols > 0 ? (double)ptotal / bcols : 0.0;
      int sms = 0;
      cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
      if (yb1 - yb0 >= 2 * std::max(sms, 1) || mean_pieces * (Dy + 1) / 3.0 > 0.6 * cap2) {
        k_list_rows<<<(yb1 - yb0 + 255) / 256, 256, 0, ctx->stream>>>(yb1 - yb0, list, ctx->d_flags);
      } else {
        k_env2<false><<<yb1 - yb0, kE2Threads, e2_smem_bytes(false), ctx->stream>>>(a2, yb1 - yb0);
      }
      ctx->launches += 1;
      rc = flags_now();
      const int nl = hflags[kFlagListed];
      ctx->ovf_cols += nl;
      if (!rc && !hflags[kFlagFatal] && nl > 0) {
        // the listed rows sweep with global-memory state (2.6 MB per row), in chunks of rows whose
        // state fits a quarter of the free device memory
        size_t freeb = 0, totb = 0;
        cudaMemGetInfo(&freeb, &totb);
        const size_t per_row = (size_t)2 * kE2CapBig * (sizeof(double2) + sizeof(uint32_t));
        int chunk = (int)std::max<size_t>(1, std::min<size_t>((size_t)nl, freeb / 4 / per_row));
        if (const char *rc_env = std::getenv("VO_ENVELOPE_ROW_CHUNK")) {  // tests: smaller chunks
          const int v = std::atoi(rc_env);
          if (v > 0) chunk = std::min(chunk, v);
        }
        rc = dalloc(ctx, &gz2, (size_t)2 * kE2CapBig * chunk);
        if (!rc) rc = dalloc(ctx, &gk2, (size_t)2 * kE2CapBig * chunk);
        for (int r0 = 0; !rc && r0 < nl && !hflags[kFlagFatal]; r0 += chunk) {
          const int cnt = std::min(chunk, nl - r0);
          E2Args ab = a2;
          ab.gz = gz2;
          ab.gk = gk2;
          ab.list = list + r0;
          k_env2<true><<<cnt, kE2Threads, e2_smem_bytes(true), ctx->stream>>>(ab, cnt);
          ctx->launches += 1;
          rc = flags_now();
        }
        dfree(ctx, gz2);
        dfree(ctx, gk2);
        gz2 = nullptr;
        gk2 = nullptr;
      }
      if (!rc && hflags[kFlagFatal]) fallback = 1;
    }
    cudaEventRecord(e2, ctx->stream);
    cudaEventSynchronize(e2);
    float t1 = 0, t2 = 0;
    cudaEventElapsedTime(&t1, e0, e1);
    cudaEventElapsedTime(&t2, e1, e2);
    ms1 += t1;
    ms2 += t2;
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaEventDestroy(e2);
    dfree(ctx, poff);
    dfree(ctx, pz);
    dfree(ctx, pd);
    dfree(ctx, ghist);
    poff = nullptr;
    pz = nullptr;
    pd = nullptr;
    ghist = nullptr;
  }
  // ---- output
  long long total = 0;
  if (!rc && !fallback) {
    rc = volume_alloc(ctx, g, 0, &res);
    if (!rc) rc = scan_counts(ctx, counts, res->offs, ncols, &total);
    if (!rc) {
      res->nseg = total;
      rc = dalloc(ctx, &res->z, (size_t)total);
    }
    if (!rc) {
      k_env_compact<<<(ncols + 7) / 8, 256, 0, ctx->stream>>>(ncols, slots, res->offs, res->z);
      ctx->launches += 1;
      VO_CK(ctx, cudaGetLastError());
    }
  }
  if (!rc && tm) {
    float c1 = 0;
    cudaEventSynchronize(ctx->ev[1]);
    cudaEventElapsedTime(&c1, ctx->ev[0], ctx->ev[1]);
    tm->pass1_ms += c1 + ms1;
    tm->pass2_ms += ms2;
    tm->kernel_ms[0] += c1;
    tm->kernel_ms[1] += ms1;
    tm->kernel_ms[2] += ms2;
    tm->mid_pieces += mid;
  }
  dfree(ctx, nF);
  dfree(ctx, nB);
  dfree(ctx, counts);
  dfree(ctx, bcnt);
  dfree(ctx, list);
  dfree(ctx, rowp);
  dfree(ctx, slots);
  dfree(ctx, gz1);
  dfree(ctx, gl1);
  dfree(ctx, poff);
  dfree(ctx, pz);
  dfree(ctx, pd);
  dfree(ctx, ghist);
  if (rc || fallback) {
    if (res) vo_volume_free(ctx, res);
    if (!rc && hflags[kFlagTimeout]) return set_error(ctx, VO_ETIMEOUT, "envelope: a staged copy did not arrive");
    return rc ? rc : 1;
  }
  *out = res;
  return VO_OK;
}

}  // namespace vo
