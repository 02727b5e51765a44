// Dexel morphology kernels for sm_103a and their host drivers.
//
// Separable dilation ("ours", src/vor3d/VoronoiVorPower.cpp:24-96) runs as
// two passes, each count -> scan -> fill, one thread per output column:
//
//   pass 1 (replaces the y-sweeps of Voronoi2D.cpp + the radius-aware
//   appendSegment/unionSegs of MorphologyOperators.cpp:37-95, .hpp:74-127):
//   the column's pieces, labelled with the lattice distance d of the nearest
//   column (x, y+-d) covering them. Painter over d = 0..Dy: the union of the
//   two level-d columns is clipped to the gaps of the pieces found so far.
//   The working list keeps pieces with touching runs merged, which preserves
//   the gap structure exactly (also for inverted pairs, see below).
//
//   pass 2 (replaces SeparatePower2D.cpp's x-sweeps and getLine, :295-341):
//   the output column is the union of [a - h, b + h], h = H[d][|dx|] =
//   sqrt(r(d)^2 - dx^2), over the pieces of columns (x+dx, y) alive at |dx|
//   (floor(x_s + r) + 1 > i, SeparatePower2D.cpp:258-273), merged as closed
//   intervals (touching merges, MorphologyOperators.cpp:15-34).
//
// Inverted pairs [a, b], a > b, appear when erosion complements a column
// whose values left [zmin, zmax] (negate_ray, MorphologyOperators.cpp:230-259);
// pass 2 then contributes their two endpoint circles, as the reference's
// power-diagram points do (SeparatePower2D.cpp:215-226).
//
// Every table value is computed on the host with the reference's FP64
// expressions; the device only adds/subtracts (round-to-nearest intrinsics,
// never contracted) and compares, so results are bit-identical to the oracle
// restatement and to the reference on the same inputs.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "vo_internal.cuh"

namespace vo {
namespace {

constexpr int kBX = 32, kBY = 4;  // 2D thread block: x-major, 128 threads
constexpr int kBigThreads = 32;   // threads per block of the overflow re-run kernels

__device__ __forceinline__ double dsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ double dadd(double a, double b) { return __dadd_rn(a, b); }

// ---------------------------------------------------------------- pass 1

// Streams the union of two sorted segment lists (closed intervals, touching
// merges) in increasing order. Ties take list B first (unionSegs order,
// MorphologyOperators.cpp:117-158): A = column (x, y-d), B = column (x, y+d).
struct MergeStream {
  const double2 *z;
  int ia, ea, ib, eb;
  __device__ bool next(double &ma, double &mb) {
    if (ia >= ea && ib >= eb) return false;
    double2 s;
    if (ib < eb && (ia >= ea || z[ib].x <= z[ia].x))
      s = z[ib++];
    else
      s = z[ia++];
    ma = s.x;
    mb = s.y;
    for (;;) {
      double nx;
      bool fromb;
      if (ib < eb && (ia >= ea || z[ib].x <= z[ia].x)) {
        nx = z[ib].x;
        fromb = true;
      } else if (ia < ea) {
        nx = z[ia].x;
        fromb = false;
      } else {
        break;
      }
      if (!(nx <= mb)) break;
      double ny = fromb ? z[ib++].y : z[ia++].y;
      if (ny > mb) mb = ny;
    }
    return true;
  }
};

__device__ __forceinline__ bool list_append(double2 *Q, int &nQ, int cap, double lo, double hi) {
  if (nQ > 0 && Q[nQ - 1].y == lo) {
    Q[nQ - 1].y = hi;
    return true;
  }
  if (nQ >= cap) return false;
  Q[nQ++] = make_double2(lo, hi);
  return true;
}

// Pieces of column (x, y). Returns the piece count, or -1 when the working
// list exceeds `cap`. In FILL mode pieces go to outz/outd in painter order
// (by label, then z).
template <bool FILL>
__device__ int pass1_column(int x, int y, int nx, int ny, const int32_t *__restrict__ offs,
                            const double2 *__restrict__ z, int Dy, double2 *P, double2 *Q,
                            int cap, double2 *outz, uint8_t *outd) {
  int nP = 0, np = 0;
  for (int d = 0; d <= Dy; ++d) {
    MergeStream ms;
    ms.z = z;
    ms.ia = ms.ea = ms.ib = ms.eb = 0;
    const int ya = y - d, yb = y + d;
    if (ya >= 0) {
      const int c = x + nx * ya;
      ms.ia = offs[c];
      ms.ea = offs[c + 1];
    }
    if (d > 0 && yb < ny) {
      const int c = x + nx * yb;
      ms.ib = offs[c];
      ms.eb = offs[c + 1];
    }
    if (ms.ia == ms.ea && ms.ib == ms.eb) continue;
    double ma = 0, mb = 0;
    bool mv = ms.next(ma, mb);
    int nQ = 0;
    for (int k = 0; k <= nP; ++k) {
      if (k > 0 && !list_append(Q, nQ, cap, P[k - 1].x, P[k - 1].y)) return -1;
      const double g1 = k == 0 ? -INFINITY : P[k - 1].y;
      const double g2 = k == nP ? INFINITY : P[k].x;
      if (!(g1 < g2)) continue;
      while (mv && mb <= g1) mv = ms.next(ma, mb);
      while (mv && ma < g2) {
        const double lo = ma > g1 ? ma : g1;
        const double hi = mb < g2 ? mb : g2;
        if (FILL) {
          outz[np] = make_double2(lo, hi);
          outd[np] = (uint8_t)d;
        }
        ++np;
        if (!list_append(Q, nQ, cap, lo, hi)) return -1;
        if (mb >= g2) break;
        mv = ms.next(ma, mb);
      }
    }
    double2 *t = P;
    P = Q;
    Q = t;
    nP = nQ;
  }
  return np;
}

// ---------------------------------------------------------------- union

// Inserts [lo, hi] into a sorted list of disjoint closed intervals, merging
// overlapping or touching ones. Same procedure as the oracle's union_insert.
__device__ __forceinline__ bool union_insert(double2 *A, int &n, int cap, double lo, double hi) {
  int l = 0, r = n;
  while (l < r) {
    const int m = (l + r) >> 1;
    if (A[m].y >= lo)
      r = m;
    else
      l = m + 1;
  }
  const int i = l;
  if (i == n || A[i].x > hi) {
    if (n >= cap) return false;
    for (int k = n; k > i; --k) A[k] = A[k - 1];
    A[i] = make_double2(lo, hi);
    ++n;
    return true;
  }
  int j = i;
  while (j + 1 < n && A[j + 1].x <= hi) ++j;
  const double nlo = A[i].x < lo ? A[i].x : lo;
  const double nhi = A[j].y > hi ? A[j].y : hi;
  A[i] = make_double2(nlo, nhi);
  if (j > i) {
    const int sh = j - i;
    for (int k = i + 1; k + sh < n; ++k) A[k] = A[k + sh];
    n -= sh;
  }
  return true;
}

// ---------------------------------------------------------------- pass 2

template <bool FILL>
__device__ int pass2_column(int x, int y, int nx, const int32_t *__restrict__ poffs,
                            const double2 *__restrict__ pz, const uint8_t *__restrict__ pd,
                            const DevTables t, const double *__restrict__ sH,
                            const int *__restrict__ sDx, double2 *A, int cap, double2 *outz) {
  int nA = 0;
  const int W = t.W;
  for (int adx = 0; adx < W; ++adx) {
    for (int s = 0; s < 2; ++s) {
      if (adx == 0 && s == 1) break;
      const int xs = s == 0 ? x - adx : x + adx;
      if (xs < 0 || xs >= nx) continue;
      const int c = xs + nx * y;
      const int b = poffs[c], e = poffs[c + 1];
      bool open = false;
      double glo = 0, ghi = 0;
      for (int k = b; k < e; ++k) {
        const int d = pd[k];
        if (adx > sDx[d]) continue;
        const double h = sH[d * W + adx];
        const double2 p = pz[k];
        if (p.x > p.y) {
          if (!union_insert(A, nA, cap, dsub(p.x, h), dadd(p.x, h))) return -1;
          if (!union_insert(A, nA, cap, dsub(p.y, h), dadd(p.y, h))) return -1;
          continue;
        }
        const double lo = dsub(p.x, h), hi = dadd(p.y, h);
        if (open && lo <= ghi && hi >= glo) {
          if (lo < glo) glo = lo;
          if (hi > ghi) ghi = hi;
        } else {
          if (open && !union_insert(A, nA, cap, glo, ghi)) return -1;
          open = true;
          glo = lo;
          ghi = hi;
        }
      }
      if (open && !union_insert(A, nA, cap, glo, ghi)) return -1;
    }
  }
  if (FILL)
    for (int k = 0; k < nA; ++k) outz[k] = A[k];
  return nA;
}

// ---------------------------------------------------------------- brute force

// VoronoiBruteForce.cpp:16-68 for one column: every lattice neighbour within
// the disc (dx^2 + dy^2 <= R*R) contributes [z1 - dz, z2 + dz].
template <bool FILL>
__device__ int brute_column(int x, int y, int nx, int ny, const int32_t *__restrict__ offs,
                            const double2 *__restrict__ z, const DevTables t,
                            const double *__restrict__ sHB, double2 *A, int cap, double2 *outz) {
  int nA = 0;
  const int D = t.Dy;
  for (int dy = -D; dy <= D; ++dy) {
    const int ys = y + dy;
    if (ys < 0 || ys >= ny) continue;
    for (int dx = -D; dx <= D; ++dx) {
      const int xs = x + dx;
      if (xs < 0 || xs >= nx) continue;
      const double dz = sHB[(dy < 0 ? -dy : dy) * (D + 1) + (dx < 0 ? -dx : dx)];
      if (isnan(dz)) continue;
      const int c = xs + nx * ys;
      for (int k = offs[c]; k < offs[c + 1]; ++k) {
        const double2 s = z[k];
        if (!union_insert(A, nA, cap, dsub(s.x, dz), dadd(s.y, dz))) return -1;
      }
    }
  }
  if (FILL)
    for (int k = 0; k < nA; ++k) outz[k] = A[k];
  return nA;
}

// ---------------------------------------------------------------- kernels

struct OvfList {
  int *count;  // device counter
  int *cols;   // device list of overflowing columns
  int *fatal;  // set when even the large capacity overflows
};

__device__ __forceinline__ void record_overflow(const OvfList &o, int col) {
  const int i = atomicAdd(o.count, 1);
  o.cols[i] = col;
}

// Shared-memory copies of the small tables.
struct SmemTables {
  static __device__ void load(const DevTables &t, double *sH, int *sDx, int nH) {
    for (int i = threadIdx.x + blockDim.x * threadIdx.y; i < nH; i += blockDim.x * blockDim.y)
      sH[i] = t.H[i];
    for (int i = threadIdx.x + blockDim.x * threadIdx.y; i <= t.Dy; i += blockDim.x * blockDim.y)
      sDx[i] = t.Dx[i];
  }
};

template <bool FILL>
__global__ void __launch_bounds__(kBX *kBY) k_pass1(int nx, int ny, const int32_t *__restrict__ offs,
                                                    const double2 *__restrict__ z, int Dy,
                                                    int32_t *__restrict__ counts,
                                                    const int32_t *__restrict__ poffs,
                                                    double2 *__restrict__ pz, uint8_t *__restrict__ pd,
                                                    OvfList ovf) {
  const int x = blockIdx.x * kBX + threadIdx.x;
  const int y = blockIdx.y * kBY + threadIdx.y;
  if (x >= nx || y >= ny) return;
  const int c = x + nx * y;
  double2 P[kCapSmall], Q[kCapSmall];
  double2 *oz = FILL ? pz + poffs[c] : nullptr;
  uint8_t *od = FILL ? pd + poffs[c] : nullptr;
  const int n = pass1_column<FILL>(x, y, nx, ny, offs, z, Dy, P, Q, kCapSmall, oz, od);
  if (!FILL) {
    if (n < 0) {
      record_overflow(ovf, c);
      counts[c] = 0;
    } else {
      counts[c] = n;
    }
  }
}

template <bool FILL>
__global__ void __launch_bounds__(kBigThreads) k_pass1_big(int nx, int ny, const int32_t *__restrict__ offs,
                                                          const double2 *__restrict__ z, int Dy,
                                                          int32_t *__restrict__ counts,
                                                          const int32_t *__restrict__ poffs,
                                                          double2 *__restrict__ pz,
                                                          uint8_t *__restrict__ pd, OvfList ovf,
                                                          double2 *scratch) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int nthreads = gridDim.x * blockDim.x;
  double2 *P = scratch + (size_t)tid * 2 * kCapLarge;
  double2 *Q = P + kCapLarge;
  const int n_ovf = *ovf.count;
  for (int i = tid; i < n_ovf; i += nthreads) {
    const int c = ovf.cols[i];
    const int x = c % nx, y = c / nx;
    double2 *oz = FILL ? pz + poffs[c] : nullptr;
    uint8_t *od = FILL ? pd + poffs[c] : nullptr;
    const int n = pass1_column<FILL>(x, y, nx, ny, offs, z, Dy, P, Q, kCapLarge, oz, od);
    if (n < 0) {
      *ovf.fatal = 1;
      if (!FILL) counts[c] = 0;
    } else if (!FILL) {
      counts[c] = n;
    }
  }
}

template <bool FILL>
__global__ void __launch_bounds__(kBX *kBY) k_pass2(int nx, int ny, const int32_t *__restrict__ poffs,
                                                    const double2 *__restrict__ pz,
                                                    const uint8_t *__restrict__ pd, DevTables t,
                                                    int32_t *__restrict__ counts,
                                                    const int32_t *__restrict__ ooffs,
                                                    double2 *__restrict__ oz, OvfList ovf) {
  extern __shared__ double smem[];
  const int nH = (t.Dy + 1) * t.W;
  double *sH = smem;
  int *sDx = (int *)(smem + nH);
  SmemTables::load(t, sH, sDx, nH);
  __syncthreads();
  const int x = blockIdx.x * kBX + threadIdx.x;
  const int y = blockIdx.y * kBY + threadIdx.y;
  if (x >= nx || y >= ny) return;
  const int c = x + nx * y;
  double2 A[kCapSmall];
  const int n = pass2_column<FILL>(x, y, nx, poffs, pz, pd, t, sH, sDx, A, kCapSmall,
                                   FILL ? oz + ooffs[c] : nullptr);
  if (!FILL) {
    if (n < 0) {
      record_overflow(ovf, c);
      counts[c] = 0;
    } else {
      counts[c] = n;
    }
  }
}

template <bool FILL>
__global__ void __launch_bounds__(kBigThreads) k_pass2_big(int nx, int ny, const int32_t *__restrict__ poffs,
                                                          const double2 *__restrict__ pz,
                                                          const uint8_t *__restrict__ pd, DevTables t,
                                                          int32_t *__restrict__ counts,
                                                          const int32_t *__restrict__ ooffs,
                                                          double2 *__restrict__ oz, OvfList ovf,
                                                          double2 *scratch) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int nthreads = gridDim.x * blockDim.x;
  double2 *A = scratch + (size_t)tid * 2 * kCapLarge;
  const int n_ovf = *ovf.count;
  for (int i = tid; i < n_ovf; i += nthreads) {
    const int c = ovf.cols[i];
    const int x = c % nx, y = c / nx;
    const int n = pass2_column<FILL>(x, y, nx, poffs, pz, pd, t, t.H, t.Dx, A, 2 * kCapLarge,
                                     FILL ? oz + ooffs[c] : nullptr);
    if (n < 0) {
      *ovf.fatal = 1;
      if (!FILL) counts[c] = 0;
    } else if (!FILL) {
      counts[c] = n;
    }
  }
}

// Persistent: one wave of blocks pulls kBX x kBY tiles of output columns from
// a work queue (raster order) until none is left. `queue` is zeroed before
// each launch.
template <bool FILL>
__global__ void __launch_bounds__(kBX *kBY) k_brute(int nx, int ny, const int32_t *__restrict__ offs,
                                                    const double2 *__restrict__ z, DevTables t,
                                                    int32_t *__restrict__ counts,
                                                    const int32_t *__restrict__ ooffs,
                                                    double2 *__restrict__ oz, OvfList ovf, int *queue) {
  extern __shared__ double smem[];
  __shared__ int s_tile;
  const int nB = (t.Dy + 1) * (t.Dy + 1);
  const int tid = threadIdx.x + blockDim.x * threadIdx.y;
  for (int i = tid; i < nB; i += blockDim.x * blockDim.y) smem[i] = t.HB[i];
  const int tiles_x = (nx + kBX - 1) / kBX;
  const int ntiles = tiles_x * ((ny + kBY - 1) / kBY);
  for (;;) {
    __syncthreads();  // the table is loaded; the previous tile's index has been read
    if (tid == 0) s_tile = atomicAdd(queue, 1);
    __syncthreads();
    const int tile = s_tile;
    if (tile >= ntiles) break;
    const int x = (tile % tiles_x) * kBX + threadIdx.x;
    const int y = (tile / tiles_x) * kBY + threadIdx.y;
    if (x >= nx || y >= ny) continue;
    const int c = x + nx * y;
    double2 A[kCapSmall];
    const int n = brute_column<FILL>(x, y, nx, ny, offs, z, t, smem, A, kCapSmall,
                                     FILL ? oz + ooffs[c] : nullptr);
    if (!FILL) {
      if (n < 0) {
        record_overflow(ovf, c);
        counts[c] = 0;
      } else {
        counts[c] = n;
      }
    }
  }
}

template <bool FILL>
__global__ void __launch_bounds__(kBigThreads) k_brute_big(int nx, int ny, const int32_t *__restrict__ offs,
                                                          const double2 *__restrict__ z, DevTables t,
                                                          int32_t *__restrict__ counts,
                                                          const int32_t *__restrict__ ooffs,
                                                          double2 *__restrict__ oz, OvfList ovf,
                                                          double2 *scratch) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x;
  const int nthreads = gridDim.x * blockDim.x;
  double2 *A = scratch + (size_t)tid * 2 * kCapLarge;
  const int n_ovf = *ovf.count;
  for (int i = tid; i < n_ovf; i += nthreads) {
    const int c = ovf.cols[i];
    const int x = c % nx, y = c / nx;
    const int n = brute_column<FILL>(x, y, nx, ny, offs, z, t, t.HB, A, 2 * kCapLarge,
                                     FILL ? oz + ooffs[c] : nullptr);
    if (n < 0) {
      *ovf.fatal = 1;
      if (!FILL) counts[c] = 0;
    } else if (!FILL) {
      counts[c] = n;
    }
  }
}

// ---------------------------------------------------------------- erosion

// negate (Voronoi.cpp:18-55) + negate_ray (MorphologyOperators.cpp:230-259):
// grown grid (nx+2) x (ny+2), border columns empty before complementing.
__device__ __forceinline__ int negate_src(int X, int Y, int nx, int ny) {
  return (X >= 1 && X <= nx && Y >= 1 && Y <= ny) ? (X - 1) + nx * (Y - 1) : -1;
}

__global__ void k_negate_count(int nx, int ny, const int32_t *__restrict__ offs,
                               const double2 *__restrict__ z, double zmin, double zmax,
                               int32_t *__restrict__ counts) {
  const int NX = nx + 2, NY = ny + 2;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= NX * NY) return;
  const int src = negate_src(i % NX, i / NX, nx, ny);
  int n2 = 0;
  double v0 = 0, vl = 0;
  if (src >= 0) {
    n2 = 2 * (offs[src + 1] - offs[src]);
    if (n2) {
      v0 = z[offs[src]].x;
      vl = z[offs[src + 1] - 1].y;
    }
  }
  int w;
  if (n2 == 0) {
    w = 2;
  } else {
    w = n2 + (v0 == zmin ? -1 : 1);
    w += (vl == zmax) ? -1 : 1;
  }
  counts[i] = w / 2;
}

__global__ void k_negate_fill(int nx, int ny, const int32_t *__restrict__ offs,
                              const double2 *__restrict__ z, double zmin, double zmax,
                              const int32_t *__restrict__ ooffs, double *__restrict__ oz) {
  const int NX = nx + 2, NY = ny + 2;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= NX * NY) return;
  const int src = negate_src(i % NX, i / NX, nx, ny);
  double *out = oz + 2 * (size_t)ooffs[i];
  const int n2 = src >= 0 ? 2 * (offs[src + 1] - offs[src]) : 0;
  if (n2 == 0) {
    out[0] = zmin;
    out[1] = zmax;
    return;
  }
  const double *v = (const double *)(z + offs[src]);
  int w = 0, k = 0;
  if (v[0] == zmin)
    k = 1;
  else
    out[w++] = zmin;
  for (; k < n2; ++k) out[w++] = v[k];
  if (out[w - 1] == zmax)
    --w;
  else
    out[w++] = zmax;
}

// negateInv (Voronoi.cpp:57-89) + negate_ray_range (MorphologyOperators.cpp:282-315).
template <bool FILL>
__global__ void k_negate_inv(int nx, int ny, const int32_t *__restrict__ offs,
                             const double2 *__restrict__ z, double ymin, double ymax,
                             int32_t *__restrict__ counts, const int32_t *__restrict__ ooffs,
                             double *__restrict__ oz) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nx * ny) return;
  const int x = i % nx, y = i / nx;
  const int c = (x + 1) + (nx + 2) * (y + 1);
  const double *v = (const double *)(z + offs[c]);
  const int n2 = 2 * (offs[c + 1] - offs[c]);
  double *out = FILL ? oz + 2 * (size_t)ooffs[i] : nullptr;
  int w = 0;
  if (n2 == 0) {
    if (FILL) {
      out[0] = ymin;
      out[1] = ymax;
    }
    w = 2;
  } else {
    int b = 0, e = n2, count_first = 0, count_last = 0;
    while (v[b] <= ymin) {
      ++b;
      ++count_first;
      if (b == e) break;
    }
    int has_front = (count_first % 2 == 0);
    for (;;) {
      double back;
      if (e > b)
        back = v[e - 1];
      else if (has_front)
        back = ymin;
      else
        break;
      if (!(back >= ymax)) break;
      if (e > b)
        --e;
      else
        has_front = 0;
      ++count_last;
      if (e == b && !has_front) break;
    }
    if (has_front) {
      if (FILL) out[w] = ymin;
      ++w;
    }
    for (int k = b; k < e; ++k) {
      if (FILL) out[w] = v[k];
      ++w;
    }
    if (count_last % 2 == 0) {
      if (FILL) out[w] = ymax;
      ++w;
    }
  }
  if (!FILL) counts[i] = w / 2;  // w is even for valid (even-length) columns
}

// ---------------------------------------------------------------- scan

constexpr int kScanThreads = 1024, kScanItems = 8, kScanTile = kScanThreads * kScanItems;

__device__ long long block_exclusive_scan(long long v, long long *warp_sums, long long &total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  long long incl = v;
  for (int o = 1; o < 32; o <<= 1) {
    long long t = __shfl_up_sync(0xffffffffu, incl, o);
    if (lane >= o) incl += t;
  }
  if (lane == 31) warp_sums[wid] = incl;
  __syncthreads();
  if (wid == 0) {
    long long s = lane < (int)(blockDim.x >> 5) ? warp_sums[lane] : 0;
    long long si = s;
    for (int o = 1; o < 32; o <<= 1) {
      long long t = __shfl_up_sync(0xffffffffu, si, o);
      if (lane >= o) si += t;
    }
    warp_sums[lane] = si - s;
    if (lane == 31) warp_sums[32] = si;
  }
  __syncthreads();
  total = warp_sums[32];
  const long long r = warp_sums[wid] + incl - v;
  __syncthreads();
  return r;
}

// Per tile: local exclusive scan into offs (as int64 partials), tile sums out.
__global__ void __launch_bounds__(kScanThreads) k_scan_tiles(const int32_t *__restrict__ in, int n,
                                                            long long *__restrict__ tmp,
                                                            long long *__restrict__ tile_sums) {
  __shared__ long long ws[33];
  const int base = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
  long long v[kScanItems];
  long long s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    v[k] = (base + k < n) ? in[base + k] : 0;
    s += v[k];
  }
  long long total;
  long long ex = block_exclusive_scan(s, ws, total);
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    if (base + k < n) tmp[base + k] = ex;
    ex += v[k];
  }
  if (threadIdx.x == 0) tile_sums[blockIdx.x] = total;
}

__global__ void __launch_bounds__(kScanThreads) k_scan_sums(long long *tile_sums, int ntiles,
                                                           long long *d_total) {
  __shared__ long long ws[33];
  const int base = threadIdx.x * kScanItems;
  long long v[kScanItems];
  long long s = 0;
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    v[k] = (base + k < ntiles) ? tile_sums[base + k] : 0;
    s += v[k];
  }
  long long total;
  long long ex = block_exclusive_scan(s, ws, total);
#pragma unroll
  for (int k = 0; k < kScanItems; ++k) {
    if (base + k < ntiles) tile_sums[base + k] = ex;
    ex += v[k];
  }
  if (threadIdx.x == 0) *d_total = total;
}

__global__ void k_scan_finish(const long long *__restrict__ tmp, const long long *__restrict__ tile_sums,
                              int n, const long long *__restrict__ d_total, int32_t *__restrict__ offs) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  const long long tot = *d_total;
  const bool ok = tot <= 2147483647LL;
  if (i < n) offs[i] = ok ? (int32_t)(tmp[i] + tile_sums[i / kScanTile]) : 0;
  if (i == n) offs[n] = ok ? (int32_t)tot : 0;
}

// ---------------------------------------------------------------- normalisation

// Inverted pairs [a, b], a > b (left by negate_ray on a column whose values
// exceed [zmin, zmax]) are rewritten as the points [b, b] and [a, a]; such a
// column is then re-sorted and merged as closed intervals. This is what the
// reference's power-diagram pass sees of them (SeparatePower2D.cpp:215-226
// inserts both endpoints as circles).
constexpr int kNormCap = 64;

__global__ void k_detect_inverted(const double2 *__restrict__ z, int64_t nseg, int *flag) {
  bool f = false;
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < nseg; i += (int64_t)gridDim.x * blockDim.x) {
    const double2 s = z[i];
    f |= s.x > s.y;
  }
  if (__any_sync(0xffffffffu, f) && (threadIdx.x & 31) == 0) atomicOr(flag, 1);
}

__device__ int norm_column(const double2 *__restrict__ z, int k0, int k1, double2 *buf, int cap, double2 *out) {
  bool inv = false;
  for (int k = k0; k < k1; ++k) inv |= z[k].x > z[k].y;
  if (!inv) {
    if (out)
      for (int k = k0; k < k1; ++k) out[k - k0] = z[k];
    return k1 - k0;
  }
  int n = 0;
  for (int k = k0; k < k1; ++k) {
    const double2 s = z[k];
    double2 parts[2];
    int np = 0;
    if (s.x > s.y) {
      parts[np++] = make_double2(s.y, s.y);
      parts[np++] = make_double2(s.x, s.x);
    } else {
      parts[np++] = s;
    }
    for (int q = 0; q < np; ++q) {
      if (n >= cap) return -1;
      int i = n++;  // insertion sort by (lo, hi)
      while (i > 0 && (buf[i - 1].x > parts[q].x || (buf[i - 1].x == parts[q].x && buf[i - 1].y > parts[q].y))) {
        buf[i] = buf[i - 1];
        --i;
      }
      buf[i] = parts[q];
    }
  }
  int w = 0;
  for (int i = 0; i < n; ++i) {
    if (w > 0 && !(buf[w - 1].y < buf[i].x)) {
      if (buf[i].y > buf[w - 1].y) buf[w - 1].y = buf[i].y;
    } else {
      buf[w++] = buf[i];
    }
  }
  if (out)
    for (int i = 0; i < w; ++i) out[i] = buf[i];
  return w;
}

template <bool FILL>
__global__ void k_norm(int ncols, const int32_t *__restrict__ offs, const double2 *__restrict__ z,
                       int32_t *counts, const int32_t *ooffs, double2 *oz, OvfList ovf) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncols) return;
  double2 buf[kNormCap];
  const int n = norm_column(z, offs[c], offs[c + 1], buf, kNormCap, FILL ? oz + ooffs[c] : nullptr);
  if (!FILL) {
    if (n < 0) {
      record_overflow(ovf, c);
      counts[c] = 0;
    } else {
      counts[c] = n;
    }
  }
}

template <bool FILL>
__global__ void k_norm_big(const int32_t *__restrict__ offs, const double2 *__restrict__ z, int32_t *counts,
                           const int32_t *ooffs, double2 *oz, OvfList ovf, double2 *scratch) {
  const int tid = blockIdx.x * blockDim.x + threadIdx.x, nth = gridDim.x * blockDim.x;
  double2 *buf = scratch + (size_t)tid * 2 * kCapLarge;
  for (int i = tid; i < *ovf.count; i += nth) {
    const int c = ovf.cols[i];
    const int n = norm_column(z, offs[c], offs[c + 1], buf, 2 * kCapLarge, FILL ? oz + ooffs[c] : nullptr);
    if (n < 0) *ovf.fatal = 1;
    if (!FILL) counts[c] = n < 0 ? 0 : n;
  }
}

// ---------------------------------------------------------------- slot layout

// Fixed-capacity "slot" volumes hold column c's segments at z[c*cap ..
// c*cap + n_c) with end[c] = c*cap + n_c; they let a chain of stages run
// without knowing output sizes in advance (no host synchronisation), which is
// what the batched executor needs to capture a whole batch in a CUDA graph.

// negate_ray on the values v[0..n2) within [zmin, zmax] (MorphologyOperators.cpp:230-259);
// returns the number of values written to out.
__device__ int negate_vals(const double *v, int n2, double zmin, double zmax, double *out) {
  if (n2 == 0) {
    out[0] = zmin;
    out[1] = zmax;
    return 2;
  }
  int w = 0, k = 0;
  if (v[0] == zmin)
    k = 1;
  else
    out[w++] = zmin;
  for (; k < n2; ++k) out[w++] = v[k];
  if (out[w - 1] == zmax)
    --w;
  else
    out[w++] = zmax;
  return w;
}

// negate_ray_range (MorphologyOperators.cpp:282-315); returns the value count.
__device__ int negate_range_vals(const double *v, int n2, double ymin, double ymax, double *out) {
  if (n2 == 0) {
    out[0] = ymin;
    out[1] = ymax;
    return 2;
  }
  int b = 0, e = n2, count_first = 0, count_last = 0, w = 0;
  while (v[b] <= ymin) {
    ++b;
    ++count_first;
    if (b == e) break;
  }
  int has_front = (count_first % 2 == 0);
  for (;;) {
    double back;
    if (e > b)
      back = v[e - 1];
    else if (has_front)
      back = ymin;
    else
      break;
    if (!(back >= ymax)) break;
    if (e > b)
      --e;
    else
      has_front = 0;
    ++count_last;
    if (e == b && !has_front) break;
  }
  if (has_front) out[w++] = ymin;
  for (int k = b; k < e; ++k) out[w++] = v[k];
  if (count_last % 2 == 0) out[w++] = ymax;
  return w;
}

__global__ void k_slot_beg(int ncols, int cap, int32_t *beg) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c < ncols) beg[c] = c * cap;
}


// negate (Voronoi.cpp:18-55) into a grown (nx+2) x (ny+2) slot volume.
__global__ void k_negate_slot(int nx, int ny, const int32_t *__restrict__ beg, const int32_t *__restrict__ end,
                              const double2 *__restrict__ z, double zmin, double zmax, int cap, int32_t *oend,
                              double2 *oz, int *overflow) {
  const int NX = nx + 2, NY = ny + 2;
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= NX * NY) return;
  const int src = negate_src(i % NX, i / NX, nx, ny);
  const int n2 = src >= 0 ? 2 * (end[src] - beg[src]) : 0;
  if (n2 / 2 + 1 > cap) {
    atomicOr(overflow, 1);
    oend[i] = i * cap;
    return;
  }
  const int w = negate_vals(src >= 0 ? (const double *)(z + beg[src]) : nullptr, n2, zmin, zmax,
                            (double *)(oz + (size_t)i * cap));
  oend[i] = i * cap + w / 2;
}

// Inverted-pair normalisation (see norm_column) slot to slot.
__global__ void k_norm_slot(int ncols, const int32_t *__restrict__ beg, const int32_t *__restrict__ end,
                            const double2 *__restrict__ z, int cap, int32_t *oend, double2 *oz, int *overflow) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= ncols) return;
  double2 buf[kNormCap];
  const int k0 = beg[c], k1 = end[c];
  int n = -1;
  if (k1 - k0 + 2 <= cap) n = norm_column(z, k0, k1, buf, kNormCap, oz + (size_t)c * cap);
  if (n < 0 || n > cap) {
    atomicOr(overflow, 1);
    n = 0;
  }
  oend[c] = c * cap + n;
}

// negateInv (Voronoi.cpp:57-89): crop the one-column border, complement within [ymin, ymax].
__global__ void k_negate_inv_slot(int nx, int ny, const int32_t *__restrict__ beg, const int32_t *__restrict__ end,
                                  const double2 *__restrict__ z, double ymin, double ymax, int cap, int32_t *oend,
                                  double2 *oz, int *overflow) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nx * ny) return;
  const int c = (i % nx + 1) + (nx + 2) * (i / nx + 1);
  const int n2 = 2 * (end[c] - beg[c]);
  if (n2 / 2 + 1 > cap) {
    atomicOr(overflow, 1);
    oend[i] = i * cap;
    return;
  }
  const int w = negate_range_vals((const double *)(z + beg[c]), n2, ymin, ymax, (double *)(oz + (size_t)i * cap));
  oend[i] = i * cap + w / 2;
}

__global__ void k_slot_counts(int ncols, const int32_t *beg, const int32_t *end, int32_t *counts, int *maxc) {
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  int n = 0;
  if (c < ncols) {
    n = end[c] - beg[c];
    if (counts) counts[c] = n;
  }
  if (maxc) {
    for (int o = 16; o > 0; o >>= 1) n = max(n, __shfl_xor_sync(0xffffffffu, n, o));
    if ((threadIdx.x & 31) == 0) atomicMax(maxc, n);
  }
}

__global__ void k_slot_compact(int ncols, const int32_t *__restrict__ beg, const double2 *__restrict__ z,
                               const int32_t *__restrict__ ooffs, double2 *__restrict__ oz) {
  const int w = (blockIdx.x * blockDim.x + threadIdx.x) >> 5, lane = threadIdx.x & 31;
  if (w >= ncols) return;
  const int n = ooffs[w + 1] - ooffs[w];
  for (int k = lane; k < n; k += 32) oz[ooffs[w] + k] = z[beg[w] + k];
}

}  // namespace

// ================================================================ host side

int scan_counts(vo_ctx *ctx, const int32_t *counts, int32_t *offs, int n, long long *total) {
  const int ntiles = (n + kScanTile - 1) / kScanTile;
  if (ntiles > kScanTile) return set_error(ctx, VO_ERANGE, "scan: too many columns");
  long long *tmp = nullptr, *sums = nullptr;
  int rc = dalloc(ctx, &tmp, (size_t)n + 1);
  if (rc) return rc;
  rc = dalloc(ctx, &sums, (size_t)ntiles + 1);
  if (rc) {
    dfree(ctx, tmp);
    return rc;
  }
  if (n > 0) {
    k_scan_tiles<<<ntiles, kScanThreads, 0, ctx->stream>>>(counts, n, tmp, sums);
    k_scan_sums<<<1, kScanThreads, 0, ctx->stream>>>(sums, ntiles, ctx->d_total);
  } else {
    cudaMemsetAsync(ctx->d_total, 0, sizeof(long long), ctx->stream);
  }
  k_scan_finish<<<(n + 1 + 255) / 256, 256, 0, ctx->stream>>>(tmp, sums, n, ctx->d_total, offs);
  ctx->launches += n > 0 ? 3 : 1;
  cudaMemcpyAsync(ctx->h_total, ctx->d_total, sizeof(long long), cudaMemcpyDeviceToHost, ctx->stream);
  dfree(ctx, tmp);
  dfree(ctx, sums);
  VO_CK(ctx, cudaStreamSynchronize(ctx->stream));
  VO_CK(ctx, cudaGetLastError());
  *total = *ctx->h_total;
  if (*total > 2147483647LL) return set_error(ctx, VO_ERANGE, "result exceeds int32 CSR offsets");
  return VO_OK;
}

namespace {

struct Scratch {
  int32_t *counts = nullptr;
  int *ovf_cols = nullptr;
  double2 *big = nullptr;
};

int big_grid() {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms > 0 ? sms : 148;
}

int alloc_scratch(vo_ctx *ctx, int ncols, Scratch &s) {
  int rc = dalloc(ctx, &s.counts, (size_t)ncols);
  if (!rc) rc = dalloc(ctx, &s.ovf_cols, (size_t)ncols);
  if (!rc) rc = dalloc(ctx, &s.big, (size_t)big_grid() * kBigThreads * 2 * kCapLarge);
  return rc;
}

void free_scratch(vo_ctx *ctx, Scratch &s) {
  dfree(ctx, s.counts);
  dfree(ctx, s.ovf_cols);
  dfree(ctx, s.big);
  s = Scratch();
}

int check_fatal(vo_ctx *ctx) {
  int h[2] = {0, 0};
  VO_CK(ctx, cudaMemcpyAsync(h, ctx->d_flags, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
  VO_CK(ctx, cudaStreamSynchronize(ctx->stream));
  ctx->ovf_cols += h[0];
  if (h[1]) return set_error(ctx, VO_EINTERNAL, "column exceeds the large working-list capacity");
  return VO_OK;
}

}  // namespace

int normalize_inverted(vo_ctx *ctx, const vo_volume *in, vo_volume **out) {
  *out = nullptr;
  if (in->inverted == 0 || in->nseg == 0) {
    in->inverted = 0;
    return VO_OK;
  }
  if (in->inverted < 0) {
    int h = 0;
    VO_CK(ctx, cudaMemsetAsync(ctx->d_flags + 2, 0, sizeof(int), ctx->stream));
    const int grid = (int)std::min<int64_t>((in->nseg + 255) / 256, 152 * 16);
    k_detect_inverted<<<grid, 256, 0, ctx->stream>>>(in->z, in->nseg, ctx->d_flags + 2);
    ctx->launches += 1;
    VO_CK(ctx, cudaMemcpyAsync(&h, ctx->d_flags + 2, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    VO_CK(ctx, cudaStreamSynchronize(ctx->stream));
    in->inverted = h ? 1 : 0;
    if (!h) return VO_OK;
  }
  const int ncols = in->grid.nx * in->grid.ny;
  Scratch s;
  int rc = alloc_scratch(ctx, ncols, s);
  if (rc) return rc;
  OvfList ovf{ctx->d_flags, s.ovf_cols, ctx->d_flags + 1};
  vo_volume *res = nullptr;
  long long total = 0;
  const int gbig = big_grid();
  cudaMemsetAsync(ctx->d_flags, 0, 2 * sizeof(int), ctx->stream);
  k_norm<false><<<(ncols + 127) / 128, 128, 0, ctx->stream>>>(ncols, in->offs, in->z, s.counts, nullptr, nullptr,
                                                              ovf);
  k_norm_big<false><<<gbig, kBigThreads, 0, ctx->stream>>>(in->offs, in->z, s.counts, nullptr, nullptr, ovf, s.big);
  ctx->launches += 2;
  rc = volume_alloc(ctx, in->grid, 0, &res);
  if (!rc) rc = scan_counts(ctx, s.counts, res->offs, ncols, &total);
  if (!rc) {
    res->nseg = total;
    rc = dalloc(ctx, &res->z, (size_t)total);
  }
  if (!rc) {
    k_norm<true><<<(ncols + 127) / 128, 128, 0, ctx->stream>>>(ncols, in->offs, in->z, nullptr, res->offs, res->z,
                                                               ovf);
    k_norm_big<true><<<gbig, kBigThreads, 0, ctx->stream>>>(in->offs, in->z, nullptr, res->offs, res->z, ovf, s.big);
    ctx->launches += 2;
    rc = check_fatal(ctx);
  }
  free_scratch(ctx, s);
  if (rc) {
    if (res) vo_volume_free(ctx, res);
    return rc;
  }
  res->inverted = 0;
  *out = res;
  return VO_OK;
}

int dilate(vo_ctx *ctx, int method, double R, const vo_volume *in_user, vo_volume **out,
           vo_timings *tm) {
  vo_volume *norm = nullptr;
  int nrc = normalize_inverted(ctx, in_user, &norm);
  if (nrc) return nrc;
  const vo_volume *in = norm ? norm : in_user;
  if (method == VO_METHOD_ENVELOPE) {
    nrc = dilate_envelope(ctx, R, in, out, tm);
    if (nrc == 1) {  // beyond the sweeps' working capacities: the painter form has none
      ctx->err.clear();
      method = VO_METHOD_SEPARABLE;
    } else {
      if (norm) vo_volume_free(ctx, norm);
      if (!nrc) (*out)->inverted = 0;
      return nrc;
    }
  }
  if (method == VO_METHOD_FAST) {
    nrc = dilate_fast(ctx, R, in, out, tm);
    if (norm) vo_volume_free(ctx, norm);
    if (!nrc) (*out)->inverted = 0;
    return nrc;
  }
  const vo_grid g = in->grid;
  const int nx = g.nx, ny = g.ny, ncols = nx * ny;
  const DeviceTables *T = nullptr;
  int rc = get_tables(ctx, R, std::max(nx, ny), &T);
  Scratch s;
  if (!rc) rc = alloc_scratch(ctx, ncols, s);
  if (rc) {
    if (norm) vo_volume_free(ctx, norm);
    return rc;
  }
  const DevTables t = T->view();
  OvfList ovf{ctx->d_flags, s.ovf_cols, ctx->d_flags + 1};
  const dim3 blk(kBX, kBY), grd((nx + kBX - 1) / kBX, (ny + kBY - 1) / kBY);
  const int gbig = big_grid();
  vo_volume *res = nullptr;
  long long total = 0;

  if (method == VO_METHOD_BRUTE) {
    cudaEventRecord(ctx->ev[0], ctx->stream);
    const size_t shb = sizeof(double) * (size_t)(t.Dy + 1) * (t.Dy + 1);
    if (shb > 200 * 1024) {
      free_scratch(ctx, s);
      if (norm) vo_volume_free(ctx, norm);
      return set_error(ctx, VO_EINVAL, "brute force supports radius < 160");
    }
    cudaFuncSetAttribute(k_brute<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shb);
    cudaFuncSetAttribute(k_brute<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)shb);
    // one wave of persistent blocks; d_flags[4] is the tile queue
    int per_sm = 0, sms = 0;
    cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_brute<false>, kBX * kBY, shb);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, ctx->device);
    const int pgrid = std::max(1, per_sm) * std::max(1, sms);
    int *queue = ctx->d_flags + 4;
    cudaMemsetAsync(ctx->d_flags, 0, 2 * sizeof(int), ctx->stream);
    cudaMemsetAsync(queue, 0, sizeof(int), ctx->stream);
    cudaEventRecord(ctx->ev[4], ctx->stream);
    k_brute<false><<<pgrid, blk, shb, ctx->stream>>>(nx, ny, in->offs, in->z, t, s.counts, nullptr,
                                                     nullptr, ovf, queue);
    k_brute_big<false><<<gbig, kBigThreads, 0, ctx->stream>>>(nx, ny, in->offs, in->z, t, s.counts,
                                                             nullptr, nullptr, ovf, s.big);
    ctx->launches += 2;
    cudaEventRecord(ctx->ev[5], ctx->stream);
    rc = volume_alloc(ctx, g, 0, &res);
    if (!rc) rc = scan_counts(ctx, s.counts, res->offs, ncols, &total);
    if (!rc) {
      res->nseg = total;
      rc = dalloc(ctx, &res->z, (size_t)total);
    }
    if (!rc) {
      cudaEventRecord(ctx->ev[6], ctx->stream);
      cudaMemsetAsync(queue, 0, sizeof(int), ctx->stream);
      k_brute<true><<<pgrid, blk, shb, ctx->stream>>>(nx, ny, in->offs, in->z, t, nullptr, res->offs,
                                                      res->z, ovf, queue);
      k_brute_big<true><<<gbig, kBigThreads, 0, ctx->stream>>>(nx, ny, in->offs, in->z, t, nullptr,
                                                              res->offs, res->z, ovf, s.big);
      ctx->launches += 2;
      cudaEventRecord(ctx->ev[7], ctx->stream);
      rc = check_fatal(ctx);
    }
    if (!rc && tm) {
      float a = 0, b = 0, c = 0;
      cudaEventElapsedTime(&a, ctx->ev[0], ctx->ev[7]);
      cudaEventElapsedTime(&b, ctx->ev[4], ctx->ev[5]);
      cudaEventElapsedTime(&c, ctx->ev[6], ctx->ev[7]);
      tm->pass2_ms += a;
      tm->kernel_ms[2] += b;
      tm->kernel_ms[3] += c;
    }
  } else {
    // ---- pass 1
    cudaMemsetAsync(ctx->d_flags, 0, 2 * sizeof(int), ctx->stream);
    cudaEventRecord(ctx->ev[0], ctx->stream);
    k_pass1<false><<<grd, blk, 0, ctx->stream>>>(nx, ny, in->offs, in->z, t.Dy, s.counts, nullptr,
                                                 nullptr, nullptr, ovf);
    k_pass1_big<false><<<gbig, kBigThreads, 0, ctx->stream>>>(nx, ny, in->offs, in->z, t.Dy, s.counts,
                                                             nullptr, nullptr, nullptr, ovf, s.big);
    ctx->launches += 2;
    cudaEventRecord(ctx->ev[1], ctx->stream);
    int32_t *poffs = nullptr;
    double2 *pz = nullptr;
    uint8_t *pd = nullptr;
    long long ptotal = 0;
    rc = dalloc(ctx, &poffs, (size_t)ncols + 1);
    if (!rc) rc = scan_counts(ctx, s.counts, poffs, ncols, &ptotal);
    if (!rc) rc = dalloc(ctx, &pz, (size_t)ptotal);
    if (!rc) rc = dalloc(ctx, &pd, (size_t)ptotal);
    if (!rc) {
      cudaEventRecord(ctx->ev[2], ctx->stream);
      k_pass1<true><<<grd, blk, 0, ctx->stream>>>(nx, ny, in->offs, in->z, t.Dy, nullptr, poffs, pz,
                                                  pd, ovf);
      k_pass1_big<true><<<gbig, kBigThreads, 0, ctx->stream>>>(nx, ny, in->offs, in->z, t.Dy, nullptr,
                                                              poffs, pz, pd, ovf, s.big);
      ctx->launches += 2;
      cudaEventRecord(ctx->ev[3], ctx->stream);
      rc = check_fatal(ctx);
    }
    // ---- pass 2
    if (!rc) {
      const size_t sh = sizeof(double) * (size_t)(t.Dy + 1) * t.W + sizeof(int) * (t.Dy + 1);
      if (sh > 200 * 1024) {
        rc = set_error(ctx, VO_EINVAL, "radius too large for the pass-2 table");
      } else {
        cudaFuncSetAttribute(k_pass2<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sh);
        cudaFuncSetAttribute(k_pass2<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sh);
        cudaMemsetAsync(ctx->d_flags, 0, 2 * sizeof(int), ctx->stream);
        cudaEventRecord(ctx->ev[4], ctx->stream);
        k_pass2<false><<<grd, blk, sh, ctx->stream>>>(nx, ny, poffs, pz, pd, t, s.counts, nullptr,
                                                      nullptr, ovf);
        k_pass2_big<false><<<gbig, kBigThreads, 0, ctx->stream>>>(nx, ny, poffs, pz, pd, t, s.counts,
                                                                 nullptr, nullptr, ovf, s.big);
        ctx->launches += 2;
        cudaEventRecord(ctx->ev[5], ctx->stream);
        rc = volume_alloc(ctx, g, 0, &res);
        if (!rc) rc = scan_counts(ctx, s.counts, res->offs, ncols, &total);
        if (!rc) {
          res->nseg = total;
          rc = dalloc(ctx, &res->z, (size_t)total);
        }
        if (!rc) {
          cudaEventRecord(ctx->ev[6], ctx->stream);
          k_pass2<true><<<grd, blk, sh, ctx->stream>>>(nx, ny, poffs, pz, pd, t, nullptr, res->offs,
                                                       res->z, ovf);
          k_pass2_big<true><<<gbig, kBigThreads, 0, ctx->stream>>>(nx, ny, poffs, pz, pd, t, nullptr,
                                                                  res->offs, res->z, ovf, s.big);
          ctx->launches += 2;
          cudaEventRecord(ctx->ev[7], ctx->stream);
          rc = check_fatal(ctx);
        }
      }
    }
    if (!rc && tm) {
      float e[8];
      for (int i = 0; i < 4; ++i) cudaEventElapsedTime(&e[i], ctx->ev[2 * i], ctx->ev[2 * i + 1]);
      cudaEventElapsedTime(&e[4], ctx->ev[0], ctx->ev[3]);
      cudaEventElapsedTime(&e[5], ctx->ev[4], ctx->ev[7]);
      for (int i = 0; i < 4; ++i) tm->kernel_ms[i] += e[i];
      tm->pass1_ms += e[4];
      tm->pass2_ms += e[5];
      tm->mid_pieces += ptotal;
    }
    dfree(ctx, poffs);
    dfree(ctx, pz);
    dfree(ctx, pd);
  }
  free_scratch(ctx, s);
  if (norm) vo_volume_free(ctx, norm);
  if (rc) {
    if (res) vo_volume_free(ctx, res);
    return rc;
  }
  VO_CK(ctx, cudaGetLastError());
  res->inverted = 0;
  *out = res;
  return VO_OK;
}

int erode(vo_ctx *ctx, int method, double R, const vo_volume *in, vo_volume **out,
          vo_timings *tm) {
  const vo_grid g = in->grid;
  // VoronoiMorpho::erosion (Voronoi.cpp:8-17)
  const double zmin = g.origin[2] / g.spacing - 1;
  const double zmax = g.origin[2] / g.spacing + 2 * g.padding + g.extent[2] / g.spacing + 1;
  vo_grid g2 = g;
  g2.nx += 2;
  g2.ny += 2;
  const int n2 = g2.nx * g2.ny, n = g.nx * g.ny;
  int32_t *counts = nullptr;
  int rc = dalloc(ctx, &counts, (size_t)std::max(n2, n));
  if (rc) return rc;
  vo_volume *neg = nullptr, *dil = nullptr, *res = nullptr;
  long long total = 0;
  rc = volume_alloc(ctx, g2, 0, &neg);
  if (!rc) {
    k_negate_count<<<(n2 + 255) / 256, 256, 0, ctx->stream>>>(g.nx, g.ny, in->offs, in->z, zmin, zmax,
                                                             counts);
    ctx->launches += 1;
    rc = scan_counts(ctx, counts, neg->offs, n2, &total);
  }
  if (!rc) {
    neg->nseg = total;
    rc = dalloc(ctx, &neg->z, (size_t)total);
  }
  if (!rc) {
    k_negate_fill<<<(n2 + 255) / 256, 256, 0, ctx->stream>>>(g.nx, g.ny, in->offs, in->z, zmin, zmax,
                                                            neg->offs, (double *)neg->z);
    ctx->launches += 1;
    rc = dilate(ctx, method, R, neg, &dil, tm);
  }
  if (!rc) rc = volume_alloc(ctx, g, 0, &res);
  if (!rc) {
    k_negate_inv<false><<<(n + 255) / 256, 256, 0, ctx->stream>>>(g.nx, g.ny, dil->offs, dil->z, zmin + 1,
                                                                 zmax - 1, counts, nullptr, nullptr);
    ctx->launches += 1;
    rc = scan_counts(ctx, counts, res->offs, n, &total);
  }
  if (!rc) {
    res->nseg = total;
    rc = dalloc(ctx, &res->z, (size_t)total);
  }
  if (!rc) {
    k_negate_inv<true><<<(n + 255) / 256, 256, 0, ctx->stream>>>(g.nx, g.ny, dil->offs, dil->z, zmin + 1,
                                                                zmax - 1, nullptr, res->offs,
                                                                (double *)res->z);
    ctx->launches += 1;
  }
  dfree(ctx, counts);
  if (neg) vo_volume_free(ctx, neg);
  if (dil) vo_volume_free(ctx, dil);
  if (rc) {
    if (res) vo_volume_free(ctx, res);
    return rc;
  }
  VO_CK(ctx, cudaGetLastError());
  *out = res;
  return VO_OK;
}

// ---------------------------------------------------------------- slot launchers

namespace {
inline int nblocks(int64_t n, int t) { return (int)((n + t - 1) / t); }
}  // namespace

int slot_alloc(vo_ctx *ctx, const vo_grid &g, int cap, SlotVol &v) {
  v = SlotVol();
  v.grid = g;
  v.cap = cap;
  const int ncols = g.nx * g.ny;
  v.entries = (int64_t)ncols * std::max(cap, 1);
  int rc = dalloc(ctx, &v.beg, (size_t)ncols);
  if (!rc) rc = dalloc(ctx, &v.end, (size_t)ncols);
  if (!rc) rc = dalloc(ctx, &v.z, (size_t)ncols * (size_t)std::max(cap, 1));
  if (rc) {
    slot_free(ctx, v);
    return rc;
  }
  v.owns = true;
  k_slot_beg<<<nblocks(ncols, 256), 256, 0, ctx->stream>>>(ncols, cap, v.beg);
  ctx->launches += 1;
  return VO_OK;
}

void slot_free(vo_ctx *ctx, SlotVol &v) {
  if (v.owns) {
    dfree(ctx, v.beg);
    dfree(ctx, v.end);
    dfree(ctx, v.z);
  }
  v = SlotVol();
}

SlotVol slot_view(const vo_volume *in, int cap) {
  SlotVol v;
  v.grid = in->grid;
  v.cap = cap;
  v.beg = in->offs;
  v.end = in->offs + 1;
  v.z = in->z;
  v.entries = in->nseg;
  v.owns = false;
  return v;
}

void slot_negate_launch(cudaStream_t st, const SlotVol &in, const SlotVol &out, int *overflow) {
  const vo_grid &g = in.grid;
  const double zmin = g.origin[2] / g.spacing - 1;
  const double zmax = g.origin[2] / g.spacing + 2 * g.padding + g.extent[2] / g.spacing + 1;
  k_negate_slot<<<nblocks((int64_t)(g.nx + 2) * (g.ny + 2), 256), 256, 0, st>>>(
      g.nx, g.ny, in.beg, in.end, in.z, zmin, zmax, out.cap, out.end, out.z, overflow);
}

void slot_normalize_launch(cudaStream_t st, const SlotVol &in, const SlotVol &out, int *overflow) {
  const int ncols = in.grid.nx * in.grid.ny;
  k_norm_slot<<<nblocks(ncols, 128), 128, 0, st>>>(ncols, in.beg, in.end, in.z, out.cap, out.end, out.z, overflow);
}

void slot_negate_inv_launch(cudaStream_t st, const SlotVol &in, const vo_grid &g, const SlotVol &out,
                            int *overflow) {
  const double zmin = g.origin[2] / g.spacing - 1;
  const double zmax = g.origin[2] / g.spacing + 2 * g.padding + g.extent[2] / g.spacing + 1;
  k_negate_inv_slot<<<nblocks((int64_t)g.nx * g.ny, 256), 256, 0, st>>>(
      g.nx, g.ny, in.beg, in.end, in.z, zmin + 1, zmax - 1, out.cap, out.end, out.z, overflow);
}

int slot_max_count(vo_ctx *ctx, const SlotVol &v, int *d_max) {
  const int ncols = v.grid.nx * v.grid.ny;
  k_slot_counts<<<nblocks(ncols, 256), 256, 0, ctx->stream>>>(ncols, v.beg, v.end, nullptr, d_max);
  ctx->launches += 1;
  return VO_OK;
}

int slot_to_volume(vo_ctx *ctx, const SlotVol &v, vo_volume **out) {
  const int ncols = v.grid.nx * v.grid.ny;
  int32_t *counts = nullptr;
  int rc = dalloc(ctx, &counts, (size_t)ncols);
  if (rc) return rc;
  vo_volume *res = nullptr;
  long long total = 0;
  k_slot_counts<<<nblocks(ncols, 256), 256, 0, ctx->stream>>>(ncols, v.beg, v.end, counts, nullptr);
  ctx->launches += 1;
  rc = volume_alloc(ctx, v.grid, 0, &res);
  if (!rc) rc = scan_counts(ctx, counts, res->offs, ncols, &total);
  if (!rc) {
    res->nseg = total;
    rc = dalloc(ctx, &res->z, (size_t)total);
  }
  if (!rc) {
    k_slot_compact<<<nblocks((int64_t)ncols * 32, 256), 256, 0, ctx->stream>>>(ncols, v.beg, v.z, res->offs,
                                                                               res->z);
    ctx->launches += 1;
  }
  dfree(ctx, counts);
  if (rc) {
    if (res) vo_volume_free(ctx, res);
    return rc;
  }
  *out = res;
  return VO_OK;
}

}  // namespace vo
