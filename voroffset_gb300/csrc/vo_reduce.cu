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
#include <algorithm>
#include <mutex>

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

// Segment count and volume (CompressedVolume::numSegments / get_volume,
// CompressedVolume.cpp:61-83): per segment h^3 * (z2 - z1), as the reference
// adds it, summed per block of columns, then the block partials in a fixed
// order (deterministic; the reference's sequential sum rounds differently, by
// relative amounts of order 1e-15 times the segment count).
__global__ void k_measure(int ncols, const int32_t *__restrict__ offs, const double2 *__restrict__ z, double h3,
                          double *__restrict__ partial, unsigned long long *__restrict__ nseg) {
  __shared__ double s[kThreads];
  const int c = blockIdx.x * kThreads + threadIdx.x;
  double v = 0;
  unsigned long long n = 0;
  if (c < ncols) {
    for (int k = offs[c]; k < offs[c + 1]; ++k) v += h3 * (z[k].y - z[k].x);
    n = (unsigned long long)(offs[c + 1] - offs[c]);
  }
  for (int o = 16; o > 0; o >>= 1) n += __shfl_xor_sync(0xffffffffu, n, o);
  if ((threadIdx.x & 31) == 0 && n) atomicAdd(nseg, n);
  s[threadIdx.x] = v;
  __syncthreads();
  for (int o = kThreads / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) s[threadIdx.x] += s[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) partial[blockIdx.x] = s[0];
}

}  // namespace
}  // namespace vo

using namespace vo;

extern "C" int vo_volume_measure(vo_ctx *ctx, const vo_volume *v, int64_t *num_segments, double *volume) {
  if (!ctx) return VO_EINVAL;
  if (!v || !num_segments || !volume) return set_error(ctx, VO_EINVAL, "measure: NULL argument");
  cudaSetDevice(ctx->device);
  vol_wait(ctx, v);
  ctx->err.clear();
  const int ncols = v->grid.nx * v->grid.ny;
  const int nblk = std::max(1, (ncols + kThreads - 1) / kThreads);
  double *partial = nullptr, *d_out = nullptr;
  int rc = dalloc(ctx, &partial, (size_t)nblk);
  if (!rc) rc = dalloc(ctx, &d_out, 1);
  if (rc) {
    dfree(ctx, partial);
    return rc;
  }
  unsigned long long *d_n = reinterpret_cast<unsigned long long *>(ctx->d_total);
  cudaMemsetAsync(d_n, 0, sizeof(unsigned long long), ctx->stream);
  cudaMemsetAsync(partial, 0, sizeof(double) * nblk, ctx->stream);
  const double h = v->grid.spacing;
  if (ncols > 0)
    k_measure<<<nblk, kThreads, 0, ctx->stream>>>(ncols, v->offs, v->z, h * h * h, partial, d_n);
  k_sum<<<1, kThreads, 0, ctx->stream>>>(partial, nblk, d_out);
  double hv = 0;
  unsigned long long hn = 0;
  cudaMemcpyAsync(&hv, d_out, sizeof(double), cudaMemcpyDeviceToHost, ctx->stream);
  cudaMemcpyAsync(&hn, d_n, sizeof hn, cudaMemcpyDeviceToHost, ctx->stream);
  dfree(ctx, partial);
  dfree(ctx, d_out);
  VO_CK(ctx, cudaStreamSynchronize(ctx->stream));
  VO_CK(ctx, cudaGetLastError());
  *num_segments = (int64_t)hn;
  *volume = hv;
  return VO_OK;
}

extern "C" int vo_xor_volume(vo_ctx *ctx, const vo_volume *a, const vo_volume *b, double *volume) {
  if (!ctx) return VO_EINVAL;
  if (!a || !b || !volume) return set_error(ctx, VO_EINVAL, "xor: NULL argument");
  if (a->grid.nx != b->grid.nx || a->grid.ny != b->grid.ny)
    return set_error(ctx, VO_EINVAL, "xor: grids differ");
  cudaSetDevice(ctx->device);
  vol_wait(ctx, a);
  vol_wait(ctx, b);
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

// ============================================================ allocation-free variant
//
// vo_xor_volume_noalloc runs the same two kernels as vo_xor_volume, but its
// scratch (one partial sum per block of kThreads columns, plus the result)
// is the fixed-size array below instead of memory allocated per call. It is
// for callers that must not allocate device memory while they run: services
// whose device memory budget is owned by another allocator (a caching pool
// that must see every byte), and hot loops that must stay off the
// allocator's locks and its synchronisation. It is called from ordinary host
// code; like every CUDA call it must not be made from inside a host function
// enqueued on a stream. Every GPU that loads this library holds the array
// until the process exits: (kNoAllocMaxBlocks + 1) doubles, 512 KiB + 8 B.

namespace vo {
namespace {

constexpr int kNoAllocMaxBlocks = 65536;  // at most 65536 * 256 = 16,777,216 columns
constexpr int kNoAllocMaxDevices = 64;

static __device__ __align__(256) double g_xor_scratch[kNoAllocMaxBlocks + 1];

// Device address of g_xor_scratch, looked up once per device (in host code the
// symbol itself is only a host-side stand-in and must not be passed to a
// kernel). The address stays valid for the life of the device's primary
// context, so a process that uses this entry point must not reset the device
// (cudaDeviceReset) afterwards.
double *g_xor_scratch_ptr[kNoAllocMaxDevices] = {};
std::mutex g_xor_scratch_mutex;

int xor_scratch_for_device(int dev, double **out) {
  std::lock_guard<std::mutex> lock(g_xor_scratch_mutex);
  if (!g_xor_scratch_ptr[dev]) {
    void *p = nullptr;
    if (cudaGetSymbolAddress(&p, g_xor_scratch) != cudaSuccess || !p) {
      cudaGetLastError();
      return VO_ECUDA;
    }
    g_xor_scratch_ptr[dev] = static_cast<double *>(p);
  }
  *out = g_xor_scratch_ptr[dev];
  return VO_OK;
}

}  // namespace
}  // namespace vo

extern "C" int vo_xor_volume_noalloc(const vo_grid *grid, const int32_t *offs_a, const double *z_a,
                                     const int32_t *offs_b, const double *z_b, void *stream, double *volume) {
  using namespace vo;
  if (!grid || grid->nx <= 0 || grid->ny <= 0 || !volume) return VO_EINVAL;
  const int64_t ncols = (int64_t)grid->nx * grid->ny;
  if (ncols > (int64_t)kNoAllocMaxBlocks * kThreads) return VO_ERANGE;  // beyond the fixed scratch
  if (!offs_a || !offs_b || !z_a || !z_b) return VO_EINVAL;
  int dev = -1;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kNoAllocMaxDevices) {
    cudaGetLastError();
    return VO_ENODEV;
  }
  cudaStream_t st = static_cast<cudaStream_t>(stream);
  if (st) {  // the scratch address below is the current device's: the stream must run there
    int sdev = -1;
    if (cudaStreamGetDevice(st, &sdev) != cudaSuccess) {
      cudaGetLastError();
      return VO_EINVAL;
    }
    if (sdev != dev) return VO_EINVAL;
  }
  double *scratch = nullptr;
  int rc = xor_scratch_for_device(dev, &scratch);
  if (rc) return rc;
  const int nblk = (int)((ncols + kThreads - 1) / kThreads);
  // Every partial sum the reduction reads is written by this call's first
  // kernel, and the result slot by the second. The result slot is first set
  // to a NaN pattern (all bytes 0xff), so a reduction that did not run can
  // never hand back the previous call's volume.
  if (cudaMemsetAsync(scratch + kNoAllocMaxBlocks, 0xff, sizeof(double), st) != cudaSuccess) {
    cudaGetLastError();
    return VO_ECUDA;
  }
  k_xor<<<nblk, kThreads, 0, st>>>((int)ncols, offs_a, reinterpret_cast<const double2 *>(z_a), offs_b,
                                   reinterpret_cast<const double2 *>(z_b), scratch);
  if (cudaGetLastError() != cudaSuccess) return VO_ECUDA;
  k_sum<<<1, kThreads, 0, st>>>(scratch, nblk, scratch + kNoAllocMaxBlocks);
  if (cudaGetLastError() != cudaSuccess) return VO_ECUDA;
  double h = 0;
  if (cudaMemcpyAsync(&h, scratch + kNoAllocMaxBlocks, sizeof(double), cudaMemcpyDeviceToHost, st) != cudaSuccess ||
      cudaStreamSynchronize(st) != cudaSuccess) {
    cudaGetLastError();
    return VO_ECUDA;
  }
  if (h != h) return VO_ECUDA;  // the sentinel survived: the reduction did not complete
  const double sp = grid->spacing;
  *volume = sp * sp * sp * h;
  return VO_OK;
}
