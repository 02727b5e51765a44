// C ABI of libvoroffset_gpu.so (include/voroffset_gpu.h): contexts, device
// volumes, radius tables and operation chaining. The kernels live in
// vo_morph.cu (morphology), vo_dexel.cu (ray rasterisation) and vo_reduce.cu
// (xor volume).
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <new>
#include <thread>
#include <vector>

#include "vo_internal.cuh"

namespace vo {

int set_error(vo_ctx *ctx, int code, const std::string &msg) {
  if (ctx) ctx->err = msg;
  return code;
}

int cuda_error(vo_ctx *ctx, cudaError_t e, const char *where) {
  std::string m = std::string(where) + ": " + cudaGetErrorString(e);
  cudaGetLastError();  // clear a sticky-free error so the context stays usable
  return set_error(ctx, VO_ECUDA, m);
}

void dfree(vo_ctx *ctx, void *p) {
  if (p) cudaFreeAsync(p, ctx->stream);
}

// FP32 lower bound of a - b as the device computes it
// (__double2float_rd(__dsub_rd(a, b))): the FP64 difference rounded to
// nearest is moved down one ulp when its TwoSum error is negative, then the
// FP32 conversion rounded to nearest is moved down when it lies above.
static float sub_rd_f32(double a, double b) {
  const double c = -b, s = a + c, bb = s - a;
  const double e = (a - (s - bb)) + (c - bb);
  const double sd = e < 0.0 ? std::nextafter(s, -INFINITY) : s;
  float f = (float)sd;
  if ((double)f > sd) f = std::nextafterf(f, -INFINITY);
  return f;
}

// Dominance level thresholds for the tables' radius: t[0] = 0 and t[l] for
// l >= 1 the value at quantile (l - 1/2) / (kDomLevels - 1) of the sorted
// growths of H over one lattice step (x steps for a >= 1, y steps for
// d >= 1), each as the FP32 lower bound the device's pair records hold.
static void dom_levels(Tables &t) {
  std::vector<float> g;
  for (int d = 0; d <= t.Dy; ++d)
    for (int a = 0; a <= t.Dx[d]; ++a) {
      const double h = t.H[(size_t)d * t.W + a];
      if (a >= 1) g.push_back(sub_rd_f32(t.H[(size_t)d * t.W + a - 1], h));
      if (d >= 1) g.push_back(sub_rd_f32(t.H[(size_t)(d - 1) * t.W + a], h));
    }
  std::sort(g.begin(), g.end());
  t.dom.t[0] = 0.f;
  for (int l = 1; l < kDomLevels; ++l) {
    float v = 0.f;
    if (!g.empty()) {
      const double q = ((double)l - 0.5) / (double)(kDomLevels - 1);
      v = g[(size_t)std::floor(q * (double)(g.size() - 1) + 0.5)];
    }
    t.dom.t[l] = v > 0.f ? v : 0.f;
  }
}

// Host tables with the reference's expressions (compiled with
// -ffp-contract=off so a*b - c*d is never fused):
//   pass-1 radius (Voronoi2D.cpp:704-712): r = d==0 ? R : sqrt(R*R - dd*dd), dd = min(d, R)
//   pass-2 half width (SeparatePower2D.cpp:314): sqrt(r*r - dx*dx)
//   brute force (VoronoiBruteForce.cpp:41-52): sqrt(R*R - dx^2 - dy^2) inside the disc
//   expiry (Voronoi2D.cpp:619, SeparatePower2D.cpp:266): alive while floor(x_s + r) + 1 > i
int build_tables(double R, int kmax, Tables &t) {
  t = Tables();
  if (!(R >= 0.0) || R > 255.0) return VO_EINVAL;
  t.R = R;
  t.Dy = (int)std::floor(R);
  for (int k = 0; k < kmax; ++k)
    if ((int)std::floor((double)k + R) != k + t.Dy) return VO_ERADIUS;
  const int Dy = t.Dy;
  t.r1.resize(Dy + 1);
  t.Dx.resize(Dy + 1);
  for (int d = 0; d <= Dy; ++d) {
    if (d == 0) {
      t.r1[d] = R;
    } else {
      const double dd = (double)d < R ? (double)d : R;
      t.r1[d] = std::sqrt(R * R - dd * dd);
    }
    t.Dx[d] = (int)std::floor(t.r1[d]);
    for (int k = 0; k < kmax; ++k)
      if ((int)std::floor((double)k + t.r1[d]) != k + t.Dx[d]) return VO_ERADIUS;
  }
  t.W = t.Dx[0] + 1;
  t.H.assign((size_t)(Dy + 1) * t.W, NAN);
  t.Hf.assign(t.H.size(), NAN);
  for (int d = 0; d <= Dy; ++d)
    for (int dx = 0; dx <= t.Dx[d]; ++dx) {
      const double r = t.r1[d], x = (double)dx;
      t.H[(size_t)d * t.W + dx] = std::sqrt(r * r - x * x);
      t.Hf[(size_t)d * t.W + dx] = (float)t.H[(size_t)d * t.W + dx];
    }
  t.HB.assign((size_t)(Dy + 1) * (Dy + 1), NAN);
  for (int dy = 0; dy <= Dy; ++dy)
    for (int dx = 0; dx <= Dy; ++dx) {
      const double fx = (double)dx * dx, fy = (double)dy * dy;
      if (fx + fy <= R * R) t.HB[(size_t)dy * (Dy + 1) + dx] = std::sqrt(R * R - fx - fy);
    }
  dom_levels(t);
  return VO_OK;
}

int get_tables(vo_ctx *ctx, double R, int kmax, const DeviceTables **out) {
  for (DeviceTables *d : ctx->tables)
    if (d->R == R && d->kmax >= kmax) {
      *out = d;
      return VO_OK;
    }
  Tables h;
  int rc = build_tables(R, kmax, h);
  if (rc == VO_EINVAL) return set_error(ctx, rc, "radius must be in [0, 255] dexels");
  if (rc == VO_ERADIUS) {
    char b[160];
    std::snprintf(b, sizeof b,
                  "radius %.17g lies within rounding of a lattice distance; its reach would "
                  "depend on the column position",
                  R);
    return set_error(ctx, rc, b);
  }
  DeviceTables *d = new (std::nothrow) DeviceTables();
  if (!d) return set_error(ctx, VO_ENOMEM, "host allocation");
  d->R = R;
  d->kmax = kmax;
  d->host = h;
  cudaError_t e = cudaMalloc(&d->H, sizeof(double) * h.H.size());
  if (e == cudaSuccess) e = cudaMalloc(&d->Hf, sizeof(float) * h.Hf.size());
  if (e == cudaSuccess) e = cudaMalloc(&d->Dx, sizeof(int) * h.Dx.size());
  if (e == cudaSuccess) e = cudaMalloc(&d->HB, sizeof(double) * h.HB.size());
  if (e == cudaSuccess) e = cudaMalloc(&d->dH, sizeof(float) * 2 * h.H.size());
  if (e == cudaSuccess)
    e = cudaMemcpy(d->H, h.H.data(), sizeof(double) * h.H.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(d->Hf, h.Hf.data(), sizeof(float) * h.Hf.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(d->Dx, h.Dx.data(), sizeof(int) * h.Dx.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess)
    e = cudaMemcpy(d->HB, h.HB.data(), sizeof(double) * h.HB.size(), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    launch_dh_tables(ctx->stream, h.Dy, h.W, d->H, d->Dx, d->dH);
    e = cudaStreamSynchronize(ctx->stream);
  }
  if (e != cudaSuccess) {
    cudaFree(d->H);
    cudaFree(d->Hf);
    cudaFree(d->Dx);
    cudaFree(d->HB);
    cudaFree(d->dH);
    delete d;
    return cuda_error(ctx, e, "table upload");
  }
  if (ctx->tables.size() >= 16) {
    DeviceTables *old = ctx->tables.front();
    cudaFree(old->H);
    cudaFree(old->Hf);
    cudaFree(old->Dx);
    cudaFree(old->HB);
    cudaFree(old->dH);
    delete old;
    ctx->tables.erase(ctx->tables.begin());
  }
  ctx->tables.push_back(d);
  *out = d;
  return VO_OK;
}

void vol_wait(vo_ctx *ctx, const vo_volume *v) {
  if (ctx && v && v->ready) cudaStreamWaitEvent(ctx->stream, v->ready, 0);
}

int volume_alloc(vo_ctx *ctx, const vo_grid &g, int64_t nseg, vo_volume **out) {
  vo_volume *v = new (std::nothrow) vo_volume();
  if (!v) return set_error(ctx, VO_ENOMEM, "host allocation");
  v->grid = g;
  v->nseg = nseg;
  const size_t ncols = (size_t)g.nx * g.ny;
  int rc = dalloc(ctx, &v->offs, ncols + 1);
  if (!rc && nseg > 0) rc = dalloc(ctx, &v->z, (size_t)nseg);
  if (rc) {
    dfree(ctx, v->offs);
    delete v;
    return rc;
  }
  *out = v;
  return VO_OK;
}

}  // namespace vo

using namespace vo;

namespace {

// Whether offs[0..ncols] never decreases; large arrays are checked by a few
// host threads at once (the check runs while the upload's copies do).
bool offsets_monotone(const int32_t *offs, int64_t ncols) {
  auto scan = [offs](int64_t c0, int64_t c1) {
    int bad = 0;
    for (int64_t c = c0; c < c1; ++c) bad |= offs[c + 1] < offs[c];
    return bad == 0;
  };
  const unsigned hw = std::thread::hardware_concurrency();
  const int nt = ncols < (1 << 20) || hw < 2 ? 1 : (int)std::min(8u, hw);
  if (nt == 1) return scan(0, ncols);
  std::vector<char> ok(nt, 1);
  std::vector<std::thread> th;
  const int64_t per = (ncols + nt - 1) / nt;
  for (int t = 1; t < nt; ++t)
    th.emplace_back([&, t] { ok[t] = scan(std::min(ncols, t * per), std::min(ncols, (t + 1) * per)); });
  ok[0] = scan(0, std::min(ncols, per));
  for (std::thread &x : th) x.join();
  for (char v : ok)
    if (!v) return false;
  return true;
}

constexpr int64_t kCopyPiece = (64ll << 20) / 16;  // segments per asynchronous copy piece (64 MB)

bool grid_ok(const vo_grid *g) {
  return g && g->nx > 0 && g->ny > 0 && (int64_t)g->nx * g->ny < (1ll << 31) - 1 &&
         g->spacing > 0 && std::isfinite(g->spacing);
}

}  // namespace

extern "C" {

int vo_create(vo_ctx **out, int device) {
  if (!out) return VO_EINVAL;
  *out = nullptr;
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n <= 0) {
    cudaGetLastError();
    return VO_ENODEV;
  }
  if (device < 0 || device >= n) return VO_EINVAL;
  cudaDeviceProp p;
  if (cudaGetDeviceProperties(&p, device) != cudaSuccess) return VO_ENODEV;
  if (!(p.major == 10 && p.minor == 3)) return VO_ENODEV;  // built for sm_103a only
  vo_ctx *ctx = new (std::nothrow) vo_ctx();
  if (!ctx) return VO_ENOMEM;
  ctx->device = device;
  if (cudaSetDevice(device) != cudaSuccess ||
      cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaStreamCreateWithFlags(&ctx->copy_stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&ctx->ev_order, cudaEventDisableTiming) != cudaSuccess) {
    if (ctx->stream) cudaStreamDestroy(ctx->stream);
    if (ctx->copy_stream) cudaStreamDestroy(ctx->copy_stream);
    delete ctx;
    return VO_ECUDA;
  }
  for (auto &e : ctx->ev) cudaEventCreate(&e);
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
    uint64_t thr = UINT64_MAX;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &thr);
  }
  if (cudaMalloc(&ctx->d_flags, 16 * sizeof(int)) != cudaSuccess ||
      cudaMalloc(&ctx->d_total, 4 * sizeof(long long)) != cudaSuccess ||
      cudaMallocHost(&ctx->h_total, 4 * sizeof(long long)) != cudaSuccess) {
    vo_destroy(ctx);
    return VO_ENOMEM;
  }
  cudaMemset(ctx->d_flags, 0, 16 * sizeof(int));
  *out = ctx;
  return VO_OK;
}

void vo_destroy(vo_ctx *ctx) {
  if (!ctx) return;
  cudaSetDevice(ctx->device);
  if (ctx->copy_stream) cudaStreamSynchronize(ctx->copy_stream);
  if (ctx->stream) cudaStreamSynchronize(ctx->stream);
  for (DeviceTables *d : ctx->tables) {
    cudaFree(d->H);
    cudaFree(d->Hf);
    cudaFree(d->Dx);
    cudaFree(d->HB);
    cudaFree(d->dH);
    delete d;
  }
  for (auto &e : ctx->ev)
    if (e) cudaEventDestroy(e);
  cudaFree(ctx->d_flags);
  cudaFree(ctx->d_total);
  if (ctx->h_total) cudaFreeHost(ctx->h_total);
  if (ctx->ev_order) cudaEventDestroy(ctx->ev_order);
  if (ctx->copy_stream) cudaStreamDestroy(ctx->copy_stream);
  if (ctx->stream) cudaStreamDestroy(ctx->stream);
  delete ctx;
}

const char *vo_last_error(const vo_ctx *ctx) { return ctx ? ctx->err.c_str() : "no context"; }

void *vo_stream(vo_ctx *ctx) { return ctx ? (void *)ctx->stream : nullptr; }

int vo_sync(vo_ctx *ctx) {
  if (!ctx) return VO_EINVAL;
  VO_CK(ctx, cudaStreamSynchronize(ctx->copy_stream));
  VO_CK(ctx, cudaStreamSynchronize(ctx->stream));
  return VO_OK;
}

int vo_volume_upload(vo_ctx *ctx, const vo_grid *grid, const int32_t *offs, const double *z,
                     vo_volume **out) {
  if (!ctx || !out || !offs || !grid_ok(grid)) return set_error(ctx, VO_EINVAL, "upload: bad grid");
  *out = nullptr;
  const int64_t ncols = (int64_t)grid->nx * grid->ny;
  if (offs[0] != 0) return set_error(ctx, VO_EINVAL, "upload: offs[0] must be 0");
  const int64_t nseg = offs[ncols];
  if (nseg < 0) return set_error(ctx, VO_EINVAL, "upload: offsets must not decrease");
  if (nseg > 0 && !z) return set_error(ctx, VO_EINVAL, "upload: z is NULL");
  cudaSetDevice(ctx->device);
  vo_volume *v = nullptr;
  int rc = volume_alloc(ctx, *grid, nseg, &v);
  if (rc) return rc;
  // The copies are issued first; the offsets are validated on the host while
  // they run (the caller's z holds 2 * offs[ncols] values either way).
  cudaError_t e = cudaMemcpyAsync(v->offs, offs, sizeof(int32_t) * (ncols + 1),
                                  cudaMemcpyHostToDevice, ctx->stream);
  if (e == cudaSuccess && nseg > 0)
    e = cudaMemcpyAsync(v->z, z, sizeof(double) * 2 * nseg, cudaMemcpyHostToDevice, ctx->stream);
  const bool monotone = offsets_monotone(offs, ncols);
  if (e != cudaSuccess || !monotone) {
    cudaStreamSynchronize(ctx->stream);
    vo_volume_free(ctx, v);
    if (e != cudaSuccess) return cuda_error(ctx, e, "upload");
    return set_error(ctx, VO_EINVAL, "upload: offsets must not decrease");
  }
  *out = v;
  return VO_OK;
}

int vo_volume_upload_async(vo_ctx *ctx, const vo_grid *grid, const int32_t *offs, const double *z,
                           vo_volume **out) {
  if (!ctx || !out || !offs || !grid_ok(grid)) return set_error(ctx, VO_EINVAL, "upload: bad grid");
  *out = nullptr;
  const int64_t ncols = (int64_t)grid->nx * grid->ny;
  if (offs[0] != 0) return set_error(ctx, VO_EINVAL, "upload: offs[0] must be 0");
  const int64_t nseg = offs[ncols];
  if (nseg < 0) return set_error(ctx, VO_EINVAL, "upload: offsets must not decrease");
  if (nseg > 0 && !z) return set_error(ctx, VO_EINVAL, "upload: z is NULL");
  cudaSetDevice(ctx->device);
  vo_volume *v = nullptr;
  int rc = volume_alloc(ctx, *grid, nseg, &v);
  if (rc) return rc;
  // the memory is allocated in the context's stream order: the copy stream starts after that
  cudaError_t e = cudaEventCreateWithFlags(&v->ready, cudaEventDisableTiming);
  if (e == cudaSuccess) e = cudaEventRecord(ctx->ev_order, ctx->stream);
  if (e == cudaSuccess) e = cudaStreamWaitEvent(ctx->copy_stream, ctx->ev_order, 0);
  if (e == cudaSuccess)
    e = cudaMemcpyAsync(v->offs, offs, sizeof(int32_t) * (ncols + 1), cudaMemcpyHostToDevice, ctx->copy_stream);
  // in pieces of 64 MB, so that small copies of the compute stream can be scheduled between them
  // rather than behind one long transfer
  for (int64_t k = 0; e == cudaSuccess && k < nseg; k += kCopyPiece)
    e = cudaMemcpyAsync(v->z + k, z + 2 * k, sizeof(double) * 2 * std::min<int64_t>(kCopyPiece, nseg - k),
                        cudaMemcpyHostToDevice, ctx->copy_stream);
  if (e == cudaSuccess) e = cudaEventRecord(v->ready, ctx->copy_stream);
  const bool monotone = offsets_monotone(offs, ncols);
  if (e != cudaSuccess || !monotone) {
    cudaStreamSynchronize(ctx->copy_stream);
    vo_volume_free(ctx, v);
    if (e != cudaSuccess) return cuda_error(ctx, e, "upload_async");
    return set_error(ctx, VO_EINVAL, "upload: offsets must not decrease");
  }
  *out = v;
  return VO_OK;
}

int vo_volume_info(vo_ctx *ctx, const vo_volume *v, vo_grid *grid, int64_t *nseg) {
  if (!ctx || !v) return VO_EINVAL;
  if (grid) *grid = v->grid;
  if (nseg) *nseg = v->nseg;
  return VO_OK;
}

int vo_volume_download(vo_ctx *ctx, const vo_volume *v, int32_t *offs, double *z) {
  if (!ctx || !v || !offs || (v->nseg > 0 && !z)) return set_error(ctx, VO_EINVAL, "download: NULL buffer");
  cudaSetDevice(ctx->device);
  vol_wait(ctx, v);
  const int64_t ncols = (int64_t)v->grid.nx * v->grid.ny;
  VO_CK(ctx, cudaMemcpyAsync(offs, v->offs, sizeof(int32_t) * (ncols + 1), cudaMemcpyDeviceToHost,
                             ctx->stream));
  if (v->nseg > 0)
    VO_CK(ctx, cudaMemcpyAsync(z, v->z, sizeof(double) * 2 * v->nseg, cudaMemcpyDeviceToHost,
                               ctx->stream));
  VO_CK(ctx, cudaStreamSynchronize(ctx->stream));
  return VO_OK;
}

int vo_volume_download_async(vo_ctx *ctx, const vo_volume *v, int32_t *offs, double *z) {
  if (!ctx || !v || !offs || (v->nseg > 0 && !z)) return set_error(ctx, VO_EINVAL, "download: NULL buffer");
  cudaSetDevice(ctx->device);
  vol_wait(ctx, v);
  if (!v->copied) VO_CK(ctx, cudaEventCreateWithFlags(&v->copied, cudaEventDisableTiming));
  // the copies start once the context's stream has produced the volume
  VO_CK(ctx, cudaEventRecord(ctx->ev_order, ctx->stream));
  VO_CK(ctx, cudaStreamWaitEvent(ctx->copy_stream, ctx->ev_order, 0));
  const int64_t ncols = (int64_t)v->grid.nx * v->grid.ny;
  VO_CK(ctx, cudaMemcpyAsync(offs, v->offs, sizeof(int32_t) * (ncols + 1), cudaMemcpyDeviceToHost,
                             ctx->copy_stream));
  for (int64_t k = 0; k < v->nseg; k += kCopyPiece)
    VO_CK(ctx, cudaMemcpyAsync(z + 2 * k, v->z + k, sizeof(double) * 2 * std::min<int64_t>(kCopyPiece, v->nseg - k),
                               cudaMemcpyDeviceToHost, ctx->copy_stream));
  VO_CK(ctx, cudaEventRecord(v->copied, ctx->copy_stream));
  return VO_OK;
}

int vo_volume_device_ptrs(vo_ctx *ctx, const vo_volume *v, void **offs, void **z) {
  if (!ctx || !v) return VO_EINVAL;
  if (v->ready) cudaEventSynchronize(v->ready);  // the caller's own work may use another stream
  if (offs) *offs = v->offs;
  if (z) *z = v->z;
  return VO_OK;
}

void vo_volume_free(vo_ctx *ctx, vo_volume *v) {
  if (!ctx || !v) return;
  if (v->copied) {
    // downloaded asynchronously: freed in the copy stream's order, after the download and after the
    // work queued so far on the compute stream, which then need not wait for the download
    cudaEventRecord(ctx->ev_order, ctx->stream);
    cudaStreamWaitEvent(ctx->copy_stream, ctx->ev_order, 0);
    if (v->owns) {
      if (v->offs) cudaFreeAsync(v->offs, ctx->copy_stream);
      if (v->z) cudaFreeAsync(v->z, ctx->copy_stream);
    }
  } else {
    if (v->ready) cudaStreamWaitEvent(ctx->stream, v->ready, 0);  // after its upload
    if (v->owns) {
      dfree(ctx, v->offs);
      dfree(ctx, v->z);
    }
  }
  if (v->ready) cudaEventDestroy(v->ready);
  if (v->copied) cudaEventDestroy(v->copied);
  delete v;
}

int vo_morph(vo_ctx *ctx, int op, int method, double radius, const vo_volume *in, vo_volume **out,
             vo_timings *tm) {
  if (!ctx) return VO_EINVAL;
  if (!in || !out) return set_error(ctx, VO_EINVAL, "morph: NULL volume");
  if (op < VO_DILATION || op > VO_CLOSING) return set_error(ctx, VO_EINVAL, "morph: unknown op");
  if (method != VO_METHOD_SEPARABLE && method != VO_METHOD_BRUTE && method != VO_METHOD_FAST &&
      method != VO_METHOD_ENVELOPE)
    return set_error(ctx, VO_EINVAL, "morph: unknown method");
  if (!(radius >= 0) || radius > 255) return set_error(ctx, VO_EINVAL, "morph: radius must be in [0, 255]");
  cudaSetDevice(ctx->device);
  vol_wait(ctx, in);
  *out = nullptr;
  ctx->err.clear();
  ctx->launches = 0;
  ctx->ovf_cols = 0;
  vo_timings local;
  std::memset(&local, 0, sizeof local);
  vo_timings *t = tm ? tm : &local;
  std::memset(t, 0, sizeof *t);
  const auto t0 = std::chrono::steady_clock::now();
  vo_volume *tmp = nullptr;
  int rc;
  switch (op) {
    case VO_DILATION:
      rc = dilate(ctx, method, radius, in, out, t);
      break;
    case VO_EROSION:
      rc = erode(ctx, method, radius, in, out, t);
      break;
    case VO_OPENING:
      rc = erode(ctx, method, radius, in, &tmp, t);
      if (!rc) rc = dilate(ctx, method, radius, tmp, out, t);
      break;
    default:  // VO_CLOSING
      rc = dilate(ctx, method, radius, in, &tmp, t);
      if (!rc) rc = erode(ctx, method, radius, tmp, out, t);
      break;
  }
  if (tmp) vo_volume_free(ctx, tmp);
  if (!rc) {
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) rc = cuda_error(ctx, e, "morph");
  }
  t->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  t->in_segments = in->nseg;
  t->out_segments = (!rc && *out) ? (*out)->nseg : 0;
  t->kernel_launches = ctx->launches;
  t->overflow_columns = ctx->ovf_cols;
  if (rc && *out) {
    vo_volume_free(ctx, *out);
    *out = nullptr;
  }
  return rc;
}

int vo_morph_batched(vo_ctx *ctx, int n, const int *ops, const double *radii, int method,
                     const vo_volume *const *ins, vo_volume **outs, vo_timings *tm) {
  if (!ctx || n < 0 || (n > 0 && (!ops || !radii || !ins || !outs))) return VO_EINVAL;
  for (int i = 0; i < n; ++i) outs[i] = nullptr;
  if (method == VO_METHOD_FAST) {
    for (int i = 0; i < n; ++i) {
      if (!ins[i] || ops[i] < VO_DILATION || ops[i] > VO_CLOSING || !(radii[i] >= 0) || radii[i] > 255)
        return set_error(ctx, VO_EINVAL, "morph_batched: bad volume, op or radius");
    }
    cudaSetDevice(ctx->device);
    for (int i = 0; i < n; ++i) vol_wait(ctx, ins[i]);
    ctx->err.clear();
    ctx->launches = 0;
    return morph_batched_fast(ctx, n, ops, radii, ins, outs, tm);
  }
  vo_timings acc;
  std::memset(&acc, 0, sizeof acc);
  for (int i = 0; i < n; ++i) {
    vo_timings t;
    int rc = vo_morph(ctx, ops[i], method, radii[i], ins[i], &outs[i], &t);
    if (rc) {
      for (int j = 0; j < i; ++j) {
        vo_volume_free(ctx, outs[j]);
        outs[j] = nullptr;
      }
      return rc;
    }
    acc.total_ms += t.total_ms;
    acc.pass1_ms += t.pass1_ms;
    acc.pass2_ms += t.pass2_ms;
    acc.in_segments += t.in_segments;
    acc.mid_pieces += t.mid_pieces;
    acc.out_segments += t.out_segments;
    acc.kernel_launches += t.kernel_launches;
    acc.overflow_columns += t.overflow_columns;
  }
  if (tm) *tm = acc;
  return VO_OK;
}

}  // extern "C"
