// Learned sizing for batched dilation (no reference counterpart).
//
// A small MLP predicts, for every 32 x 32 tile of output columns, the largest
// and the mean output segment count per column and the mean number of
// candidate intervals per column (the work), from statistics of the input
// columns (occupancy, mean / max segment count, a histogram of the gaps
// between consecutive segments in 8 log2 bins, coverage, the radius). The
// batched executor uses the predictions to size each tile's output slots and
// to order its work queue, which removes the exact count pass; any column that
// outgrows its predicted slot is detected exactly and its volume re-runs
// through the plain path, so results never depend on the prediction.
//
// Network: 16 inputs -> 64 ReLU -> 64 ReLU -> 4 outputs (3 used), weights in
// BF16 for inference, FP32 master copies, FP32 accumulation everywhere;
// trained on the GPU with the kernels below (squared error on log2 targets,
// under-prediction of the max count weighted 4x; Adam). Layout of the flat parameter vector: W1[16][64], b1[64],
// W2[64][64], b2[64], W3[64][4], b3[4] (row-major, [in][out]).
#include <cuda_bf16.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include "vo_internal.cuh"

namespace vo {
namespace {

constexpr int NF = VO_SIZER_FEATURES, NH = 64, NO = 4, NUSED = VO_SIZER_OUTPUTS;
constexpr int OFF_W1 = 0, OFF_B1 = OFF_W1 + NF * NH, OFF_W2 = OFF_B1 + NH, OFF_B2 = OFF_W2 + NH * NH,
              OFF_W3 = OFF_B2 + NH, OFF_B3 = OFF_W3 + NH * NO, NPARAM = OFF_B3 + NO;
constexpr int kTile = kSizerTile;

// ---------------------------------------------------------------- features

// One block per 32 x 32 tile of columns: occupancy, mean / max count, gap
// histogram (log2 bins: < 1, < 2, ..., < 64, >= 64 dexels), coverage.
__global__ void k_tile_stats(int nx, int ny, const int32_t *__restrict__ beg, const int32_t *__restrict__ end,
                             const double2 *__restrict__ z, float *stats) {
  __shared__ float s_occ, s_sum, s_len, s_hist[8];
  __shared__ int s_max;
  const int tiles_x = (nx + kTile - 1) / kTile;
  const int t = blockIdx.x;
  const int x0 = (t % tiles_x) * kTile, y0 = (t / tiles_x) * kTile;
  if (threadIdx.x == 0) {
    s_occ = s_sum = s_len = 0;
    s_max = 0;
    for (int b = 0; b < 8; ++b) s_hist[b] = 0;
  }
  __syncthreads();
  float occ = 0, sum = 0, len = 0, hist[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  int mx = 0;
  for (int i = threadIdx.x; i < kTile * kTile; i += blockDim.x) {
    const int x = x0 + i % kTile, y = y0 + i / kTile;
    if (x >= nx || y >= ny) continue;
    const int c = x + nx * y;
    const int k0 = beg[c], k1 = end[c], n = k1 - k0;
    occ += n > 0;
    sum += n;
    mx = max(mx, n);
    for (int k = k0; k < k1; ++k) {
      const double2 s = z[k];
      len += (float)(s.y - s.x);
      if (k > k0) {
        const float gap = (float)(s.x - z[k - 1].y);
        int b = gap < 1.f ? 0 : min(7, 1 + (int)floorf(log2f(gap)));
        hist[b] += 1;
      }
    }
  }
  atomicAdd(&s_occ, occ);
  atomicAdd(&s_sum, sum);
  atomicAdd(&s_len, len);
  atomicMax(&s_max, mx);
  for (int b = 0; b < 8; ++b) atomicAdd(&s_hist[b], hist[b]);
  __syncthreads();
  if (threadIdx.x == 0) {
    const int w = min(kTile, nx - x0), h = min(kTile, ny - y0);
    const float cols = (float)(w * h);
    float *f = stats + (size_t)t * NF;
    f[0] = s_occ / cols;
    f[1] = s_sum / cols;
    f[2] = (float)s_max;
    float gaps = 0;
    for (int b = 0; b < 8; ++b) gaps += s_hist[b];
    for (int b = 0; b < 8; ++b) f[3 + b] = gaps > 0 ? s_hist[b] / gaps : 0.f;
    f[11] = s_len / cols / 64.f;
  }
}

// Final features: log-scaled counts, the 3 x 3 tile neighbourhood mean count
// (the dilation reaches across tiles) and the radius terms.
__global__ void k_tile_features(int tiles_x, int tiles_y, float radius, float npairs, const float *stats,
                                float *feats) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= tiles_x * tiles_y) return;
  const int tx = t % tiles_x, ty = t / tiles_x;
  const float *s = stats + (size_t)t * NF;
  float nb = 0;
  int cnt = 0;
  for (int dy = -1; dy <= 1; ++dy)
    for (int dx = -1; dx <= 1; ++dx) {
      const int ux = tx + dx, uy = ty + dy;
      if (ux < 0 || uy < 0 || ux >= tiles_x || uy >= tiles_y) continue;
      nb += stats[(size_t)(ux + tiles_x * uy) * NF + 1];
      ++cnt;
    }
  float *f = feats + (size_t)t * NF;
  f[0] = s[0];
  f[1] = log2f(1.f + s[1]);
  f[2] = log2f(1.f + s[2]);
  for (int b = 0; b < 8; ++b) f[3 + b] = s[3 + b];
  f[11] = s[11];
  f[12] = log2f(1.f + nb / (float)max(cnt, 1));
  f[13] = radius / 64.f;
  f[14] = log2f(1.f + npairs) / 12.f;
  f[15] = 1.f;
}

// Per column: output count (from a result) and candidate count (sum over the
// alive (|dx|, |dy|) pairs of the source columns' segment counts).
__global__ void k_tile_targets(int nx, int ny, const int32_t *__restrict__ ibeg, const int32_t *__restrict__ iend,
                               const int32_t *__restrict__ ooffs, const int2 *__restrict__ pairs, int npairs,
                               float *targets) {
  __shared__ float s_mean, s_work;
  __shared__ int s_max;
  const int tiles_x = (nx + kTile - 1) / kTile;
  const int t = blockIdx.x;
  const int x0 = (t % tiles_x) * kTile, y0 = (t / tiles_x) * kTile;
  if (threadIdx.x == 0) {
    s_mean = s_work = 0;
    s_max = 0;
  }
  __syncthreads();
  float mean = 0, work = 0;
  int mx = 0;
  for (int i = threadIdx.x; i < kTile * kTile; i += blockDim.x) {
    const int x = x0 + i % kTile, y = y0 + i / kTile;
    if (x >= nx || y >= ny) continue;
    const int c = x + nx * y;
    const int n = ooffs[c + 1] - ooffs[c];
    mean += n;
    mx = max(mx, n);
    int wk = 0;
    for (int p = 0; p < npairs; ++p) {
      const int a = pairs[p].x, d = pairs[p].y;
      for (int s = 0; s < 4; ++s) {
        if (((s & 1) && a == 0) || ((s & 2) && d == 0)) continue;
        const int xs = (s & 1) ? x + a : x - a, ys = (s & 2) ? y + d : y - d;
        if (xs < 0 || xs >= nx || ys < 0 || ys >= ny) continue;
        const int cs = xs + nx * ys;
        wk += iend[cs] - ibeg[cs];
      }
    }
    work += (float)wk;
  }
  atomicAdd(&s_mean, mean);
  atomicAdd(&s_work, work);
  atomicMax(&s_max, mx);
  __syncthreads();
  if (threadIdx.x == 0) {
    const int w = min(kTile, nx - x0), h = min(kTile, ny - y0);
    const float cols = (float)(w * h);
    float *o = targets + (size_t)t * NUSED;
    o[0] = log2f(1.f + (float)s_max);
    o[1] = log2f(1.f + s_mean / cols);
    o[2] = log2f(1.f + s_work / cols);
  }
}

// ---------------------------------------------------------------- network

// Forward pass, one sample per thread; BF16 weights staged in shared memory
// as FP32, FP32 accumulation. h1 / h2 (post-ReLU) are kept for training.
__global__ void k_mlp_forward(const float *__restrict__ X, int n, const __nv_bfloat16 *__restrict__ w,
                              float *__restrict__ out, float *__restrict__ h1s, float *__restrict__ h2s) {
  __shared__ float sw[NPARAM];
  for (int i = threadIdx.x; i < NPARAM; i += blockDim.x) sw[i] = __bfloat162float(w[i]);
  __syncthreads();
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= n) return;
  float x[NF], h1[NH];
  for (int i = 0; i < NF; ++i) x[i] = X[(size_t)s * NF + i];
  for (int j = 0; j < NH; ++j) {
    float a = sw[OFF_B1 + j];
    for (int i = 0; i < NF; ++i) a += x[i] * sw[OFF_W1 + i * NH + j];
    h1[j] = fmaxf(a, 0.f);
    if (h1s) h1s[(size_t)s * NH + j] = h1[j];
  }
  float o[NO];
  for (int k = 0; k < NO; ++k) o[k] = sw[OFF_B3 + k];
  for (int j = 0; j < NH; ++j) {
    float a = sw[OFF_B2 + j];
    for (int i = 0; i < NH; ++i) a += h1[i] * sw[OFF_W2 + i * NH + j];
    const float h = fmaxf(a, 0.f);
    if (h2s) h2s[(size_t)s * NH + j] = h;
    for (int k = 0; k < NO; ++k) o[k] += h * sw[OFF_W3 + j * NO + k];
  }
  for (int k = 0; k < NO; ++k) out[(size_t)s * NO + k] = o[k];
}

// Backward through the activations: dz2 = (dout W3^T) * [h2 > 0],
// dz1 = (dz2 W2^T) * [h1 > 0], with dout = 2 w (out - target) / (n * NUSED)
// on the used outputs. The loss is the weighted squared error with w =
// kUnderWeight where the max-count output is below its target (slots sized
// too small cost spills and re-runs, too large only memory), else 1.
constexpr float kUnderWeight = 4.f;
__global__ void k_mlp_backward_act(const float *__restrict__ out, const float *__restrict__ tgt, int n,
                                   const __nv_bfloat16 *__restrict__ w, const float *__restrict__ h1s,
                                   const float *__restrict__ h2s, float *__restrict__ dout, float *__restrict__ dz2,
                                   float *__restrict__ dz1, float *loss) {
  __shared__ float sw[NPARAM];
  for (int i = threadIdx.x; i < NPARAM; i += blockDim.x) sw[i] = __bfloat162float(w[i]);
  __syncthreads();
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  float l = 0;
  if (s < n) {
    float go[NO];
    for (int k = 0; k < NO; ++k) {
      const float e = k < NUSED ? out[(size_t)s * NO + k] - tgt[(size_t)s * NUSED + k] : 0.f;
      const float wgt = (k == 0 && e < 0.f) ? kUnderWeight : 1.f;
      l += wgt * e * e;
      go[k] = 2.f * wgt * e / (float)(n * NUSED);
      dout[(size_t)s * NO + k] = go[k];
    }
    float g2[NH];
    for (int j = 0; j < NH; ++j) {
      float a = 0;
      for (int k = 0; k < NO; ++k) a += go[k] * sw[OFF_W3 + j * NO + k];
      g2[j] = h2s[(size_t)s * NH + j] > 0.f ? a : 0.f;
      dz2[(size_t)s * NH + j] = g2[j];
    }
    for (int i = 0; i < NH; ++i) {
      float a = 0;
      for (int j = 0; j < NH; ++j) a += g2[j] * sw[OFF_W2 + i * NH + j];
      dz1[(size_t)s * NH + i] = h1s[(size_t)s * NH + i] > 0.f ? a : 0.f;
    }
  }
  for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
  if ((threadIdx.x & 31) == 0) atomicAdd(loss, l / (float)(n * NUSED));
}

// Weight gradients as reductions over the samples, dW[i][j] = sum_s A[s][i] *
// G[s][j] and db[j] = sum_s G[s][j]: one thread per parameter and chunk of
// kGradChunk samples writes a partial sum, and k_grad_sum adds the chunks in
// order (deterministic).
constexpr int kGradChunk = 512;

__global__ void k_mlp_wgrad(const float *__restrict__ X, const float *__restrict__ h1s,
                            const float *__restrict__ h2s, const float *__restrict__ dout,
                            const float *__restrict__ dz2, const float *__restrict__ dz1, int n,
                            float *__restrict__ part) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= NPARAM) return;
  const float *A = nullptr, *G = nullptr;
  int ai = -1, gj, an = 0, gn;
  if (p < OFF_B1) {
    A = X, an = NF, ai = p / NH, G = dz1, gn = NH, gj = p % NH;
  } else if (p < OFF_W2) {
    G = dz1, gn = NH, gj = p - OFF_B1;
  } else if (p < OFF_B2) {
    A = h1s, an = NH, ai = (p - OFF_W2) / NH, G = dz2, gn = NH, gj = (p - OFF_W2) % NH;
  } else if (p < OFF_W3) {
    G = dz2, gn = NH, gj = p - OFF_B2;
  } else if (p < OFF_B3) {
    A = h2s, an = NH, ai = (p - OFF_W3) / NO, G = dout, gn = NO, gj = (p - OFF_W3) % NO;
  } else {
    G = dout, gn = NO, gj = p - OFF_B3;
  }
  const int s0 = blockIdx.y * kGradChunk, s1 = min(n, s0 + kGradChunk);
  float acc = 0;
  for (int s = s0; s < s1; ++s) acc += (A ? A[(size_t)s * an + ai] : 1.f) * G[(size_t)s * gn + gj];
  part[(size_t)blockIdx.y * NPARAM + p] = acc;
}

__global__ void k_grad_sum(const float *__restrict__ part, int nchunks, float *__restrict__ grad) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= NPARAM) return;
  float acc = 0;
  for (int c = 0; c < nchunks; ++c) acc += part[(size_t)c * NPARAM + p];
  grad[p] = acc;
}

__global__ void k_adam(float *__restrict__ wm, const float *__restrict__ g, float *__restrict__ m,
                       float *__restrict__ v, __nv_bfloat16 *__restrict__ wb, float lr, float b1, float b2,
                       float c1, float c2) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= NPARAM) return;
  m[p] = b1 * m[p] + (1.f - b1) * g[p];
  v[p] = b2 * v[p] + (1.f - b2) * g[p] * g[p];
  const float mh = m[p] / c1, vh = v[p] / c2;
  wm[p] -= lr * mh / (sqrtf(vh) + 1e-8f);
  wb[p] = __float2bfloat16_rn(wm[p]);
}

__global__ void k_to_bf16(const float *__restrict__ wm, __nv_bfloat16 *__restrict__ wb) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p < NPARAM) wb[p] = __float2bfloat16_rn(wm[p]);
}

}  // namespace
}  // namespace vo

struct vo_sizer {
  float *wm = nullptr;        // FP32 master parameters
  __nv_bfloat16 *wb = nullptr;  // BF16 parameters used by the forward pass
  float *m = nullptr, *v = nullptr, *grad = nullptr;
  int step = 0;
};

using namespace vo;

namespace {

struct Work {
  float *X = nullptr, *T = nullptr, *out = nullptr, *h1 = nullptr, *h2 = nullptr, *dout = nullptr, *dz2 = nullptr,
        *dz1 = nullptr, *loss = nullptr, *part = nullptr;
};

int nchunks(int n) { return (n + kGradChunk - 1) / kGradChunk; }

int work_alloc(vo_ctx *ctx, int n, bool train, Work &w) {
  int rc = dalloc(ctx, &w.X, (size_t)n * NF);
  if (!rc) rc = dalloc(ctx, &w.out, (size_t)n * NO);
  if (train) {
    if (!rc) rc = dalloc(ctx, &w.T, (size_t)n * NUSED);
    if (!rc) rc = dalloc(ctx, &w.h1, (size_t)n * NH);
    if (!rc) rc = dalloc(ctx, &w.h2, (size_t)n * NH);
    if (!rc) rc = dalloc(ctx, &w.dout, (size_t)n * NO);
    if (!rc) rc = dalloc(ctx, &w.dz2, (size_t)n * NH);
    if (!rc) rc = dalloc(ctx, &w.dz1, (size_t)n * NH);
    if (!rc) rc = dalloc(ctx, &w.loss, 1);
    if (!rc) rc = dalloc(ctx, &w.part, (size_t)nchunks(n) * NPARAM);
  }
  return rc;
}

void work_free(vo_ctx *ctx, Work &w) {
  for (float *p : {w.X, w.T, w.out, w.h1, w.h2, w.dout, w.dz2, w.dz1, w.loss, w.part}) dfree(ctx, p);
  w = Work();
}

// One forward + backward pass over the n samples in w; gradients in s->grad.
void grad_pass(vo_ctx *ctx, vo_sizer *s, int n, Work &w) {
  const int b = 128, g = (n + b - 1) / b;
  cudaMemsetAsync(w.loss, 0, sizeof(float), ctx->stream);
  k_mlp_forward<<<g, b, 0, ctx->stream>>>(w.X, n, s->wb, w.out, w.h1, w.h2);
  k_mlp_backward_act<<<g, b, 0, ctx->stream>>>(w.out, w.T, n, s->wb, w.h1, w.h2, w.dout, w.dz2, w.dz1, w.loss);
  k_mlp_wgrad<<<dim3((NPARAM + 127) / 128, nchunks(n)), 128, 0, ctx->stream>>>(w.X, w.h1, w.h2, w.dout, w.dz2,
                                                                                 w.dz1, n, w.part);
  k_grad_sum<<<(NPARAM + 127) / 128, 128, 0, ctx->stream>>>(w.part, nchunks(n), s->grad);
  ctx->launches += 4;
}

std::vector<int2> alive_pairs(const Tables &h) {
  std::vector<int2> pairs;
  for (int d = 0; d <= h.Dy; ++d)
    for (int a = 0; a <= h.Dx[d]; ++a) pairs.push_back(make_int2(a, d));
  return pairs;
}

}  // namespace

namespace vo {

// Features of the 32 x 32 tiles of a slot view into a device array (n tiles).
int sizer_features_device(vo_ctx *ctx, const SlotVol &in, double radius, float *feats, int *ntiles) {
  const vo_grid &g = in.grid;
  const int tx = (g.nx + kTile - 1) / kTile, ty = (g.ny + kTile - 1) / kTile;
  *ntiles = tx * ty;
  const DeviceTables *T = nullptr;
  int rc = get_tables(ctx, radius, std::max(g.nx, g.ny) + 2, &T);
  if (rc) return rc;
  float *stats = nullptr;
  rc = dalloc(ctx, &stats, (size_t)tx * ty * NF);
  if (rc) return rc;
  const float npairs = (float)alive_pairs(T->host).size();
  k_tile_stats<<<tx * ty, 256, 0, ctx->stream>>>(g.nx, g.ny, in.beg, in.end, in.z, stats);
  k_tile_features<<<(tx * ty + 127) / 128, 128, 0, ctx->stream>>>(tx, ty, (float)radius, npairs, stats, feats);
  ctx->launches += 2;
  dfree(ctx, stats);
  return VO_OK;
}

// Predictions (n x VO_SIZER_OUTPUTS-padded-to-4) for device features.
int sizer_predict_device(vo_ctx *ctx, const vo_sizer *s, const float *feats, int n, float *out4) {
  if (n <= 0) return VO_OK;
  k_mlp_forward<<<(n + 127) / 128, 128, 0, ctx->stream>>>(feats, n, s->wb, out4, nullptr, nullptr);
  ctx->launches += 1;
  return VO_OK;
}

}  // namespace vo

extern "C" {

int vo_sizer_create(vo_ctx *ctx, uint64_t seed, vo_sizer **out) {
  if (!ctx || !out) return VO_EINVAL;
  *out = nullptr;
  vo_sizer *s = new vo_sizer();
  int rc = dalloc(ctx, &s->wm, NPARAM);
  if (!rc) rc = dalloc(ctx, &s->wb, NPARAM);
  if (!rc) rc = dalloc(ctx, &s->m, NPARAM);
  if (!rc) rc = dalloc(ctx, &s->v, NPARAM);
  if (!rc) rc = dalloc(ctx, &s->grad, NPARAM);
  if (rc) {
    vo_sizer_destroy(ctx, s);
    return rc;
  }
  // He-uniform initialisation from a splitmix64 stream, biases zero.
  std::vector<float> w(NPARAM, 0.f);
  uint64_t st = seed;
  auto uni = [&]() {
    uint64_t z = (st += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (double)(z >> 11) * (1.0 / 9007199254740992.0);
  };
  auto fill = [&](int off, int fan_in, int cnt) {
    const double lim = std::sqrt(6.0 / fan_in);
    for (int i = 0; i < cnt; ++i) w[off + i] = (float)((2 * uni() - 1) * lim);
  };
  fill(OFF_W1, NF, NF * NH);
  fill(OFF_W2, NH, NH * NH);
  fill(OFF_W3, NH, NH * NO);
  rc = vo_sizer_set_params(ctx, s, w.data(), NPARAM);
  if (rc) {
    vo_sizer_destroy(ctx, s);
    return rc;
  }
  *out = s;
  return VO_OK;
}

void vo_sizer_destroy(vo_ctx *ctx, vo_sizer *s) {
  if (!ctx || !s) return;
  if (ctx->sizer == s) ctx->sizer = nullptr;
  dfree(ctx, s->wm);
  dfree(ctx, s->wb);
  dfree(ctx, s->m);
  dfree(ctx, s->v);
  dfree(ctx, s->grad);
  cudaStreamSynchronize(ctx->stream);
  delete s;
}

int vo_sizer_num_params(void) { return NPARAM; }

int vo_sizer_set_params(vo_ctx *ctx, vo_sizer *s, const float *params, int count) {
  if (!ctx || !s || !params || count != NPARAM) return VO_EINVAL;
  VO_CK(ctx, cudaMemcpyAsync(s->wm, params, sizeof(float) * NPARAM, cudaMemcpyHostToDevice, ctx->stream));
  cudaMemsetAsync(s->m, 0, sizeof(float) * NPARAM, ctx->stream);
  cudaMemsetAsync(s->v, 0, sizeof(float) * NPARAM, ctx->stream);
  k_to_bf16<<<(NPARAM + 127) / 128, 128, 0, ctx->stream>>>(s->wm, s->wb);
  s->step = 0;
  VO_CK(ctx, cudaStreamSynchronize(ctx->stream));
  return VO_OK;
}

int vo_sizer_get_params(vo_ctx *ctx, const vo_sizer *s, float *params, int count) {
  if (!ctx || !s || !params || count != NPARAM) return VO_EINVAL;
  VO_CK(ctx, cudaMemcpyAsync(params, s->wm, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost, ctx->stream));
  VO_CK(ctx, cudaStreamSynchronize(ctx->stream));
  return VO_OK;
}

int vo_sizer_tile_features(vo_ctx *ctx, const vo_volume *v, double radius, float *feats, int *ntiles) {
  if (!ctx || !v || !ntiles) return VO_EINVAL;
  vol_wait(ctx, v);
  const int tx = (v->grid.nx + kTile - 1) / kTile, ty = (v->grid.ny + kTile - 1) / kTile;
  if (!feats) {
    *ntiles = tx * ty;
    return VO_OK;
  }
  float *d = nullptr;
  int rc = dalloc(ctx, &d, (size_t)tx * ty * NF);
  if (rc) return rc;
  int n = 0;
  rc = sizer_features_device(ctx, slot_view(v, 0), radius, d, &n);
  if (!rc) cudaMemcpyAsync(feats, d, sizeof(float) * n * NF, cudaMemcpyDeviceToHost, ctx->stream);
  dfree(ctx, d);
  if (rc) return rc;
  VO_CK(ctx, cudaStreamSynchronize(ctx->stream));
  *ntiles = n;
  return VO_OK;
}

int vo_sizer_tile_targets(vo_ctx *ctx, const vo_volume *in, const vo_volume *result, double radius, float *targets,
                          int *ntiles) {
  if (!ctx || !in || !result || !targets || !ntiles) return VO_EINVAL;
  if (in->grid.nx != result->grid.nx || in->grid.ny != result->grid.ny) return VO_EINVAL;
  vol_wait(ctx, in);
  vol_wait(ctx, result);
  const int nx = in->grid.nx, ny = in->grid.ny;
  const int tx = (nx + kTile - 1) / kTile, ty = (ny + kTile - 1) / kTile;
  const DeviceTables *T = nullptr;
  int rc = get_tables(ctx, radius, std::max(nx, ny) + 2, &T);
  if (rc) return rc;
  const std::vector<int2> pairs = alive_pairs(T->host);
  int2 *dp = nullptr;
  float *dt = nullptr;
  rc = dalloc(ctx, &dp, pairs.size());
  if (!rc) rc = dalloc(ctx, &dt, (size_t)tx * ty * NUSED);
  if (!rc) {
    cudaMemcpyAsync(dp, pairs.data(), sizeof(int2) * pairs.size(), cudaMemcpyHostToDevice, ctx->stream);
    k_tile_targets<<<tx * ty, 256, 0, ctx->stream>>>(nx, ny, in->offs, in->offs + 1, result->offs, dp,
                                                     (int)pairs.size(), dt);
    cudaMemcpyAsync(targets, dt, sizeof(float) * tx * ty * NUSED, cudaMemcpyDeviceToHost, ctx->stream);
  }
  dfree(ctx, dp);
  dfree(ctx, dt);
  if (rc) return rc;
  VO_CK(ctx, cudaStreamSynchronize(ctx->stream));
  *ntiles = tx * ty;
  return VO_OK;
}

int vo_sizer_forward(vo_ctx *ctx, const vo_sizer *s, const float *feats, int n, float *pred) {
  if (!ctx || !s || !feats || !pred || n < 0) return VO_EINVAL;
  if (n == 0) return VO_OK;
  Work w;
  int rc = work_alloc(ctx, n, false, w);
  if (!rc) {
    cudaMemcpyAsync(w.X, feats, sizeof(float) * n * NF, cudaMemcpyHostToDevice, ctx->stream);
    k_mlp_forward<<<(n + 127) / 128, 128, 0, ctx->stream>>>(w.X, n, s->wb, w.out, nullptr, nullptr);
    std::vector<float> o((size_t)n * NO);
    cudaMemcpyAsync(o.data(), w.out, sizeof(float) * n * NO, cudaMemcpyDeviceToHost, ctx->stream);
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) rc = cuda_error(ctx, e, "sizer forward");
    for (int i = 0; i < n && !rc; ++i)
      for (int k = 0; k < NUSED; ++k) pred[(size_t)i * NUSED + k] = o[(size_t)i * NO + k];
  }
  work_free(ctx, w);
  return rc;
}

int vo_sizer_gradients(vo_ctx *ctx, vo_sizer *s, const float *feats, const float *targets, int n, float *grads,
                       float *loss) {
  if (!ctx || !s || !feats || !targets || !grads || n <= 0) return VO_EINVAL;
  Work w;
  int rc = work_alloc(ctx, n, true, w);
  if (!rc) {
    cudaMemcpyAsync(w.X, feats, sizeof(float) * n * NF, cudaMemcpyHostToDevice, ctx->stream);
    cudaMemcpyAsync(w.T, targets, sizeof(float) * n * NUSED, cudaMemcpyHostToDevice, ctx->stream);
    grad_pass(ctx, s, n, w);
    cudaMemcpyAsync(grads, s->grad, sizeof(float) * NPARAM, cudaMemcpyDeviceToHost, ctx->stream);
    float l = 0;
    cudaMemcpyAsync(&l, w.loss, sizeof(float), cudaMemcpyDeviceToHost, ctx->stream);
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) rc = cuda_error(ctx, e, "sizer gradients");
    if (loss) *loss = l;
  }
  work_free(ctx, w);
  return rc;
}

int vo_sizer_train(vo_ctx *ctx, vo_sizer *s, const float *feats, const float *targets, int n, int steps, float lr,
                   float *final_loss) {
  if (!ctx || !s || !feats || !targets || n <= 0 || steps < 0) return VO_EINVAL;
  Work w;
  int rc = work_alloc(ctx, n, true, w);
  float l = 0;
  if (!rc) {
    cudaMemcpyAsync(w.X, feats, sizeof(float) * n * NF, cudaMemcpyHostToDevice, ctx->stream);
    cudaMemcpyAsync(w.T, targets, sizeof(float) * n * NUSED, cudaMemcpyHostToDevice, ctx->stream);
    for (int it = 0; it < steps; ++it) {
      grad_pass(ctx, s, n, w);
      ++s->step;
      const float b1 = 0.9f, b2 = 0.999f;
      k_adam<<<(NPARAM + 127) / 128, 128, 0, ctx->stream>>>(s->wm, s->grad, s->m, s->v, s->wb, lr, b1, b2,
                                                            1.f - std::pow(b1, (float)s->step),
                                                            1.f - std::pow(b2, (float)s->step));
      ctx->launches += 1;
    }
    // loss of the final parameters
    grad_pass(ctx, s, n, w);
    cudaMemcpyAsync(&l, w.loss, sizeof(float), cudaMemcpyDeviceToHost, ctx->stream);
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) rc = cuda_error(ctx, e, "sizer train");
  }
  work_free(ctx, w);
  if (final_loss) *final_loss = l;
  return rc;
}

int vo_set_sizer(vo_ctx *ctx, vo_sizer *s) {
  if (!ctx) return VO_EINVAL;
  ctx->sizer = s;
  return VO_OK;
}

}  // extern "C"
