// Batch plans: many volumes of uneven grids, radii and operations (including
// the erosion -> dilation chains of opening and closing) executed as one
// CUDA graph, with every dilation of a round in one persistent launch
// (VO_METHOD_FAST only; no reference counterpart beyond calling
// VoronoiMorpho::dilation / erosion once per volume, Voronoi.h:18-29, and the
// chaining of offset3d.cpp:124-133).
//
// Planning (vo_batch_create) walks the operation chains round by round. Every
// device step is recorded as a launch closure; the plan runs the closures
// eagerly only when a later step needs the data (the input features of a
// learned-sized dilation, the capacity of a complement of a dilation result).
// Per dilation:
//   * output slots: with a sizer attached, every 32 x 32 tile of output
//     columns gets the capacity the network predicts for its largest union
//     (plus a margin, at most kUnionCapMid); without one, every column gets
//     kUnionCap slots; either way a spill region takes the columns that need
//     more (unions beyond kUnionCap are computed by the second-tier kernel);
//   * work queue: dilations in decreasing predicted total work (the network's
//     per-tile candidate counts, or the mean cost per column), the tiles of
//     each in bands of 512 columns, all rows of a band before the next;
//   * union capacity of the main kernel (24 or 32; 48 or 64 for dense inputs,
//     more than 10 segments per column on average), block shape (1, 2 or 4
//     warps of 8 x 4 columns per block), register budget and launch mode,
//     chosen by the autotuner below and cached per context.
// Then the closures are captured into one graph. vo_batch_run replays it and
// re-runs, through the single-volume path, every volume whose overflow flag
// is set (a union larger than its slot with the spill region exhausted, or
// beyond the FP64 third tier's list), so results never depend on the
// predictions.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstring>
#include <functional>
#include <memory>
#include <vector>

#include "vo_internal.cuh"

using namespace vo;

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

using Launch = std::function<void(cudaStream_t)>;

struct DilPlan {
  int vol = 0;
  SlotVol in, out;
  const DeviceTables *T = nullptr;
  float *zf = nullptr, *E = nullptr;
  int4 *col = nullptr;
  float4 *prec = nullptr;
  unsigned *dmask = nullptr;
  int mask_bits = 32;
  unsigned int *maxbits = nullptr;
  int2 *pairs = nullptr;
  int *mid_list = nullptr, *mid_count = nullptr;
  int *big_list = nullptr, *big_count = nullptr;
  int npairs = 0;
  int32_t *tcap = nullptr, *toff = nullptr;
  int tiles32_x = 0, tiles32 = 0;
  std::vector<float> tile_work;  // predicted candidates per column of each sizing tile
  int spill_base = 0, spill_cap = 0;
  int *spill_used = nullptr;
  double cost = 0;  // mean candidates per column (no sizer)
  int64_t slot_entries = 0;
};

constexpr int kTuneShapes[] = {1, 2, 4};
constexpr int kTuneRegs[] = {64, 80};

}  // namespace

struct vo_batch {
  int n = 0;
  std::vector<int> ops;
  std::vector<double> radii;
  std::vector<const vo_volume *> ins;
  std::vector<vo_volume *> normalized;  // owned copies of inputs with inverted pairs rewritten
  std::vector<Launch> rec;             // recorded device steps, in order
  size_t executed = 0;                 // closures already run eagerly
  int kernels = 0;                     // kernel launches per replay
  std::vector<void *> dmem;            // device allocations of the plan
  std::vector<SlotVol> owned;
  std::vector<SlotVol> finals;
  int *d_flags = nullptr;  // [v]: overflow flags of volume v, [n]: complement slot overflow
  double2 *big_scratch = nullptr;  // working lists of the FP64 third tier
  struct Spill {
    int *used;
    int cap, round;
  };
  std::vector<Spill> spills;  // per dilation: spill counter and capacity
  int rounds = 0;             // dilation rounds
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
  std::vector<vo_volume *> rerun;
  // Radius tables used by the plan, copied into plan memory: the context's
  // table cache evicts entries, and the graph reads these on every replay.
  std::vector<std::unique_ptr<DeviceTables>> tables;
  vo_batch_stats stats{};
};

namespace {

template <typename T>
int plan_alloc(vo_ctx *ctx, vo_batch *b, T **p, size_t n) {
  int rc = dalloc(ctx, p, n);
  if (!rc) b->dmem.push_back((void *)*p);
  return rc;
}

// Runs the recorded closures not yet run.
void run_pending(vo_ctx *ctx, vo_batch *b) {
  for (; b->executed < b->rec.size(); ++b->executed) b->rec[b->executed](ctx->stream);
}

void record(vo_batch *b, int kernels, Launch f) {
  b->rec.push_back(std::move(f));
  b->kernels += kernels;
}

// Maximum segment count of a slot volume (synchronising).
int max_count(vo_ctx *ctx, const SlotVol &v, int *out) {
  int *d = nullptr;
  int rc = dalloc(ctx, &d, 1);
  if (rc) return rc;
  cudaMemsetAsync(d, 0, sizeof(int), ctx->stream);
  slot_max_count(ctx, v, d);
  int h = 0;
  cudaMemcpyAsync(&h, d, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream);
  dfree(ctx, d);
  VO_CK(ctx, cudaStreamSynchronize(ctx->stream));
  *out = h;
  return VO_OK;
}

// Output slot layout of one dilation: learned per-tile capacities, or fixed.
int size_output(vo_ctx *ctx, vo_batch *b, DilPlan &d, double radius) {
  const vo_grid &g = d.in.grid;
  const int ncols = g.nx * g.ny;
  d.tiles32_x = (g.nx + kSizerTile - 1) / kSizerTile;
  d.tiles32 = d.tiles32_x * ((g.ny + kSizerTile - 1) / kSizerTile);
  int rc = VO_OK;
  int64_t entries = (int64_t)ncols * kUnionCap;
  if (ctx->sizer) {
    float *feats = nullptr, *pred = nullptr;
    int nt = 0;
    rc = dalloc(ctx, &feats, (size_t)d.tiles32 * VO_SIZER_FEATURES);
    if (!rc) rc = dalloc(ctx, &pred, (size_t)d.tiles32 * 4);
    if (!rc) rc = sizer_features_device(ctx, d.in, radius, feats, &nt);
    if (!rc) rc = sizer_predict_device(ctx, ctx->sizer, feats, nt, pred);
    std::vector<float> hp((size_t)d.tiles32 * 4);
    if (!rc) {
      cudaMemcpyAsync(hp.data(), pred, sizeof(float) * hp.size(), cudaMemcpyDeviceToHost, ctx->stream);
      cudaError_t e = cudaStreamSynchronize(ctx->stream);
      if (e != cudaSuccess) rc = cuda_error(ctx, e, "sizer prediction");
    }
    dfree(ctx, feats);
    dfree(ctx, pred);
    if (rc) return rc;
    std::vector<int32_t> cap(d.tiles32), off(d.tiles32);
    d.tile_work.resize(d.tiles32);
    int64_t total = 0;
    for (int t = 0; t < d.tiles32; ++t) {
      const int tx = t % d.tiles32_x, ty = t / d.tiles32_x;
      const int cols = std::min(kSizerTile, g.nx - tx * kSizerTile) * std::min(kSizerTile, g.ny - ty * kSizerTile);
      // predicted max segments per column, with a margin against the error of a log2 estimate
      const double mx = std::exp2((double)hp[(size_t)t * 4]) - 1.0;
      const int c = (int)std::min<double>(kUnionCapMid, std::max(1.0, std::ceil(mx * 1.5 + 2.0)));
      cap[t] = c;
      off[t] = (int32_t)total;
      total += (int64_t)c * cols;
      const double w = std::exp2((double)hp[(size_t)t * 4 + 2]) - 1.0;
      d.tile_work[t] = w >= 0 && w < 1e30 ? (float)w : 0.f;  // a diverged network must not break the sort
    }
    d.spill_base = (int)total;
    d.spill_cap = (int)std::max<int64_t>(4096, total / 4);
    entries = total + d.spill_cap;
    if (entries > 2147483647LL) return set_error(ctx, VO_ERANGE, "batch: slot layout exceeds int32 offsets");
    rc = plan_alloc(ctx, b, &d.tcap, (size_t)d.tiles32);
    if (!rc) rc = plan_alloc(ctx, b, &d.toff, (size_t)d.tiles32);
    if (!rc) rc = plan_alloc(ctx, b, &d.spill_used, 1);
    if (rc) return rc;
    cudaMemcpyAsync(d.tcap, cap.data(), sizeof(int32_t) * cap.size(), cudaMemcpyHostToDevice, ctx->stream);
    cudaMemcpyAsync(d.toff, off.data(), sizeof(int32_t) * off.size(), cudaMemcpyHostToDevice, ctx->stream);
    VO_CK(ctx, cudaStreamSynchronize(ctx->stream));  // the host vectors go out of scope
  } else {
    // fixed capacity kUnionCap per column, spill space for 1/8 of that
    d.spill_base = (int)std::min<int64_t>(entries, 2147483647LL);
    d.spill_cap = (int)std::max<int64_t>(4096, entries / 8);
    entries += d.spill_cap;
    if (entries > 2147483647LL) return set_error(ctx, VO_ERANGE, "batch: slot layout exceeds int32 offsets");
    rc = plan_alloc(ctx, b, &d.spill_used, 1);
    if (rc) return rc;
  }
  d.slot_entries = entries;
  d.out = SlotVol();
  d.out.grid = g;
  d.out.cap = kUnionCap;
  d.out.entries = entries;
  d.out.owns = false;  // plan memory
  rc = plan_alloc(ctx, b, &d.out.beg, (size_t)ncols);
  if (!rc) rc = plan_alloc(ctx, b, &d.out.end, (size_t)ncols);
  if (!rc) rc = plan_alloc(ctx, b, &d.out.z, (size_t)entries);
  return rc;
}

BatchVol batch_vol(const DilPlan &d, int *ovf) {
  BatchVol v;
  const vo_grid &g = d.in.grid;
  v.A = FastArgs{g.nx, g.ny, d.T->host.W, d.in.beg, d.in.end, (const double *)d.in.z, d.zf, d.T->Hf, d.T->H,
                 d.pairs, d.npairs, d.E, d.col, d.prec, d.dmask, d.mask_bits};
  v.obeg = d.out.beg;
  v.oend = d.out.end;
  v.oz = d.out.z;
  v.tcap = d.tcap;
  v.toff = d.toff;
  v.cap = kUnionCap;
  v.tiles32_x = d.tiles32_x;
  v.spill_base = d.spill_base;
  v.spill_cap = d.spill_cap;
  v.spill_used = d.spill_used;
  v.mid_list = d.mid_list;
  v.mid_count = d.mid_count;
  v.big_list = d.big_list;
  v.big_count = d.big_count;
  v.ovf = ovf;
  return v;
}

// Work queue for blocks of kFastCols x fby columns: dilations in decreasing
// estimated total work (longest first, for the balance of the persistent
// grid), each dilation's tiles in bands of 512 columns, all rows of a band
// before the next, so that the tiles running at the same time cover a compact
// region and share their source columns in L1 / L2 (2048^2 r = 32: 7.0 GB of
// DRAM traffic per launch in full-width rows, 4.1 GB in bands, same time).
std::vector<int2> build_queue(const std::vector<DilPlan> &dils, int fby) {
  std::vector<std::pair<double, int>> order;
  for (size_t i = 0; i < dils.size(); ++i) {
    const DilPlan &d = dils[i];
    const vo_grid &g = d.in.grid;
    double w = 0;
    if (!d.tile_work.empty()) {
      for (int t = 0; t < d.tiles32; ++t) {
        const int tx = t % d.tiles32_x, ty = t / d.tiles32_x;
        w += (double)d.tile_work[t] * std::min(kSizerTile, g.nx - tx * kSizerTile) *
             std::min(kSizerTile, g.ny - ty * kSizerTile);
      }
    } else {
      w = d.cost * g.nx * (double)g.ny;
    }
    order.push_back({w, (int)i});
  }
  std::stable_sort(order.begin(), order.end(), [](const std::pair<double, int> &a, const std::pair<double, int> &b) {
    return a.first > b.first;
  });
  std::vector<int2> q;
  for (const auto &o : order) {
    const vo_grid &g = dils[o.second].in.grid;
    const int bw = kPatchX * fby;  // a block's columns: bw x kPatchY
    // tiles in bands of 512 columns, rows within a band in order: the blocks in flight then cover a
    // compact region, whose source columns stay in L2 while they are re-read
    const int tx_n = (g.nx + bw - 1) / bw, ty_n = (g.ny + kPatchY - 1) / kPatchY;
    const int band = std::max(1, 512 / bw);
    for (int b0 = 0; b0 < tx_n; b0 += band)
      for (int ty = 0; ty < ty_n; ++ty)
        for (int tx = b0; tx < std::min(tx_n, b0 + band); ++tx) q.push_back(make_int2(o.second, ty * tx_n + tx));
  }
  return q;
}

int sm_count() {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms > 0 ? sms : 1;
}

// Autotuner: times every (union capacity, register budget, block shape,
// persistent or one block per item) on a sample of the round's queue (four evenly spaced
// contiguous runs, about 1/16 of it but two to four waves of resident blocks, at least 512 items), the second tier
// included, and keeps the fastest per column. Results are cached in the
// context per (one dilation or several, log2 columns, radius bucket, dense or
// not, learned or not).
// Tuning launches write into the round's output slots, which the real launch
// overwrites.
int tune_shape(vo_ctx *ctx, vo_batch *b, const std::vector<DilPlan> &dils, const BatchVol *dvols,
               const FastArgs *single, int ka_hint, int *ka_out, int *fby_out, int *persistent_out,
               int *regs_out) {
  int64_t cols = 0;
  double rmax = 0;
  for (const DilPlan &d : dils) {
    cols += (int64_t)d.in.grid.nx * d.in.grid.ny;
    rmax = std::max(rmax, b->radii[d.vol]);
  }
  const long long key = (single ? 1LL << 40 : 0) | ((long long)std::ilogb((double)std::max<int64_t>(cols, 1)) << 16) |
                        ((long long)(rmax / 8) << 2) | (ka_hint == 64 ? 2 : 0) | (ctx->sizer ? 1 : 0);
  for (const auto &kv : ctx->tune_cache)
    if (kv.first == key) {
      *ka_out = (kv.second >> 8) & 255;
      *fby_out = kv.second & 255;
      *persistent_out = (kv.second >> 16) & 1;
      *regs_out = (kv.second >> 17) & 1 ? 80 : 64;
      return VO_OK;
    }
  // union capacities to try: 48 and 64 for dense inputs, else 24 and 32
  std::vector<int> kas = ka_hint == 64 ? std::vector<int>{48, 64} : std::vector<int>{24, 32};
  int best_ka = kas.back(), best_pers = 1, best_regs = 64;
  const int sms = sm_count();
  int best = 4;
  double best_t = 1e300;
  int *dnext = nullptr;
  int2 *dq = nullptr;
  int rc = dalloc(ctx, &dnext, 1);
  size_t qcap = 0;
  const int gmid = sms * 16;
  for (int ka : kas)
  for (int regs : kTuneRegs)
  for (int fby : kTuneShapes)
  for (int pers = 1; pers >= 0; --pers) {
    if (rc) break;
    const int per_sm = fast_batched_blocks_per_sm(ka, fby, single != nullptr, regs);
    if (per_sm <= 0) continue;
    // four contiguous runs of the queue, evenly spaced: neighbouring tiles run
    // together as in the real launch, so the sample sees its cache reuse
    const std::vector<int2> full = build_queue(dils, fby);
    // at least two waves of resident blocks: a sample smaller than a wave
    // times the tail of a partly idle GPU, not the throughput of a full one;
    // at most four (or 1/16 of the queue when that is less), so that tuning a
    // large dense round (4096^2 cylinders: 48 samples) stays a fraction of a second per sample
    const size_t waves = (size_t)2 * sms * per_sm;
    const size_t want = std::min(full.size(), std::max<size_t>({512, std::min(full.size() / 16, 2 * waves), waves}));
    std::vector<int2> sample;
    for (int r = 0; r < 4; ++r) {
      const size_t len = want / 4 + (r < (int)(want % 4) ? 1 : 0);
      const size_t at = std::min(full.size() - len, (full.size() * (2 * r + 1)) / 8);
      sample.insert(sample.end(), full.begin() + at, full.begin() + at + len);
    }
    if (sample.size() > qcap) {
      dfree(ctx, dq);
      qcap = sample.size();
      rc = dalloc(ctx, &dq, qcap);
      if (rc) break;
    }
    cudaMemcpyAsync(dq, sample.data(), sizeof(int2) * sample.size(), cudaMemcpyHostToDevice, ctx->stream);
    // persistent: one wave of blocks pulling items; otherwise one block per item
    const int grid = pers ? std::max(1, std::min<int>((int)sample.size(), sms * per_sm)) : (int)sample.size();
    float ms = 0;
    for (int rep = 0; rep < 2; ++rep) {  // the first run warms caches and clocks
      cudaMemsetAsync(dnext, 0, sizeof(int), ctx->stream);
      for (const DilPlan &d : dils) {
        cudaMemsetAsync(d.spill_used, 0, sizeof(int), ctx->stream);
        cudaMemsetAsync(d.mid_count, 0, sizeof(int), ctx->stream);
        cudaMemsetAsync(d.big_count, 0, sizeof(int), ctx->stream);
      }
      cudaEventRecord(ctx->ev[2], ctx->stream);
      fast_batched_launch(ka, fby, regs, grid, ctx->stream, dvols, dq, (int)sample.size(), dnext, single);
      fast_batched_mid_launch(ctx->stream, dvols, (int)dils.size(), gmid);  // unions beyond ka count too
      cudaEventRecord(ctx->ev[3], ctx->stream);
      cudaError_t e = cudaStreamSynchronize(ctx->stream);
      if (e != cudaSuccess) {
        rc = cuda_error(ctx, e, "autotune");
        break;
      }
      cudaEventElapsedTime(&ms, ctx->ev[2], ctx->ev[3]);
    }
    if (rc) break;
    const double per_col = ms / ((double)sample.size() * kFastCols * fby);
    if (ka == kas.back() && pers && regs == 64) b->stats.tune_ms[fby == 1 ? 0 : fby == 2 ? 1 : 2] = ms;
    if (per_col < best_t) {
      best_t = per_col;
      best = fby;
      best_ka = ka;
      best_pers = pers;
      best_regs = regs;
    }
  }
  dfree(ctx, dnext);
  dfree(ctx, dq);
  if (rc) return rc;
  ctx->tune_cache.push_back({key, ((best_regs == 80) << 17) | (best_pers << 16) | (best_ka << 8) | best});
  *ka_out = best_ka;
  *fby_out = best;
  *persistent_out = best_pers;
  *regs_out = best_regs;
  return VO_OK;
}

int plan_dilation_round(vo_ctx *ctx, vo_batch *b, std::vector<DilPlan> &dils, bool later_rounds) {
  const int sms = sm_count();
  int rc = VO_OK;
  for (DilPlan &d : dils) {
    const vo_grid &g = d.in.grid;
    const int ncols = g.nx * g.ny;
    const std::vector<int2> pairs = fast_pairs(d.T->host);
    d.npairs = (int)pairs.size();
    rc = plan_alloc(ctx, b, &d.zf, 2 * (size_t)std::max<int64_t>(d.in.entries, 1));
    if (!rc) rc = plan_alloc(ctx, b, &d.E, 1);
    if (!rc) rc = plan_alloc(ctx, b, &d.col, (size_t)ncols);
    // mean segments per column of the input, exact for CSR inputs, the capacity's half for slots
    const double mean_in = d.in.cap > 0 && d.in.owns ? d.in.cap * 0.5 : (double)d.in.entries / std::max(ncols, 1);
    d.mask_bits = mask_bits_for(mean_in);
    if (!rc) rc = plan_alloc(ctx, b, &d.dmask, mask_words((size_t)ncols, d.mask_bits));
    if (!rc) rc = plan_alloc(ctx, b, &d.prec, pairs.size());
    if (!rc) rc = plan_alloc(ctx, b, &d.mid_list, (size_t)ncols);
    if (!rc) rc = plan_alloc(ctx, b, &d.mid_count, 1);
    if (!rc) rc = plan_alloc(ctx, b, &d.big_list, (size_t)ncols);
    if (!rc) rc = plan_alloc(ctx, b, &d.big_count, 1);
    if (!rc) rc = plan_alloc(ctx, b, &d.maxbits, 1);
    if (!rc) rc = plan_alloc(ctx, b, &d.pairs, pairs.size());
    if (rc) return rc;
    cudaMemcpyAsync(d.pairs, pairs.data(), sizeof(int2) * pairs.size(), cudaMemcpyHostToDevice, ctx->stream);
    fast_pair_records(ctx->stream, d.pairs, d.npairs, *d.T, d.prec);  // static: built once, not replayed
    VO_CK(ctx, cudaStreamSynchronize(ctx->stream));
    const SlotVol in = d.in;
    float *zf = d.zf, *E = d.E;
    int4 *col = d.col;
    unsigned *dmask = d.dmask;
    const int mbits = d.mask_bits;
    unsigned int *mb = d.maxbits;
    const float R = (float)b->radii[d.vol];
    const DomLevels L = d.T->host.dom;
    record(b, 3, [in, zf, E, mb, R, col, dmask, mbits, L](cudaStream_t st) {
      fast_prepare(st, in.grid.nx, in.grid.ny, in.beg, in.end, in.z, zf, mb, R, E, col, dmask, mbits, L);
    });
    // candidates per column ~ 4 x pairs x mean segments of the input (no sizer)
    const double segs = d.in.cap > 0 && d.in.owns ? d.in.cap * 0.5 : (double)d.in.entries / std::max(ncols, 1);
    d.cost = (double)d.npairs * 4.0 * (segs + 0.5);
  }
  if (ctx->sizer) run_pending(ctx, b);  // features need the dilation inputs
  for (DilPlan &d : dils) {
    rc = size_output(ctx, b, d, b->radii[d.vol]);
    if (rc) return rc;
    b->stats.slot_bytes += d.slot_entries * (int64_t)sizeof(double2);
  }
  std::vector<BatchVol> hv;
  for (DilPlan &d : dils) hv.push_back(batch_vol(d, b->d_flags + d.vol));
  BatchVol *dvols = nullptr;
  int *dnext = nullptr;
  rc = plan_alloc(ctx, b, &dvols, hv.size());
  if (!rc) rc = plan_alloc(ctx, b, &dnext, 1);
  if (rc) return rc;
  cudaMemcpyAsync(dvols, hv.data(), sizeof(BatchVol) * hv.size(), cudaMemcpyHostToDevice, ctx->stream);
  VO_CK(ctx, cudaStreamSynchronize(ctx->stream));
  // union capacity of the round: 64 when its inputs average more than 10 segments per column
  double segs = 0, cols = 0;
  for (const DilPlan &d : dils) {
    const double nc = (double)d.in.grid.nx * d.in.grid.ny;
    segs += d.in.owns ? 0.5 * d.in.cap * nc : (double)d.in.entries;
    cols += nc;
  }
  int ka = fast_union_cap(segs / std::max(cols, 1.0)), fby = 4, persistent = 1, regs = 64;
  run_pending(ctx, b);  // tuning reads the dilation inputs
  // a round of one dilation passes its arguments as a kernel parameter
  const bool one = hv.size() == 1;
  const FastArgs a1 = hv[0].A;
  rc = tune_shape(ctx, b, dils, dvols, one ? &a1 : nullptr, ka, &ka, &fby, &persistent, &regs);
  if (rc) return rc;
  const std::vector<int2> q = build_queue(dils, fby);
  int2 *dq = nullptr;
  rc = plan_alloc(ctx, b, &dq, q.size());
  if (rc) return rc;
  cudaMemcpyAsync(dq, q.data(), sizeof(int2) * q.size(), cudaMemcpyHostToDevice, ctx->stream);
  VO_CK(ctx, cudaStreamSynchronize(ctx->stream));
  const int per_sm = std::max(1, fast_batched_blocks_per_sm(ka, fby, one, regs));
  const int grid = persistent ? std::max(1, std::min<int>((int)q.size(), sms * per_sm)) : std::max(1, (int)q.size());
  std::vector<int *> counters;  // reset before every replay
  for (DilPlan &d : dils) {
    counters.push_back(d.spill_used);
    counters.push_back(d.mid_count);
    counters.push_back(d.big_count);
  }
  if (!b->big_scratch) {
    rc = plan_alloc(ctx, b, &b->big_scratch, fast_batched_big_scratch_elems(sms));
    if (rc) return rc;
  }
  double2 *big_scratch = b->big_scratch;
  const int nq = (int)q.size(), nv = (int)dils.size(), gmid = sms * 16;
  record(b, 3, [=](cudaStream_t st) {
    cudaMemsetAsync(dnext, 0, sizeof(int), st);
    for (int *s : counters) cudaMemsetAsync(s, 0, sizeof(int), st);
    fast_batched_launch(ka, fby, regs, grid, st, dvols, dq, nq, dnext, one ? &a1 : nullptr);
    fast_batched_mid_launch(st, dvols, nv, gmid);
    fast_batched_big_launch(st, dvols, nv, sms, big_scratch);
  });
  for (const DilPlan &d : dils) b->spills.push_back({d.spill_used, d.spill_cap, b->rounds});
  ++b->rounds;
  b->stats.tile_rows = fby;
  b->stats.union_cap = ka;
  b->stats.persistent = persistent;
  b->stats.regs = regs;
  b->stats.tiles += nq;
  if (later_rounds) run_pending(ctx, b);
  return VO_OK;
}

void plan_free(vo_ctx *ctx, vo_batch *b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  for (SlotVol &s : b->owned) slot_free(ctx, s);
  for (void *p : b->dmem) dfree(ctx, p);
  for (vo_volume *v : b->normalized)
    if (v) vo_volume_free(ctx, v);
  for (vo_volume *v : b->rerun)
    if (v) vo_volume_free(ctx, v);
  cudaStreamSynchronize(ctx->stream);
  delete b;
}

// Plan-owned copy of the tables of radius R (H, Hf and dH on the device, the
// host tables), shared by the plan's volumes of the same radius. The cached
// context entry is copied before any other table lookup can evict it.
int plan_tables(vo_ctx *ctx, vo_batch *b, double R, int kmax, const DeviceTables **out) {
  for (const auto &t : b->tables)
    if (t->R == R && t->kmax >= kmax) {
      *out = t.get();
      return VO_OK;
    }
  const DeviceTables *T = nullptr;
  int rc = get_tables(ctx, R, kmax, &T);
  if (rc) return rc;
  std::unique_ptr<DeviceTables> own(new (std::nothrow) DeviceTables());
  if (!own) return set_error(ctx, VO_ENOMEM, "host allocation");
  own->R = T->R;
  own->kmax = T->kmax;
  own->host = T->host;
  const size_t nh = T->host.H.size();
  rc = plan_alloc(ctx, b, &own->H, nh);
  if (!rc) rc = plan_alloc(ctx, b, &own->Hf, nh);
  if (!rc) rc = plan_alloc(ctx, b, &own->dH, 2 * nh);
  if (rc) return rc;
  cudaMemcpyAsync(own->H, T->H, sizeof(double) * nh, cudaMemcpyDeviceToDevice, ctx->stream);
  cudaMemcpyAsync(own->Hf, T->Hf, sizeof(float) * nh, cudaMemcpyDeviceToDevice, ctx->stream);
  cudaMemcpyAsync(own->dH, T->dH, sizeof(float) * 2 * nh, cudaMemcpyDeviceToDevice, ctx->stream);
  VO_CK(ctx, cudaStreamSynchronize(ctx->stream));
  *out = own.get();
  b->tables.push_back(std::move(own));
  return VO_OK;
}

int plan_build(vo_ctx *ctx, vo_batch *b) {
  const int n = b->n;
  int rc = plan_alloc(ctx, b, &b->d_flags, (size_t)n + 1);
  if (rc) return rc;
  int *flags = b->d_flags;
  record(b, 0, [flags, n](cudaStream_t st) { cudaMemsetAsync(flags, 0, sizeof(int) * (n + 1), st); });
  std::vector<std::vector<StepKind>> chain(n);
  std::vector<SlotVol> cur(n);
  std::vector<const DeviceTables *> tabs(n);
  for (int v = 0; v < n; ++v) {
    chain[v] = steps_of(b->ops[v]);
    const vo_volume *in = b->ins[v];
    if (chain[v][0] == kDil) {  // inverted pairs in a dilation input are rewritten first
      rc = normalize_inverted(ctx, in, &b->normalized[v]);
      if (rc) return rc;
      if (b->normalized[v]) in = b->normalized[v];
    }
    cur[v] = slot_view(in, 0);
    rc = max_count(ctx, cur[v], &cur[v].cap);
    if (!rc) rc = plan_tables(ctx, b, b->radii[v], std::max(in->grid.nx, in->grid.ny) + 2, &tabs[v]);
    if (rc) return rc;
  }
  std::vector<size_t> next(n, 0);
  for (;;) {
    std::vector<DilPlan> dils;
    bool any = false;
    for (int v = 0; v < n; ++v) {
      if (next[v] >= chain[v].size()) continue;
      any = true;
      const StepKind k = chain[v][next[v]++];
      const SlotVol in = cur[v];
      SlotVol out;
      int *ovf = b->d_flags + n;
      if (k == kDil) {
        DilPlan d;
        d.vol = v;
        d.in = in;
        d.T = tabs[v];
        dils.push_back(d);
        continue;
      }
      // complement steps: slot outputs sized from the input's largest column
      if (k == kNeg) {
        vo_grid g2 = in.grid;
        g2.nx += 2;
        g2.ny += 2;
        rc = slot_alloc(ctx, g2, in.cap + 1, out);
        if (!rc) record(b, 1, [in, out, ovf](cudaStream_t st) { slot_negate_launch(st, in, out, ovf); });
      } else if (k == kNorm) {
        rc = slot_alloc(ctx, in.grid, in.cap + 2, out);
        if (!rc) record(b, 1, [in, out, ovf](cudaStream_t st) { slot_normalize_launch(st, in, out, ovf); });
      } else {
        const vo_grid g = b->ins[v]->grid;
        rc = slot_alloc(ctx, g, in.cap + 1, out);
        if (!rc) record(b, 1, [in, g, out, ovf](cudaStream_t st) { slot_negate_inv_launch(st, in, g, out, ovf); });
      }
      if (rc) return rc;
      b->owned.push_back(out);
      cur[v] = out;
    }
    if (!any) break;
    if (dils.empty()) continue;
    bool later = false;
    for (const DilPlan &d : dils) later |= next[d.vol] < chain[d.vol].size();
    rc = plan_dilation_round(ctx, b, dils, later);
    if (rc) return rc;
    for (DilPlan &d : dils) {
      cur[d.vol] = d.out;
      // a complement of this result needs its largest column (the data exists: the round ran)
      if (next[d.vol] < chain[d.vol].size()) {
        rc = max_count(ctx, d.out, &cur[d.vol].cap);
        if (rc) return rc;
      }
    }
  }
  b->finals = cur;
  // ---- capture every recorded step into one graph
  VO_CK(ctx, cudaStreamSynchronize(ctx->stream));
  VO_CK(ctx, cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
  for (Launch &f : b->rec) f(ctx->stream);
  cudaError_t e = cudaStreamEndCapture(ctx->stream, &b->graph);
  if (e != cudaSuccess) return cuda_error(ctx, e, "graph capture");
  e = cudaGraphInstantiate(&b->exec, b->graph, 0);
  if (e != cudaSuccess) return cuda_error(ctx, e, "graph instantiate");
  size_t nodes = 0;
  cudaGraphGetNodes(b->graph, nullptr, &nodes);
  b->stats.graph_nodes = (int)nodes;
  b->stats.graph_kernels = b->kernels;
  b->stats.learned = ctx->sizer ? 1 : 0;
  return VO_OK;
}

// Single-volume re-run of volume v (any union size).
int rerun_volume(vo_ctx *ctx, vo_batch *b, int v, vo_volume **out) {
  vo_timings t;
  std::memset(&t, 0, sizeof t);
  const vo_volume *in = b->ins[v];
  const double r = b->radii[v];
  switch (b->ops[v]) {
    case VO_DILATION:
      return dilate(ctx, VO_METHOD_FAST, r, in, out, &t);
    case VO_EROSION:
      return erode(ctx, VO_METHOD_FAST, r, in, out, &t);
    default: {
      vo_volume *tmp = nullptr;
      const bool open = b->ops[v] == VO_OPENING;
      int rc = open ? erode(ctx, VO_METHOD_FAST, r, in, &tmp, &t) : dilate(ctx, VO_METHOD_FAST, r, in, &tmp, &t);
      if (!rc) rc = open ? dilate(ctx, VO_METHOD_FAST, r, tmp, out, &t) : erode(ctx, VO_METHOD_FAST, r, tmp, out, &t);
      if (tmp) vo_volume_free(ctx, tmp);
      return rc;
    }
  }
}

int volume_copy(vo_ctx *ctx, const vo_volume *src, vo_volume **out) {
  vo_volume *v = nullptr;
  int rc = volume_alloc(ctx, src->grid, src->nseg, &v);
  if (rc) return rc;
  const size_t ncols = (size_t)src->grid.nx * src->grid.ny;
  cudaMemcpyAsync(v->offs, src->offs, sizeof(int32_t) * (ncols + 1), cudaMemcpyDeviceToDevice, ctx->stream);
  if (src->nseg > 0)
    cudaMemcpyAsync(v->z, src->z, sizeof(double2) * src->nseg, cudaMemcpyDeviceToDevice, ctx->stream);
  v->inverted = src->inverted;
  *out = v;
  return VO_OK;
}

bool valid_batch(int n, const int *ops, const double *radii, int method, const vo_volume *const *ins) {
  if (n < 0 || (n > 0 && (!ops || !radii || !ins))) return false;
  if (method != VO_METHOD_FAST) return false;
  for (int i = 0; i < n; ++i)
    if (!ins[i] || ops[i] < VO_DILATION || ops[i] > VO_CLOSING || !(radii[i] >= 0) || radii[i] > 255) return false;
  return true;
}

}  // namespace

extern "C" {

int vo_batch_create(vo_ctx *ctx, int n, const int *ops, const double *radii, int method,
                    const vo_volume *const *ins, vo_batch **out) {
  if (!ctx || !out) return VO_EINVAL;
  *out = nullptr;
  if (!valid_batch(n, ops, radii, method, ins))
    return set_error(ctx, VO_EINVAL, "batch: bad volume, op, radius or method (VO_METHOD_FAST only)");
  cudaSetDevice(ctx->device);
  for (int i = 0; i < n; ++i) vol_wait(ctx, ins[i]);  // before any capture: the plan then reads them in order
  ctx->err.clear();
  const auto t0 = std::chrono::steady_clock::now();
  vo_batch *b = new vo_batch();
  b->n = n;
  b->ops.assign(ops, ops + n);
  b->radii.assign(radii, radii + n);
  b->ins.assign(ins, ins + n);
  b->normalized.assign(n, nullptr);
  b->rerun.assign(n, nullptr);
  std::memset(&b->stats, 0, sizeof b->stats);
  const int rc = plan_build(ctx, b);
  if (rc) {
    cudaStreamSynchronize(ctx->stream);
    cudaGetLastError();
    plan_free(ctx, b);
    return rc;
  }
  b->stats.plan_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
  *out = b;
  return VO_OK;
}

int vo_batch_run(vo_ctx *ctx, vo_batch *b, vo_timings *tm) {
  if (!ctx || !b) return VO_EINVAL;
  cudaSetDevice(ctx->device);
  const auto t0 = std::chrono::steady_clock::now();
  for (vo_volume *&v : b->rerun)
    if (v) {
      vo_volume_free(ctx, v);
      v = nullptr;
    }
  const int n = b->n;
  std::vector<int> flags(n + 1, 0);
  cudaEventRecord(ctx->ev[0], ctx->stream);
  VO_CK(ctx, cudaGraphLaunch(b->exec, ctx->stream));
  cudaEventRecord(ctx->ev[1], ctx->stream);
  cudaMemcpyAsync(flags.data(), b->d_flags, sizeof(int) * (n + 1), cudaMemcpyDeviceToHost, ctx->stream);
  VO_CK(ctx, cudaStreamSynchronize(ctx->stream));
  float graph_ms = 0;
  cudaEventElapsedTime(&graph_ms, ctx->ev[0], ctx->ev[1]);
  // spill use of every dilation (the largest fraction and its round)
  b->stats.spill_peak = 0;
  b->stats.spill_peak_round = -1;
  for (const auto &sp : b->spills) {
    int used = 0;
    if (cudaMemcpy(&used, sp.used, sizeof(int), cudaMemcpyDeviceToHost) != cudaSuccess) break;
    const double f = sp.cap > 0 ? (double)used / sp.cap : 0.0;
    if (f > b->stats.spill_peak) {
      b->stats.spill_peak = f;
      b->stats.spill_peak_round = sp.round;
    }
  }
  int reruns = 0;
  const int launches0 = ctx->launches;
  b->stats.rerun_first = -1;
  b->stats.rerun_cause = 0;
  for (int v = 0; v < n; ++v) {
    if (!flags[v] && !flags[n]) continue;
    if (reruns == 0) {
      b->stats.rerun_first = v;
      b->stats.rerun_cause = flags[v] | (flags[n] ? 2 : 0);
    }
    ++reruns;
    const int rc = rerun_volume(ctx, b, v, &b->rerun[v]);
    if (rc) return rc;
  }
  b->stats.reruns = reruns;
  if (tm) {
    std::memset(tm, 0, sizeof *tm);
    tm->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    tm->pass2_ms = graph_ms;
    tm->kernel_ms[3] = graph_ms;
    for (int v = 0; v < n; ++v) tm->in_segments += b->ins[v]->nseg;
    tm->kernel_launches = b->kernels + (ctx->launches - launches0);
    tm->overflow_columns = reruns;
  }
  return VO_OK;
}

int vo_batch_outputs(vo_ctx *ctx, vo_batch *b, vo_volume **outs) {
  if (!ctx || !b || (b->n > 0 && !outs)) return VO_EINVAL;
  cudaSetDevice(ctx->device);
  int rc = VO_OK;
  for (int v = 0; v < b->n; ++v) outs[v] = nullptr;
  for (int v = 0; v < b->n && !rc; ++v)
    rc = b->rerun[v] ? volume_copy(ctx, b->rerun[v], &outs[v]) : slot_to_volume(ctx, b->finals[v], &outs[v]);
  if (!rc) {
    cudaError_t e = cudaStreamSynchronize(ctx->stream);
    if (e != cudaSuccess) rc = cuda_error(ctx, e, "batch outputs");
  }
  if (rc)
    for (int v = 0; v < b->n; ++v)
      if (outs[v]) {
        vo_volume_free(ctx, outs[v]);
        outs[v] = nullptr;
      }
  return rc;
}

int vo_batch_stats_get(vo_ctx *ctx, const vo_batch *b, vo_batch_stats *s) {
  if (!ctx || !b || !s) return VO_EINVAL;
  *s = b->stats;
  return VO_OK;
}

void vo_batch_destroy(vo_ctx *ctx, vo_batch *b) {
  if (!ctx || !b) return;
  cudaSetDevice(ctx->device);
  plan_free(ctx, b);
}

}  // extern "C"

namespace vo {

int morph_batched_fast(vo_ctx *ctx, int n, const int *ops, const double *radii, const vo_volume *const *ins,
                       vo_volume **outs, vo_timings *tm) {
  const auto t0 = std::chrono::steady_clock::now();
  vo_batch *b = nullptr;
  int rc = vo_batch_create(ctx, n, ops, radii, VO_METHOD_FAST, ins, &b);
  if (rc) return rc;
  rc = vo_batch_run(ctx, b, tm);
  if (!rc) rc = vo_batch_outputs(ctx, b, outs);
  if (!rc && tm) {
    tm->total_ms = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - t0).count();
    for (int v = 0; v < n; ++v) tm->out_segments += outs[v]->nseg;
  }
  vo_batch_destroy(ctx, b);
  return rc;
}

}  // namespace vo
