// Internal declarations shared by the CUDA translation units of
// libvoroffset_gpu.so. Not part of the public ABI (include/voroffset_gpu.h).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "voroffset_gpu.h"

namespace vo {

// Per-thread capacities of the in-register/local-memory working lists. A
// column that needs more is flagged and re-run by the large-capacity variant
// of the same kernel, whose lists live in global scratch.
constexpr int kCapSmall = 32;    // pass-1 touching-merged piece list / pass-2 union
constexpr int kCapLarge = 2048;  // overflow re-run capacity per column

// Dominance levels of the FP32 kernels: a segment is dominated at level l
// in a direction when its width there is <= t[l]; a pair uses the largest
// level whose threshold is <= its FP32 lower bound of the growth of H. Any
// thresholds keep the pruning exact; t[0] = 0 and the others are quantiles of
// the pairs' growths for the radius, so that levels fall where pairs are.
constexpr int kDomLevels = 11;  // 15 in a pair record means "no level"
// Segment dominance masks hold one bit per segment of columns with at most
// mask_bits segments (16 or 32 per dilation: 16 when the input averages at
// most kMask16MeanSegs segments per column — 0.02 % of the 2048^2 workload's
// columns have more than 16 — else 32); a column with more takes the dense
// path: every segment, with the whole-column width test.
constexpr double kMask16MeanSegs = 8.0;
inline int mask_bits_for(double mean_segments_per_column) {
  return mean_segments_per_column <= kMask16MeanSegs ? 16 : 32;
}
// 32-bit words of the mask planes [4 directions][kDomLevels][ncols]
inline size_t mask_words(size_t ncols, int bits) { return (4 * (size_t)kDomLevels * ncols * bits + 31) / 32; }
struct DomLevels {
  float t[kDomLevels];
};

// Radius tables, computed on the host with the reference's own FP64
// expressions (so device results match bit for bit) and uploaded once per
// (radius, grid extent).
struct Tables {
  double R = 0;
  int Dy = 0;                 // max pass-1 lattice distance (floor(R))
  int W = 0;                  // Dx[0] + 1 (row stride of H)
  std::vector<double> r1;     // [Dy+1] pass-1 radius per label
  std::vector<int> Dx;        // [Dy+1] max |dx| per label
  std::vector<double> H;      // [(Dy+1)*W] sqrt(r1*r1 - dx*dx), NaN beyond Dx
  std::vector<float> Hf;      // FP32 rounding of H
  std::vector<double> HB;     // [(Dy+1)^2] brute force sqrt(R*R - dx^2 - dy^2), NaN outside
  DomLevels dom{};            // dominance level thresholds for this radius
};

// Device view of the tables (kernel argument by value).
struct DevTables {
  int Dy, W;
  const double *H;
  const float *Hf;
  const int *Dx;
  const double *HB;
};

// Builds tables for radius R serving sweep indices 0..kmax-1; returns VO_OK,
// VO_EINVAL or VO_ERADIUS.
int build_tables(double R, int kmax, Tables &t);

struct DeviceTables {
  double R = -1;
  int kmax = 0;
  double *H = nullptr;
  float *Hf = nullptr;
  int *Dx = nullptr;
  double *HB = nullptr;
  // FP32 lower bounds of the growth of H one lattice step toward the centre:
  // dH[d*W + a] <= H[d][a-1] - H[d][a] (x step, a >= 1) and
  // dH[(Dy+1)*W + d*W + a] <= H[d-1][a] - H[d][a] (y step, d >= 1); -inf where
  // no step exists (used by the dominance test of the FP32 kernels).
  float *dH = nullptr;
  Tables host;
  DevTables view() const { return DevTables{host.Dy, host.W, H, Hf, Dx, HB}; }
};

}  // namespace vo

struct vo_volume {
  vo_grid grid;
  int64_t nseg = 0;      // host-known segment count
  // Whether some pair has z1 > z2 (an inverted pair left by complementing a
  // column whose values exceed [zmin, zmax]): 0 no, 1 yes, -1 not yet known.
  mutable int inverted = -1;
  int32_t *offs = nullptr;  // device [nx*ny+1]
  double2 *z = nullptr;     // device [nseg]
  bool owns = true;
  // Copies on the context's copy stream (vo_volume_upload_async /
  // vo_volume_download_async): `ready` completes when the upload has landed,
  // `copied` when the last download has left; null when none was made.
  mutable cudaEvent_t ready = nullptr, copied = nullptr;
};

struct vo_ctx {
  int device = 0;
  cudaStream_t stream = nullptr;
  cudaStream_t copy_stream = nullptr;  // asynchronous uploads and downloads
  cudaEvent_t ev_order = nullptr;      // orders the copy stream after the compute stream
  std::string err;
  std::vector<vo::DeviceTables *> tables;  // small cache keyed by (R, kmax)
  cudaEvent_t ev[8] = {};
  int launches = 0;  // kernel launches of the current call
  int ovf_cols = 0;
  // persistent small device scratch
  int *d_flags = nullptr;  // [0]: overflow count, [1..]: misc status
  long long *d_total = nullptr;
  long long *h_total = nullptr;  // pinned
  vo_sizer *sizer = nullptr;     // learned sizing for the batched executor (not owned)
  int64_t dexel_odd_columns = -1;  // odd-hit columns of the last vo_dexelize (-1: none yet)
  std::vector<std::pair<long long, int>> tune_cache;  // batch autotuner: shape key -> rows per block
};

namespace vo {

// Orders the context's stream after the asynchronous upload of v, if any (every
// entry point that reads a volume calls it first).
void vol_wait(vo_ctx *ctx, const vo_volume *v);

// Error helpers: set ctx->err and return a status.
int set_error(vo_ctx *ctx, int code, const std::string &msg);
int cuda_error(vo_ctx *ctx, cudaError_t e, const char *where);

#define VO_CK(ctx, call)                                 \
  do {                                                   \
    cudaError_t e_ = (call);                             \
    if (e_ != cudaSuccess) return vo::cuda_error((ctx), e_, #call); \
  } while (0)

// Stream-ordered allocation helpers on ctx->stream.
template <typename T>
int dalloc(vo_ctx *ctx, T **p, size_t n) {
  *p = nullptr;
  if (n == 0) n = 1;
  cudaError_t e = cudaMallocAsync((void **)p, n * sizeof(T), ctx->stream);
  if (e != cudaSuccess) return cuda_error(ctx, e, "cudaMallocAsync");
  return VO_OK;
}
void dfree(vo_ctx *ctx, void *p);

// Tables for radius R, cached in the context.
int get_tables(vo_ctx *ctx, double R, int kmax, const DeviceTables **out);

// Exclusive scan of int32 counts into int32 offsets (n+1 entries); the total
// is returned through ctx->h_total (synchronising read). Returns VO_ERANGE if
// the total exceeds INT32_MAX.
int scan_counts(vo_ctx *ctx, const int32_t *counts, int32_t *offs, int n, long long *total);

// The separable scheme in its sweeping envelope form, FP64 (vo_env.cu).
// Returns VO_OK, an error, or 1 when the volume exceeds the kernels' working
// capacities and must take the painter form (VO_METHOD_SEPARABLE).
int dilate_envelope(vo_ctx *ctx, double R, const vo_volume *in, vo_volume **out, vo_timings *tm);

// Exact FP32-guarded separable dilation (vo_fast.cu).
int dilate_fast(vo_ctx *ctx, double R, const vo_volume *in, vo_volume **out, vo_timings *tm);

// Rewrites inverted pairs as their two endpoints (points) and re-sorts / merges
// the affected columns (vo_morph.cu). *out is a new volume, or nullptr when
// `in` has no inverted pair.
int normalize_inverted(vo_ctx *ctx, const vo_volume *in, vo_volume **out);

// Morphology drivers (vo_morph.cu).
int dilate(vo_ctx *ctx, int method, double R, const vo_volume *in, vo_volume **out,
           vo_timings *tm);
int erode(vo_ctx *ctx, int method, double R, const vo_volume *in, vo_volume **out,
          vo_timings *tm);

// Slot volume: column c holds z[beg[c], end[c]). slot_alloc gives the
// fixed-capacity layout beg[c] = c*cap; a CSR volume is viewed as one with
// beg = offs, end = offs + 1; batch dilations write per-tile layouts. `cap`
// bounds every column's count, `entries` is the length of z.
struct SlotVol {
  vo_grid grid{};
  int cap = 0;
  int64_t entries = 0;
  int32_t *beg = nullptr, *end = nullptr;
  double2 *z = nullptr;
  bool owns = false;
};
int slot_alloc(vo_ctx *ctx, const vo_grid &g, int cap, SlotVol &v);
void slot_free(vo_ctx *ctx, SlotVol &v);
SlotVol slot_view(const vo_volume *in, int cap);
// Complement with a one-column border (negate), normalisation of inverted
// pairs, and complement back on the inner range (negate_inv), as launches into
// already allocated slot outputs (batch plans record them for graph capture).
void slot_negate_launch(cudaStream_t st, const SlotVol &in, const SlotVol &out, int *overflow);
void slot_normalize_launch(cudaStream_t st, const SlotVol &in, const SlotVol &out, int *overflow);
void slot_negate_inv_launch(cudaStream_t st, const SlotVol &in, const vo_grid &g, const SlotVol &out,
                            int *overflow);
int slot_max_count(vo_ctx *ctx, const SlotVol &v, int *d_max);
int slot_to_volume(vo_ctx *ctx, const SlotVol &v, vo_volume **out);

// Arguments of the FP32-guarded dilation of one volume (vo_fast.cu).
struct FastArgs {
  int nx, ny, W;
  // Column c's segments are [beg[c], end[c]); for CSR input beg = offs and
  // end = offs + 1, for a slot layout beg / end are the slot arrays.
  const int32_t *beg, *end;
  const double *zd;     // FP64 values, 2 per segment
  const float *zf;      // FP32 copies
  const float *Hf;      // [(Dy+1) * W]
  const double *H64;    // [(Dy+1) * W]
  const int2 *pairs;    // (a, d) sorted by decreasing H
  int npairs;
  const float *E;       // guard band (device scalar)
  // Column records (beg, end, dominance widths x- | x+ << 16, y- | y+ << 16 as
  // FP16) and pair records (a | d << 16 as float bits, H in FP32, dH of an x
  // step, dH of a y step), both built by the fast_* helpers below.
  const int4 *col;
  const float4 *prec;
  // Segment dominance masks [4 directions][kDomLevels][ncols] of mask_bits
  // (16 or 32) bits: bit j of a column with at most mask_bits segments is set
  // when its segment j lies in a neighbour segment widened by the level's
  // threshold.
  const void *dmask;
  int mask_bits;
};

// One dilation of a batch (device array element of the persistent kernel).
constexpr int kSizerTile = 32;  // side of a sizing tile (columns)
constexpr int kUnionCap = 32;      // union capacity of the main FP32 kernels
constexpr int kUnionCapMid = 128;  // union capacity of their second tier
struct BatchVol {
  FastArgs A;
  int32_t *obeg, *oend;  // output slot arrays, written for every column
  double2 *oz;           // output values: tile slots, then the spill region
  const int32_t *tcap;   // per sizing tile capacity, or nullptr: `cap` for all
  const int32_t *toff;   // per sizing tile offset into oz
  int cap;
  int tiles32_x;
  int spill_base, spill_cap;
  int *spill_used;
  int *mid_list, *mid_count;  // columns whose union exceeds the main capacity (second tier)
  int *big_list, *big_count;  // columns whose union exceeds kUnionCapMid (third tier, FP64)
  int *ovf;  // flags: 1 a union beyond the FP64 list, 4 spill region exhausted
};

// Fills DeviceTables::dH from H on the device (directed rounding).
void launch_dh_tables(cudaStream_t st, int Dy, int W, const double *H, const int *Dx, float *dH);

// (a, d) pairs with a <= Dx[d], sorted by decreasing H (the candidate order of
// the FP32 kernels).
std::vector<int2> fast_pairs(const Tables &h);
// FP32 copies of the values of a slot volume, the guard band scalar, the
// column records (ncols int4) and the dominance masks (4 * kDomLevels * ncols).
void fast_prepare(cudaStream_t st, int nx, int ny, const int32_t *beg, const int32_t *end, const double2 *z,
                  float *zf, unsigned int *maxbits, float R, float *E, int4 *col, void *dmask, int mask_bits,
                  const DomLevels &L);
// Pair records (npairs float4) from the device tables of radius T.
void fast_pair_records(cudaStream_t st, const int2 *pairs, int npairs, const DeviceTables &T, float4 *prec);
// Union capacity (24, 32 or 64) of the main FP32 kernels for inputs with the
// given mean segment count per column.
int fast_union_cap(double mean_segments_per_column);
// Launch of the batch kernel with union capacity ka (24, 32 or 64), `fby`
// rows of kFastCols columns per block (1, 2 or 4) and a register budget of
// regs (64 or 80) per thread; fast_batched_blocks_per_sm is the occupancy of
// that variant (0: unusable). single: the round's one dilation's arguments
// (passed as a kernel parameter), or nullptr for a round of several.
int fast_batched_launch(int ka, int fby, int regs, int grid, cudaStream_t st, const BatchVol *vols,
                        const int2 *queue, int nq, int *next, const FastArgs *single);
int fast_batched_blocks_per_sm(int ka, int fby, bool single, int regs);
// Second tier of a batch round over the dilations vols[0..nv) (grid-stride).
void fast_batched_mid_launch(cudaStream_t st, const BatchVol *vols, int nv, int grid);
// Third tier (FP64) of a batch round; scratch holds
// fast_batched_big_scratch_elems(grid) intervals.
size_t fast_batched_big_scratch_elems(int grid);
void fast_batched_big_launch(cudaStream_t st, const BatchVol *vols, int nv, int grid, double2 *scratch);
// Columns of a warp of the FP32 kernels: a kPatchX x kPatchY patch, lane l at
// (l % kPatchX, l / kPatchX). Lanes iterate to the warp's longest candidate
// list, and a compact patch keeps their lists closer in length than a row of
// 32 (2048^2 r=32 dilation: 217 vs 243 ms). A block of FBY warps covers FBY
// patches side by side in x.
constexpr int kPatchX = 8, kPatchY = 4;
constexpr int kFastCols = kPatchX * kPatchY;  // columns per warp

// Batch plans (vo_batch.cu).
int morph_batched_fast(vo_ctx *ctx, int n, const int *ops, const double *radii, const vo_volume *const *ins,
                       vo_volume **outs, vo_timings *tm);

// Learned sizing (vo_sizer.cu): tile features of a slot volume into a device
// array of ntiles x VO_SIZER_FEATURES, and predictions (ntiles x 4, three used).
int sizer_features_device(vo_ctx *ctx, const SlotVol &in, double radius, float *feats, int *ntiles);
int sizer_predict_device(vo_ctx *ctx, const vo_sizer *s, const float *feats, int n, float *out4);

// Volume allocation (vo_api.cu).
int volume_alloc(vo_ctx *ctx, const vo_grid &g, int64_t nseg, vo_volume **out);

}  // namespace vo
