/*
 * voroffset_gpu.h -- C ABI of the GB300 (sm_103a) dexel morphology library.
 *
 * This is the drop-in boundary for Voroffset's 3D path: it replaces the
 * reference's method layer (src/vor3d/Voronoi.h:13-44, class VoronoiMorpho and
 * its implementations VoronoiMorphoVorPower "ours" and
 * VoronoiMorphoBruteForce "brute_force") and the ray rasteriser
 * (src/vor3d/Dexelize.h:25-28, create_dexels). Plain C types only: int32
 * offsets and FP64 endpoint pairs, no C++ or torch types, no exceptions; every
 * entry point returns a status code (VO_OK == 0) and records a message
 * retrievable with vo_last_error().
 *
 * Data model (src/vor3d/CompressedVolume.h:28-29, CompressedVolumeBase.h:17-21):
 *   a volume is an nx*ny grid of columns, column index c = x + nx*y; each
 *   column is a sorted list of disjoint closed z-intervals [z1, z2] in dexel
 *   units (absolute z / spacing). In CSR form: offs[nx*ny+1] (int32, counted
 *   in segments, offs[0] == 0) and z[2*offs[nx*ny]] (FP64 pairs).
 *   `origin` is the stored origin, already shifted by -padding*spacing the way
 *   the CompressedVolume constructor leaves it (CompressedVolume.cpp:11-23).
 *
 * All device work of a context runs on the context's own CUDA stream, in
 * order. A context must not be used from two host threads at once.
 */
#ifndef VOROFFSET_GPU_H
#define VOROFFSET_GPU_H
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---- */
#define VO_OK 0
#define VO_EINVAL -1    /* bad argument */
#define VO_ENOMEM -2    /* host or device allocation failed */
#define VO_ECUDA -3     /* CUDA runtime error (message in vo_last_error) */
#define VO_ERADIUS -4   /* radius within rounding of a lattice distance: its lattice reach would
                           depend on the column position (floor(x + r) != x + floor(r)) */
#define VO_ERANGE -5    /* result does not fit int32 CSR offsets */
#define VO_ENODEV -6    /* no usable sm_103 device */
#define VO_ETIMEOUT -7  /* a device-side bounded wait gave up */
#define VO_EINTERNAL -8 /* internal consistency check failed */

/* ---- operations (app/cli3d/offset3d.cpp:48-49, 116-136) ---- */
#define VO_DILATION 0
#define VO_EROSION 1
#define VO_OPENING 2 /* erosion then dilation */
#define VO_CLOSING 3 /* dilation then erosion */

/* ---- methods ----
 * VO_METHOD_SEPARABLE: the separable "ours" scheme (VoronoiVorPower.cpp:24-96),
 *   FP64 end to end, count -> scan -> fill. Results match the reference's
 *   FP64 CPU output (exact topology, endpoints within 1e-9).
 * VO_METHOD_BRUTE: the lattice-disc brute force (VoronoiBruteForce.cpp:16-68),
 *   the in-GPU cross-check.
 * VO_METHOD_FAST: the separable scheme with FP32 envelope arithmetic guarded by
 *   FP64 re-evaluation of near-tie merge/touch decisions (no reference
 *   counterpart).
 * VO_METHOD_ENVELOPE: the separable scheme as the reference sweeps it, FP64:
 *   pass 1 sweeps each x-line keeping the half-space Voronoi envelope of the
 *   segments (Voronoi2D.cpp:591-723), pass 2 sweeps each row keeping the live
 *   stadiums of the pass-1 pieces and takes their union on every line
 *   (SeparatePower2D.cpp:228-541), one warp per line / one block per row.
 *   Same results as VO_METHOD_SEPARABLE. Environment: VO_ENVELOPE_BAND_PIECES
 *   caps the pass-1 pieces held at once (rows are then swept in bands);
 *   VO_ENVELOPE_STATE_CAP lowers the shared-memory stadium capacity of
 *   pass 2 (rows beyond it sweep with global-memory state);
 *   VO_ENVELOPE_ROW_CHUNK caps the rows of one global-memory launch. */
#define VO_METHOD_SEPARABLE 0
#define VO_METHOD_BRUTE 1
#define VO_METHOD_FAST 2
#define VO_METHOD_ENVELOPE 3

typedef struct vo_ctx vo_ctx;
typedef struct vo_volume vo_volume; /* a device-resident CSR volume */

typedef struct {
  int32_t nx, ny;
  double origin[3];
  double extent[3];
  double spacing;
  int32_t padding;
} vo_grid;

typedef struct {
  double total_ms;  /* wall time of the call on the host */
  double pass1_ms;  /* device time of the pass-1 kernels (time_1 of VoronoiVorPower.cpp:66) */
  double pass2_ms;  /* device time of the pass-2 kernels (time_2 of VoronoiVorPower.cpp:95) */
  int64_t in_segments;
  int64_t mid_pieces; /* pass-1 intermediate size (summed over chained ops) */
  int64_t out_segments;
  int32_t kernel_launches; /* kernels this call launched */
  int32_t overflow_columns; /* columns re-run through the large-capacity path (envelope
                             * form: lines and rows whose sweep ran with its state in
                             * global memory) */
  /* device time (CUDA events on the context stream) of the pass-1 count,
   * pass-1 fill, pass-2 count and pass-2 fill kernels, summed over the call
   * (brute force: [2] count, [3] fill) */
  double kernel_ms[4];
} vo_timings;

/* Context (replaces std::make_unique<VoronoiMorphoVorPower>() at offset3d.cpp:104-112).
 * device: CUDA ordinal; the device must be sm_103. */
int vo_create(vo_ctx **ctx, int device);
void vo_destroy(vo_ctx *ctx);
/* Last error message of this context (never NULL; "" when none). */
const char *vo_last_error(const vo_ctx *ctx);
/* The context's cudaStream_t, as void*, so a host can order its own work or
 * record events on it. */
void *vo_stream(vo_ctx *ctx);
/* Blocks until the context's streams (compute and copy) are idle. */
int vo_sync(vo_ctx *ctx);

/* Volumes. Upload copies host CSR into a new device volume
 * (the value semantics of VoronoiMorpho::dilation's by-value input, Voronoi.h:18).
 * The copies run on the context's stream: from page-locked host memory they
 * are asynchronous, so such buffers must stay unchanged until the next call
 * that returns results (vo_morph, vo_volume_download, ...) has returned. */
int vo_volume_upload(vo_ctx *ctx, const vo_grid *grid, const int32_t *offs, const double *z,
                     vo_volume **out);
/* Asynchronous copies on the context's second (copy) stream, so that they
 * overlap the kernels of its compute stream (no reference counterpart).
 * vo_volume_upload_async: as vo_volume_upload (same checks, returns before the
 *   copy ends); the host buffers must be page-locked and stay unchanged until
 *   vo_sync, or a call that returns results, has returned. Every entry point
 *   that reads the volume orders its device work after the copy.
 * vo_volume_download_async: copies the volume into page-locked host buffers
 *   once the work already queued on the compute stream has produced it, and
 *   returns; the buffers hold the result after vo_sync. Freeing the volume
 *   waits for the copy in stream order. */
int vo_volume_upload_async(vo_ctx *ctx, const vo_grid *grid, const int32_t *offs, const double *z,
                           vo_volume **out);
int vo_volume_download_async(vo_ctx *ctx, const vo_volume *v, int32_t *offs, double *z);
/* Grid and segment count of a volume (the size query before a download). */
int vo_volume_info(vo_ctx *ctx, const vo_volume *v, vo_grid *grid, int64_t *nseg);
/* Copies a volume to caller-allocated host buffers: offs[nx*ny+1], z[2*nseg]. */
int vo_volume_download(vo_ctx *ctx, const vo_volume *v, int32_t *offs, double *z);
/* Device pointers of a volume (offs: int32*, z: double*), valid until freed. */
int vo_volume_device_ptrs(vo_ctx *ctx, const vo_volume *v, void **offs, void **z);
void vo_volume_free(vo_ctx *ctx, vo_volume *v);

/* Morphology (replaces VoronoiMorpho::dilation / erosion, Voronoi.h:18-29, and
 * the opening/closing chaining of offset3d.cpp:124-133). radius in dexels.
 * *out receives a new volume with the input's grid. timings may be NULL. */
int vo_morph(vo_ctx *ctx, int op, int method, double radius, const vo_volume *in,
             vo_volume **out, vo_timings *timings);

/* Many independent volumes (uneven grids, radii and ops) in one call; no
 * reference counterpart beyond calling vo_morph n times. */
int vo_morph_batched(vo_ctx *ctx, int n, const int *ops, const double *radii, int method,
                     const vo_volume *const *ins, vo_volume **outs, vo_timings *timings);

/* Batch plans (no reference counterpart): the work of vo_morph_batched with
 * VO_METHOD_FAST, split so that the planned work can be replayed. Create
 * plans the chains of every volume (erosion -> dilation for opening and
 * closing), sizes the output slots (from the attached sizer, see
 * vo_set_sizer, or a fixed capacity), orders the persistent work queue,
 * chooses the block shape with the autotuner (cached per context), and
 * captures all device steps into one CUDA graph; it keeps pointers to `ins`,
 * which must outlive the plan and keep their contents. Run replays the graph
 * and re-runs, one by one through vo_morph's path, the volumes whose output
 * overflowed its slots. Outputs returns new CSR volumes (caller frees). */
typedef struct vo_batch vo_batch;
typedef struct {
  int64_t slot_bytes;   /* output slot memory of the dilations */
  int32_t tiles;        /* work-queue items over all rounds */
  int32_t tile_rows;    /* warps (8 x 4 column patches) per block chosen by the autotuner (last round): 1, 2 or 4 */
  int32_t union_cap;    /* union slots per column of the main kernel (last round): 24, 32, 48 or 64; one holds a sentinel */
  int32_t persistent;   /* 1: one wave of blocks pulling queue items; 0: one block per item (last round) */
  int32_t regs;         /* register budget per thread of the batch kernel (last round): 64 or 80 */
  int32_t graph_nodes;  /* nodes of the captured graph */
  int32_t graph_kernels;/* kernel launches per replay */
  int32_t learned;      /* 1 when slots and queue came from a sizer */
  int32_t reruns;       /* volumes re-run by the last vo_batch_run */
  int32_t rerun_first;  /* index of the first of them (-1: none) */
  int32_t rerun_cause;  /* its overflow flags: 1 union beyond the FP64 list, 2 complement slot, 4 spill exhausted */
  double spill_peak;    /* largest fraction of a dilation's spill region used by the last run (> 1: exhausted) */
  int32_t spill_peak_round; /* its dilation round */
  double plan_ms;       /* host time of vo_batch_create */
  double tune_ms[4];    /* autotuner sample times for 1, 2, 4 rows (persistent, 64 registers, the largest union
                           capacity tried; 0: cached); [3] unused */
} vo_batch_stats;
int vo_batch_create(vo_ctx *ctx, int n, const int *ops, const double *radii, int method,
                    const vo_volume *const *ins, vo_batch **out);
int vo_batch_run(vo_ctx *ctx, vo_batch *b, vo_timings *timings);
int vo_batch_outputs(vo_ctx *ctx, vo_batch *b, vo_volume **outs);
int vo_batch_stats_get(vo_ctx *ctx, const vo_batch *b, vo_batch_stats *stats);
void vo_batch_destroy(vo_ctx *ctx, vo_batch *b);

/* Mesh -> dexels by vertical ray casting (replaces create_dexels + compute_sign,
 * Dexelize.cpp:166-274). verts[3*nv] FP64, tris[3*nt] int32 (0-based).
 * num_dexels > 0: spacing = longest bbox side / num_dexels; otherwise *spacing
 * is used as given. *spacing returns the spacing used. */
int vo_dexelize(vo_ctx *ctx, const double *verts, int nv, const int32_t *tris, int nt,
                double *spacing, int padding, int num_dexels, vo_volume **out);

/* Columns of this context's last successful vo_dexelize whose ray met the mesh
 * an odd number of times (an open or self-intersecting mesh). The reference
 * keeps such a column's odd value list (Dexelize.cpp:208-213), but every
 * consumer reads values in pairs (CompressedVolume::iterate), so its last hit
 * is never used; the CSR pairs here have no place for it and drop it. */
int vo_dexelize_odd_columns(vo_ctx *ctx, int64_t *count);

/* Segment count and enclosed volume of a volume, reduced on the device
 * (CompressedVolume::numSegments and get_volume, CompressedVolume.cpp:61-83;
 * volume in world units: spacing^3 times the summed segment lengths). */
int vo_volume_measure(vo_ctx *ctx, const vo_volume *v, int64_t *num_segments, double *volume);

/* Xor volume of two volumes on the same grid (Voronoi.cpp:91-111,
 * calculateXor's return value), computed on the device. */
int vo_xor_volume(vo_ctx *ctx, const vo_volume *a, const vo_volume *b, double *volume);

/* Allocation-free xor volume. No counterpart in the reference: the same result
 * as vo_xor_volume, for callers that must not allocate device memory while
 * they run (services whose device memory is owned by another allocator, hot
 * loops kept off the allocator). Call it from ordinary host code, not from a
 * host function enqueued on a stream, where no CUDA call is allowed. It takes
 * no context: offs_a/z_a and offs_b/z_b are the device CSR arrays of two
 * volumes on `grid` (e.g. from vo_volume_device_ptrs), all non-NULL, on the
 * current device; the work runs on `stream` (a cudaStream_t of the current
 * device, NULL for the default stream; another device's stream returns
 * VO_EINVAL), which is synchronised before *volume is written.
 * Scratch is a fixed file-scope device array of 65537 doubles (512 KiB) that
 * every GPU loading the library keeps until exit; grids with more than
 * 16,777,216 columns (nx*ny) return VO_ERANGE. The first call on each device
 * looks up that array's device address, so make it before any stream capture,
 * and do not reset the device (cudaDeviceReset) after using this function.
 * All calls share the array: calls that overlap on the GPU (different streams
 * or threads) race and must be serialised by the caller. */
int vo_xor_volume_noalloc(const vo_grid *grid, const int32_t *offs_a, const double *z_a,
                          const int32_t *offs_b, const double *z_b, void *stream, double *volume);

/* ---- 2D images (src/vor2d CompressedImage: dilate / erode / open / close,
 * CompressedImage.cpp:608-647) ----
 * An image is `height` rows of `width` pixels (1 <= width <= 50000); row i is a
 * sorted list of half-open pixel spans given as events [a0, b0, a1, b1, ...],
 * strictly increasing within [0, width], in CSR form: row_offs[height + 1]
 * counts events (the rows of CompressedImage, CompressedImage.h:32-41, and its
 * save/load layout). op: VO_DILATION, VO_EROSION, VO_OPENING, VO_CLOSING with
 * the reference's semantics (lattice disc of radius r, dy = floor(sqrt(r*r -
 * t*t)); erosion treats everything outside the image as empty). The result is
 * written to out_row_offs[height + 1] and out_events (capacity out_capacity
 * events); when that is too small, VO_ERANGE is returned with the required
 * count in out_row_offs[height]. radius in pixels, at most 1e6. */
int vo_image_morph(vo_ctx *ctx, int op, double radius, int width, int height, const int32_t *row_offs,
                   const int32_t *events, int32_t *out_row_offs, int32_t *out_events, int64_t out_capacity);

/* The FP64 twin (src/vor2d DoubleCompressedImage, DoubleCompressedImage.cpp:680-720):
 * rows of closed spans with FP64 events sorted within [0, width]. As in the
 * reference, dilation scales the radius by the row count (R = radius * height,
 * at most 255 after scaling) and erosion uses it as given; erosion treats
 * everything outside the image as empty. Output and VO_ERANGE as for
 * vo_image_morph. */
int vo_image_morph_f64(vo_ctx *ctx, int op, double radius, int width, int height, const int32_t *row_offs,
                       const double *events, int32_t *out_row_offs, double *out_events, int64_t out_capacity);

/* ---- learned sizing for vo_morph_batched (no reference counterpart) ----
 * A small MLP (16 tile features -> 64 -> 64 -> 3 outputs, ReLU, BF16 weights
 * with FP32 accumulation) predicts per 32 x 32 tile of output columns
 * log2(1 + max output segments per column), log2(1 + mean output segments)
 * and log2(1 + candidate intervals per column). When a sizer is attached to a
 * context, vo_morph_batched with VO_METHOD_FAST sizes each tile's output slots
 * from the first prediction and orders its work queue by the third; a column
 * that outgrows its slot is detected exactly and its volume re-runs through
 * vo_morph, so results never depend on the network. Training runs on the
 * device (mean squared error, Adam) with hand-written forward / backward
 * kernels. */
#define VO_SIZER_FEATURES 16
#define VO_SIZER_OUTPUTS 3
typedef struct vo_sizer vo_sizer;
/* New network with He-uniform weights drawn from `seed`. */
int vo_sizer_create(vo_ctx *ctx, uint64_t seed, vo_sizer **out);
void vo_sizer_destroy(vo_ctx *ctx, vo_sizer *s);
/* Number of FP32 parameters (W1[16][64], b1, W2[64][64], b2, W3[64][4], b3). */
int vo_sizer_num_params(void);
/* Copy parameters in (resets the optimiser state) / out. count must equal
 * vo_sizer_num_params(). */
int vo_sizer_set_params(vo_ctx *ctx, vo_sizer *s, const float *params, int count);
int vo_sizer_get_params(vo_ctx *ctx, const vo_sizer *s, float *params, int count);
/* Features [ntiles][VO_SIZER_FEATURES] of a volume's tiles for a dilation of
 * `radius`; feats == NULL returns the tile count only. */
int vo_sizer_tile_features(vo_ctx *ctx, const vo_volume *v, double radius, float *feats, int *ntiles);
/* Training targets [ntiles][VO_SIZER_OUTPUTS] from an input and its dilation. */
int vo_sizer_tile_targets(vo_ctx *ctx, const vo_volume *in, const vo_volume *result, double radius,
                          float *targets, int *ntiles);
/* Predictions [n][VO_SIZER_OUTPUTS] for host features [n][VO_SIZER_FEATURES]. */
int vo_sizer_forward(vo_ctx *ctx, const vo_sizer *s, const float *feats, int n, float *pred);
/* Gradient of the mean squared error over the n samples w.r.t. every
 * parameter (grads[vo_sizer_num_params()]) and the loss, without updating. */
int vo_sizer_gradients(vo_ctx *ctx, vo_sizer *s, const float *feats, const float *targets, int n,
                       float *grads, float *loss);
/* `steps` full-batch Adam steps at learning rate lr; *final_loss (may be NULL)
 * is the loss after the last step. */
int vo_sizer_train(vo_ctx *ctx, vo_sizer *s, const float *feats, const float *targets, int n, int steps,
                   float lr, float *final_loss);
/* Attach (s != NULL) or detach (NULL) a sizer used by vo_morph_batched. The
 * context does not own it. */
int vo_set_sizer(vo_ctx *ctx, vo_sizer *s);

#ifdef __cplusplus
}
#endif
#endif
