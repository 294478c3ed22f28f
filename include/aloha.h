/*
 * aloha.h -- C ABI of the GB300 volume hot path (one GPU, bricks as virtual ranks).
 *
 * Replaces, for the volume path only:
 *   - the renderer host API mpi::DistributedRenderer / maui::Renderer
 *     (DistributedRenderer.h:29-71, waikikiRenderer.h:28-118): camera, resize,
 *     colour map and render(fb) events;
 *   - the OWL launch of the raygen renderFrame (waikikiRenderer.cpp:1021-1028,
 *     deviceCode.cpp:340-421) with the brick march integrateBrick
 *     (deviceCode.cpp:256-298);
 *   - the IceT ordered BLEND composite of the per-rank images
 *     (waikikiRenderer.cpp:895-917,1030-1079).
 *
 * Conventions: every call returns an aloha_status (0 = ALOHA_OK); the library
 * never exits or traps.  Pointers may be host or device memory unless stated;
 * when an output is host memory the call copies into it and returns after the
 * stream has finished.  `stream` is a cudaStream_t (NULL = default stream).
 * Calls on one context are not thread-safe and must not overlap on the GPU
 * (the reference's renderer is single-threaded per rank as well).
 */
#ifndef ALOHA_GB300_ALOHA_H
#define ALOHA_GB300_ALOHA_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ALOHA_ABI_VERSION 1

typedef enum {
  ALOHA_OK = 0,
  ALOHA_ERR_INVALID_ARGUMENT = 1, /* bad size, NaN camera, bad enum value */
  ALOHA_ERR_NULL_POINTER = 2,
  ALOHA_ERR_OUT_OF_RANGE = 3,     /* view / brick / rank index out of range */
  ALOHA_ERR_NOT_READY = 4,        /* no bricks, transfer function or camera yet */
  ALOHA_ERR_OUT_OF_MEMORY = 5,    /* request larger than free device memory */
  ALOHA_ERR_CUDA = 6,             /* a CUDA runtime call failed (see aloha_last_error) */
  ALOHA_ERR_TIMEOUT = 7,          /* a bounded device-side wait gave up */
  ALOHA_ERR_MISSING_BRICK = 8,    /* a virtual rank has no data (brick never uploaded) */
  ALOHA_ERR_UNSUPPORTED = 9
} aloha_status;

enum { ALOHA_JITTER_NONE = 0, ALOHA_JITTER_CONST = 1, ALOHA_JITTER_HASH = 2 };
enum { ALOHA_COMPOSITE_FP32 = 0, ALOHA_COMPOSITE_UBYTE = 1 };
enum { ALOHA_ORDER_FACES = 0, ALOHA_ORDER_REFERENCE_KD = 1 };
enum { ALOHA_SPLIT_AUTO = 0, ALOHA_SPLIT_PIXELS = 1, ALOHA_SPLIT_RANKS = 2 };
enum { ALOHA_CHUNKS_AUTO = 0, ALOHA_CHUNKS_RING = 1, ALOHA_CHUNKS_PROBED = 2 };
enum { ALOHA_STAGING_NONE = 0, ALOHA_STAGING_NEXT_SAMPLE = 1 };

typedef struct aloha_ctx aloha_ctx;

/* One brick, byte-identical to a .vol brick header (chopSuey.cpp:342-345,
 * read at waikikiRenderer.cpp:615-618; VolBrick fields deviceCode.h:35-50):
 * cellRange, voxelRange (half-open, with chopSuey's upper ghost layer),
 * spaceRange (voxel units), valueRange. */
typedef struct {
  int32_t cell_lo[3], cell_hi[3];
  int32_t voxel_lo[3], voxel_hi[3];
  float space_lo[3], space_hi[3];
  float value_range[2];
} aloha_brick_desc;

/* Render settings (LaunchParams::render, deviceCode.h:90-95, plus the values
 * the reference hard-codes: dt = 2 at waikikiRenderer.cpp:1023, ET .99 at
 * deviceCode.cpp:270,391, crosshair always on at deviceCode.cpp:410-414). */
typedef struct {
  float dt;               /* step along the ray in voxels */
  float et_alpha;         /* early ray termination threshold */
  int32_t jitter_mode;    /* ALOHA_JITTER_*: ils_t0 = 0, jitter_value, or a hash of (pixel, accum_id, draw) */
  float jitter_value;
  int32_t crosshair;      /* invert column W/2 and row H/2 of each rank image */
  int32_t spp;            /* samples per pixel (repeat the march, new jitter draws) */
  int32_t accum_id;       /* progressive frame index; > 0 adds the accumulation buffer */
  int32_t accumulate;     /* keep a per-view, per-rank float4 accumulation buffer */
  int32_t heat_map;       /* blend a heat map of per-pixel sample counts */
  float heat_map_scale;
  int32_t composite_mode; /* ALOHA_COMPOSITE_FP32 (one rounding) or _UBYTE (RGBA8 blend, IceT-style) */
  int32_t island_id;      /* image-parallel islands: 16x16 tiles with tile % num_islands == island_id */
  int32_t num_islands;
  int32_t order_mode;     /* ALOHA_ORDER_FACES or _REFERENCE_KD (midplane KD of partitionKD) */
} aloha_render_params;

typedef struct {
  uint64_t samples;       /* march loop-body executions of the last render/batch call */
  int32_t n_bricks;
  int32_t n_ranks;
  uint64_t brick_bytes;   /* device bytes held for bricks (padded layout) */
} aloha_stats;

int aloha_abi_version(void);
const char* aloha_status_string(int status);

/* Context = one renderer on one GPU (replaces maui::Renderer's constructor,
 * waikikiRenderer.cpp:344-846, minus MPI/IceT/OWL set-up). */
int aloha_create(int device, aloha_ctx** out);
int aloha_destroy(aloha_ctx* ctx);
const char* aloha_last_error(const aloha_ctx* ctx);

int aloha_default_render_params(aloha_render_params* out);
int aloha_set_render_params(aloha_ctx* ctx, const aloha_render_params* params);

/* Upload `n` bricks (replaces the brick upload of waikikiRenderer.cpp:637-777).
 * voxels[i] holds brick i's voxel range, x fastest, float32 (host or device).
 * The library keeps its own device copy.  Resets the rank partition to one
 * rank per brick: partitionKD's numbering, or brick i -> rank i for brick sets
 * partitionKD cannot split (see aloha_set_ranks); frames are the same. */
int aloha_set_bricks(aloha_ctx* ctx, const aloha_brick_desc* descs, const float* const* voxels, int n);

/* Replace one brick's voxels (same voxel range), e.g. after a density update. */
int aloha_update_brick(aloha_ctx* ctx, int brick, const float* voxels);

/* Mark one brick's data as lost (a virtual rank that went away): renders
 * return ALOHA_ERR_MISSING_BRICK instead of an image without that brick,
 * until aloha_update_brick supplies the data again.  No reference
 * counterpart: the reference has no failure handling (Headless.cpp:52-57). */
int aloha_drop_brick(aloha_ctx* ctx, int brick);

/* Transfer function: n RGBA float entries (handleColorMapEvent,
 * waikikiRenderer.cpp:945-1013). */
int aloha_set_transfer_function(aloha_ctx* ctx, const float* rgba, int n);

/* Virtual ranks: partitionKD of the bricks over n_ranks ranks
 * (waikikiRenderer.cpp:150-270, called at 630-631), or an explicit
 * assignment brick -> rank.  partitionKD splits a group at the midplane of
 * its bounds' longest axis; where the bricks of a group are separated only
 * along a shorter axis that split makes no progress (the reference repeats it
 * forever) and aloha_set_ranks returns ALOHA_ERR_INVALID_ARGUMENT: use
 * aloha_set_rank_assignment for such brick sets. */
int aloha_set_ranks(aloha_ctx* ctx, int n_ranks);
int aloha_set_rank_assignment(aloha_ctx* ctx, const int* brick_rank, int n_bricks, int n_ranks);

/* Per-view camera and size (handleCameraEvent / handleResizeEvent,
 * waikikiRenderer.cpp:853-920).  Views are numbered 0..4095. */
int aloha_set_camera(aloha_ctx* ctx, int view, const float* org, const float* dir_00, const float* dir_du,
                     const float* dir_dv);
int aloha_resize(aloha_ctx* ctx, int view, int width, int height);

/* Front-to-back rank order for a view (computeCompositeOrder,
 * waikikiRenderer.cpp:281-316, or the face-based order). */
int aloha_get_composite_order(aloha_ctx* ctx, int view, int* rank_order, int max_ranks, int* n_ranks);

/* Pixel chunk a warp of the persistent render takes per grab (rendered as
 * 8x4-pixel sub-tiles): 8x4, 8x8, 16x8 or 32x4; 0x0 (the default) is 8x4,
 * which ends a frame soonest after its slowest chunk.  No reference
 * counterpart (the raygen launches one thread per pixel). */
int aloha_set_render_tile(aloha_ctx* ctx, int tile_w, int tile_h);

/* How aloha_render divides a frame among warps.  ALOHA_SPLIT_PIXELS: one
 * thread marches every virtual rank of its pixel and blends them (the chunk
 * shape above applies).  ALOHA_SPLIT_RANKS: a work item is one 8x4-pixel
 * chunk of one rank whose projected bricks cover the chunk, so the bricks
 * along a ray are marched in parallel; rank images go through a scratch plane
 * set of n_ranks*width*height float4 and the last rank of each chunk blends
 * it.  Both give bit-identical frames.  The rank split needs 2..64 virtual
 * ranks and at most 16 GiB of scratch (else ALOHA_ERR_UNSUPPORTED);
 * aloha_render_partials and a single rank always use the pixel split.
 * ALOHA_SPLIT_AUTO (the default) takes the rank split from 32 virtual ranks
 * up (when it applies) and the pixel split below.  No reference counterpart
 * (each reference rank is its own process). */
int aloha_set_render_split(aloha_ctx* ctx, int mode);

/* The order in which warps take the chunks of a single-view render (and of
 * the rank split's (chunk, rank) items, and of aloha_forward).
 * ALOHA_CHUNKS_RING: centre-out square rings.  ALOHA_CHUNKS_PROBED:
 * most expensive first, by a coarse probe of each chunk's centre ray through
 * the empty-space tables (two small kernels before the render), so that the
 * frame does not end on a long chunk started late.  Frames are bit-identical
 * either way.  ALOHA_CHUNKS_AUTO (the default) probes frames of 512^2 pixels
 * or more, except for the rank split from 32 virtual ranks up (its items are
 * short already).  No reference counterpart. */
int aloha_set_chunk_order(aloha_ctx* ctx, int mode);

/* Where the single-view render kernel takes each sample's stencil rows from:
 * ALOHA_STAGING_NONE (the default) loads them from the brick when the sample
 * is evaluated; ALOHA_STAGING_NEXT_SAMPLE copies the next sample's rows into
 * the thread's own shared-memory slots with cp.async while the current
 * sample is evaluated (double buffering, 24 KB of shared memory per CTA).
 * Frames are bit-identical either way.  No reference counterpart (the
 * reference samples 3D textures, deviceCode.cpp:279-289). */
int aloha_set_render_staging(aloha_ctx* ctx, int mode);

/* Sample-parallel lane groups for the costliest chunks of a single-view
 * render: the first `permille` / 1000 of the cost order's 8x4 chunks are
 * rendered with 4 lanes per ray (each lane evaluates one of 4 consecutive
 * samples; the samples are composited in order, so frames and sample counts
 * are bit-identical), which shortens the frame's longest chunks.  Applies to
 * cost-ordered frames (ALOHA_CHUNKS_PROBED or automatic from 512^2) with the
 * 8x4 chunk, direct stencil loads and a frame buffer only (not to
 * aloha_render_partials, accumulation or the rank split).  0 (the default)
 * is off.  No reference counterpart (one OptiX thread per pixel). */
int aloha_set_lane_groups(aloha_ctx* ctx, int permille);

/* Render one view into an RGBA8 frame buffer of width*height uint32
 * (Renderer::render, waikikiRenderer.cpp:1015-1080): all virtual ranks march
 * their bricks and their images are composited in one fused kernel.  fb may
 * be device memory, page-locked host memory (cudaHostAlloc / cudaMallocHost:
 * the kernel writes it directly) or pageable host memory (copied from a
 * device staging buffer); with host memory the call returns once the frame
 * is there. */
int aloha_render(aloha_ctx* ctx, int view, uint32_t* fb, void* stream);

/* The unfused form: per-rank images after renderFrame's output stage
 * (float RGBA, [n_ranks][height][width][4], indexed by rank id) and per-rank
 * depth ([n_ranks][height][width], fbDepth of deviceCode.cpp:388,397;
 * may be NULL). */
int aloha_render_partials(aloha_ctx* ctx, int view, float* rank_images, float* rank_depth, void* stream);

/* IceT stand-in: blend n_ranks float RGBA images front to back in `order`
 * (ordered BLEND, waikikiRenderer.cpp:910-917,1042-1079) into RGBA8.  Mode
 * ALOHA_COMPOSITE_FP32 blends in fp32 and rounds once; _UBYTE quantises each
 * image first and blends in 8 bits.  Context-free. */
int aloha_composite_over(const float* rank_images, const int* order, int n_ranks, int width, int height,
                         int mode, uint32_t* fb, void* stream);

/* IceT stand-in for external RGBA8 rank images ([n_ranks][height][width]
 * uint32, premultiplied), blended in 8 bits front to back in `order`. */
int aloha_composite_over_rgba8(const uint32_t* rank_fbs, const int* order, int n_ranks, int width, int height,
                               uint32_t* fb, void* stream);

/* The ordered composite of aloha_composite_over for callers that cannot
 * allocate device memory during the call (for example a compositing stage
 * inside another library's frame loop whose memory pool forbids new
 * allocations, or a real-time host that bans allocation after start-up).  No
 * reference counterpart.  It allocates nothing: the composite order is staged
 * in a 16 KB device array compiled into the library (held by every GPU that
 * loads it until exit), whose address is looked up on the first call made on
 * each device.  It cannot be recorded into a CUDA graph: on a capturing
 * stream it returns ALOHA_ERR_UNSUPPORTED and leaves the capture untouched.
 * rank_images and fb must be device memory of the current device, order host
 * memory; at most 4096 ranks (else ALOHA_ERR_OUT_OF_RANGE).  The call reads
 * `order` once into a private host snapshot, checks it and copies the
 * snapshot, so the caller may change or free its buffer as soon as the call
 * returns; that copy is from pageable memory, so the call first waits for the
 * stream's earlier work.  Calls share the staging array, so calls that
 * overlap on the GPU race: use one stream or wait in between. */
int aloha_composite_over_noalloc(const float* rank_images, const int* order, int n_ranks, int width, int height,
                                 int mode, uint32_t* fb, void* stream);

int aloha_get_stats(aloha_ctx* ctx, aloha_stats* out);

/* ---- Batched form: many views in one persistent launch (no reference
 * counterpart; the reference renders one camera per launch,
 * waikikiRenderer.cpp:1028).  A batch fixes a list of (view, device frame
 * buffer) items; aloha_batch_launch only enqueues kernels and memsets, so it
 * can be captured into a CUDA graph; aloha_batch_launch_graph captures it
 * once and replays the graph.  Camera changes of the batch's views are picked
 * up at the next launch. */
typedef struct aloha_batch aloha_batch;

int aloha_batch_create(aloha_ctx* ctx, const int* views, int n_items, uint32_t* const* fbs, aloha_batch** out);
/* Ray-tile shape of the persistent kernel: 8x4, 8x8, 16x8 or 32x4 pixels per
 * warp chunk; ctas_per_sm = 0 picks the occupancy limit. */
int aloha_batch_set_config(aloha_batch* b, int tile_w, int tile_h, int ctas_per_sm);
int aloha_batch_get_config(const aloha_batch* b, int* tile_w, int* tile_h, int* ctas_per_sm);
/* Stencil staging of the batch kernel (ALOHA_STAGING_*, as
 * aloha_set_render_staging). */
int aloha_batch_set_staging(aloha_batch* b, int stage);
int aloha_batch_get_staging(const aloha_batch* b, int* stage);

/* March steps per loop trip of the batch's render kernel: 1 (default) or 2,
 * the march loop written out two steps per trip (direct stencil loads only;
 * with ALOHA_STAGING_NEXT_SAMPLE the setting is kept but not used).  Frames
 * are bit-identical.  No reference counterpart (the step-unroll axis of the
 * batch autotuner, which sweeps it with the chunk shape and the staging). */
int aloha_batch_set_unroll(aloha_batch* batch, int steps);
int aloha_batch_get_unroll(const aloha_batch* batch, int* steps);

int aloha_batch_launch(aloha_batch* b, void* stream);
int aloha_batch_launch_graph(aloha_batch* b, void* stream);
/* Time every tile shape with direct loads, direct loads two steps per trip,
 * and staged loads (`reps` launches each, CUDA events) and keep the fastest;
 * returns its shape and mean milliseconds per launch
 * (aloha_batch_get_staging and aloha_batch_get_unroll give the rest). */
int aloha_batch_autotune(aloha_batch* b, void* stream, int reps, int* tile_w, int* tile_h, float* ms);
int aloha_batch_destroy(aloha_batch* b);

/* Convenience: render n views (fbs may be host or device) in one batched
 * launch and wait for it. */
int aloha_render_batch(aloha_ctx* ctx, const int* views, int n_items, uint32_t* const* fbs, void* stream);

/* ---- Differentiable form (no reference counterpart).  Needs one virtual
 * rank (aloha_set_ranks(ctx, 1)), spp 1, accum_id 0, no accumulation,
 * crosshair, heat map or islands; otherwise ALOHA_ERR_UNSUPPORTED.
 *
 * aloha_forward renders `view` into float RGBA (premultiplied, before
 * quantisation; [height][width][4], host or device), bit-identical to the
 * frame aloha_render composites, and keeps a checkpoint of the march state
 * every `checkpoint_every` samples for the view's next aloha_backward. */
int aloha_forward(aloha_ctx* ctx, int view, float* rgba, int checkpoint_every, void* stream);

/* aloha_forward of views[0..n_views) in one persistent launch: rgba[i]
 * receives views[i]'s image (host or device), and each view keeps the
 * checkpoints its aloha_backward / aloha_backward_views needs; images and
 * checkpoints are those of n aloha_forward calls, bit for bit.  Each view at
 * most once.  Views small enough to leave part of the GPU idle (a 256^2 frame
 * has fewer 8x4 chunks than a GB300 holds warps) gain most. */
int aloha_forward_views(aloha_ctx* ctx, int n_views, const int* views, float* const* rgba, int checkpoint_every,
                        void* stream);

/* Gradient of a loss L with respect to the transfer function and the voxel
 * densities, given dL/dRGBA of the last aloha_forward of `view`
 * ([height][width][4] float).  Accumulates (+=) into dl_dtf ([n_tf][4]) and
 * into dl_ddensity, a float grid [dims z][dims y][dims x] whose voxel (0,0,0)
 * is grid_lo; every brick's voxel range must lie inside it, and the grid may
 * hold at most 2^40 voxels in at most 2^31 - 1 (y, z) rows (else
 * ALOHA_ERR_OUT_OF_RANGE, before anything is allocated).  Ghost voxels and
 * clamped edge taps add into the voxel they copy.  Host or device buffers.
 * dl_dtf may be NULL: only the density gradient is computed, and the replay
 * then skips empty macrocells (their samples have transfer-function alpha 0,
 * so they contribute to the alpha entries of dl_dtf only).  dl_ddensity may
 * be NULL (grid_lo and grid_dims are then ignored): only the transfer-function
 * gradient is computed, without the shading and stencil adjoints.  At least
 * one of the two must be given (else ALOHA_ERR_NULL_POINTER). */
int aloha_backward(aloha_ctx* ctx, int view, const float* dl_drgba, float* dl_dtf, float* dl_ddensity,
                   const int* grid_lo, const int* grid_dims, void* stream);

/* aloha_backward of several views, summed: dl_dtf and dl_ddensity receive the
 * sum over views[0..n_views) of each view's gradient, with dl_drgba[i] the
 * dL/dRGBA of views[i] (each view at most once, each with a current
 * aloha_forward).  Same arguments and rules as aloha_backward otherwise.  The
 * views' replays accumulate into one device buffer that is folded into the
 * density grid once (the fold leaves it clear for the next call), their checkpoint-overflow flags are read with
 * one host wait, and one persistent launch replays every view's segments, so
 * n views cost less than n calls of aloha_backward.  The views may have been
 * forwarded with different checkpoint intervals.
 * The sum is taken in a different order than n calls would take it (float
 * atomics), so results agree with those calls to rounding. */
int aloha_backward_views(aloha_ctx* ctx, int n_views, const int* views, const float* const* dl_drgba,
                         float* dl_dtf, float* dl_ddensity, const int* grid_lo, const int* grid_dims,
                         void* stream);

#ifdef __cplusplus
}
#endif

#endif /* ALOHA_GB300_ALOHA_H */
