// internal.h -- structures shared by the host side and the kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/aloha.h"

namespace aloha {

// Padded brick storage: every brick is stored with an apron of kApron voxels
// on each side, filled with the clamped edge values (cudaAddressModeClamp of
// waikikiRenderer.cpp:753-755), so the march loop needs no per-tap clamps.
// Each stored element is a yz-quad: the float4 (V(x,y,z), V(x,y+1,z),
// V(x,y,z+1), V(x,y+1,z+1)) (indices clamped), so one 16-byte load fetches a
// voxel's 2x2 (y, z) neighbourhood and the stencil's core comes from three
// neighbouring elements of one row (x-quads, V(x..x+3), took the same bytes
// from four rows and hit L1 less often).  Quads cut the loads per sample from
// 20 to 7 at four times the HBM footprint.
constexpr int kApron = 2;
constexpr int kMaxViews = 4096;
constexpr int kMaxTF = 2048;  // (n + 4) float4 entries stay under 48 KB of shared memory

// Empty-space macrocells: kMacro^3 voxels; a sample whose value-tap cell lies
// in an empty macrocell has transfer-function alpha exactly 0.
constexpr int kMacroShift = 3;
constexpr int kMacro = 1 << kMacroShift;

// One brick as the kernels see it (72 bytes).
struct DevBrick {
  const float4* base;    // yz-quad of voxel (0,0,0) of the voxel range inside the padded array
  const uint8_t* empty;  // [mz][my][mx] 1 = every sample there has alpha 0 (null: no skipping)
  int sy, sz;            // padded row and slice pitch, in quads
  int n[3];              // voxel range size
  float lo[3];           // voxelRange.lower (voxel-unit origin of the brick)
  float space_lo[3], space_hi[3];
};

// Per-view state read by the kernels.
struct DevView {
  float org[3], dir_00[3], dir_du[3], dir_dv[3];
  int width, height;
  float max_depth;
  int n_ranks;
  int sched;          // offset of the view's schedule in the schedule buffer:
                      // [rank_order n_ranks][rank_start n_ranks+1][rank_bricks n_bricks]
  int pixel_offset;   // offset of the view's first pixel in batched outputs
  int rects;          // offset of the ranks' screen rectangles in the schedule buffer:
                      // per rank [cx0, cy0, cx1, cy1] in 8x4 chunks, inclusive
  int pad;
};

// Everything one render launch needs, passed by value.
struct FrameArgs {
  const DevBrick* bricks;
  const DevView* views;
  const int* sched;
  const float4* tf;
  int n_tf;
  float dt, et_alpha;
  int jitter_mode;
  float jitter_value;
  int crosshair, spp, accum_id, accumulate, heat_map;
  float heat_map_scale;
  int composite_mode, island_id, num_islands;
  // outputs
  uint32_t* fb;                 // [H*W] (single view) RGBA8
  float4* rank_images;          // [n_ranks][H*W] or null
  float* rank_depth;            // [n_ranks][H*W] or null
  float4* accum;                // [n_ranks][H*W] or null
  unsigned long long* counter;  // total samples (atomic) or null
};

// One persistent render launch over a list of (view, output) items: warps
// pull pixel chunks from an atomic work counter.  A single view leaves
// view_ids, fbs and tile_prefix null and uses single_view and f.fb.
struct BatchArgs {
  FrameArgs f;
  const int* view_ids;       // [n_items] view of each batch item
  uint32_t* const* fbs;      // [n_items] output frame buffers (device)
  const int* tile_prefix;    // [n_items+1] prefix sum of chunks per item
  int n_items;
  int single_view;
  int total_tiles;           // chunks in the launch
  unsigned int* work_counter;
  const int* chunk_order;    // single view: chunk ids in the order to render them, or null (ring order)
  int group_chunks;          // single view in cost order: the first group_chunks chunks of chunk_order are
                             // rendered by lane groups (kLaneGroup lanes per ray), as kLaneGroup items each
};

// Lanes per ray of the lane-group render (march_brick_group).
constexpr int kLaneGroup = 4;

// Cost-ordered chunks of one view (schedule.cu): a coarse probe per chunk
// estimates its cost, and the chunks are sorted stably by cost class, most
// expensive first, so the frame does not end on a long chunk started last.
constexpr int kOrderClasses = 64;  // cost classes, a quarter octave apart
struct ChunkOrderArgs {
  FrameArgs f;
  int view;
  int cw, ch;        // chunk shape
  int n_slots;       // ring slots of the chunk grid (the probe's input order)
  uint8_t* key;      // [n_slots] cost class per slot (0xff off the grid)
  int* cid;          // [n_slots] chunk id per slot
  uint32_t* hist;    // [kOrderClasses][chunk_order_blocks(n_slots)] counts, then offsets; zero between launches
  int* order;        // [chunks] chunk ids, most expensive first
  int n_chunks;      // chunks of the grid (entries of `order`)
  // counters of the render launch that follows, zeroed by the probe (or null)
  unsigned int* zero_work;
  unsigned long long* zero_samples;
};
int chunk_order_blocks(int n_slots);
cudaError_t launch_chunk_order(const ChunkOrderArgs& a, cudaStream_t s);

// Rank-split render of one view into f.fb: work items are (8x4 chunk, rank)
// pairs for the ranks whose screen rectangle covers the chunk; f.rank_images
// is the scratch plane set [n_ranks][H*W] of the marched ranks.  At most
// kSplitMaxRanks ranks (one mask bit each).
constexpr int kSplitMaxRanks = 64;
constexpr uint32_t kSplitBackground = 127u;  // item code of a chunk no rank covers
struct SplitArgs {
  FrameArgs f;
  int view;
  int n_slots;                     // work positions: ring slots of 8x4 chunks, or chunks when ordered (< 2^25)
  const int* chunk_order;          // chunk ids by position (cost order), or null (ring order)
  unsigned long long* masks;       // [n_slots] covering ranks per slot
  uint32_t* offsets;               // [n_slots] first item of each slot
  uint32_t* block_sums;            // [ceil(n_slots / 1024)] scan scratch
  uint32_t* items;                 // [n_slots * max(1, n_ranks)] slot << 7 | rank position
  uint32_t* n_items;               // items listed (written by the plan kernel)
  unsigned int* chunk_done;        // [n_slots] tickets, zero between launches
  unsigned int* work_counter;
};

// Chunk shapes (pixels a warp takes per work-counter grab, rendered as 8x4
// sub-tiles): 8x4, 8x8, 16x8 or 32x4.
inline bool known_chunk(int w, int h) {
  return (w == 8 && h == 4) || (w == 8 && h == 8) || (w == 16 && h == 8) || (w == 32 && h == 4);
}
// Chunks are handed out centre-out, in square rings around the image centre
// (the longest rays usually cross the middle, so they start first and the
// frame's tail is short).  Work slots cover the smallest odd square of rings
// that contains the chunk grid; slots outside the grid are skipped.
__host__ __device__ inline int ring_radius(int cxn, int cyn) {
  const int cx = (cxn - 1) / 2, cy = (cyn - 1) / 2;
  int r = cx > cxn - 1 - cx ? cx : cxn - 1 - cx;
  const int ry = cy > cyn - 1 - cy ? cy : cyn - 1 - cy;
  return r > ry ? r : ry;
}
__host__ __device__ inline int ring_slots(int width, int height, int cw, int ch) {
  const int r = ring_radius((width + cw - 1) / cw, (height + ch - 1) / ch);
  return (2 * r + 1) * (2 * r + 1);
}
constexpr int kRenderThreads = 128;
cudaError_t launch_composite_f32(const float4* imgs, const int* order, int n_ranks, int npx, int mode, uint32_t* fb,
                                 cudaStream_t s);
cudaError_t launch_composite_u8(const uint32_t* imgs, const int* order, int n_ranks, int npx, uint32_t* fb,
                                cudaStream_t s);
cudaError_t launch_pad_brick(const float* src, int nx, int ny, int nz, float4* dst_alloc, int px, int py, int pz,
                             int* nonfinite_flag, cudaStream_t s);
// Persistent render launch; `batch` selects the instance tuned for batches.
constexpr int kSingleRenderBlocks = 5, kBatchRenderBlocks = 7;  // CTAs per SM
// CTAs per SM of the differentiable form's forward (checkpointed march): a
// launch of few chunks ends on its longest rays and runs faster with fewer,
// faster warps; one of at least kTrainManyChunksPerWarp chunks per resident
// warp is throughput-bound and runs faster with more.
constexpr int kTrainForwardBlocks = 5, kTrainForwardBlocksMany = 7;
constexpr int kTrainManyChunksPerWarp = 16;
// `stage`: ALOHA_STAGING_NONE or _NEXT_SAMPLE (the stencil loads), or, for
// batches, kStageUnroll2: direct loads with the march loop written out two
// steps per trip.
constexpr int kStageUnroll2 = 2;
// `lane_groups`: the instance that renders the first a.group_chunks chunks of
// the cost order with lane groups (single view, 8x4 chunks, direct loads).
cudaError_t launch_render_warps(const BatchArgs& a, int chunk_w, int chunk_h, int grid, bool batch, cudaStream_t s,
                                int stage = ALOHA_STAGING_NONE, bool lane_groups = false);
cudaError_t launch_macrocell_range(const DevBrick& b, float2* out, cudaStream_t s);
cudaError_t launch_macrocell_empty(const float2* ranges, int count, const int* prefix, int n, uint8_t* empty,
                                   cudaStream_t s);
inline int macrocells(const DevBrick& b) {
  return ((b.n[0] + kMacro - 1) >> kMacroShift) * ((b.n[1] + kMacro - 1) >> kMacroShift) *
         ((b.n[2] + kMacro - 1) >> kMacroShift);
}
// CTAs of the render kernel that fit on one SM for a chunk shape (0 if the shape is unknown).
int render_blocks_per_sm(int chunk_w, int chunk_h, int n_tf, bool batch, int stage = ALOHA_STAGING_NONE,
                         bool lane_groups = false);
// `many_ranks` selects the instance tuned for many short (chunk, rank) items.
constexpr int kManyRankSplitBlocks = 7;  // CTAs per SM
cudaError_t launch_render_split(const SplitArgs& a, int grid, bool many_ranks, cudaStream_t s);
int render_split_blocks_per_sm(int n_tf, bool many_ranks);

}  // namespace aloha
