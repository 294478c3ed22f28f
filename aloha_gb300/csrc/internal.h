// internal.h -- structures shared by the host side and the kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/aloha.h"

namespace aloha {

// Padded brick storage: every brick is stored with an apron of kApron voxels
// on each side, filled with the clamped edge values (cudaAddressModeClamp of
// waikikiRenderer.cpp:753-755), so the march loop needs no per-tap clamps.
constexpr int kApron = 2;
constexpr int kMaxViews = 4096;
constexpr int kMaxTF = 2048;  // (n + 4) float4 entries stay under 48 KB of shared memory

// Empty-space macrocells: kMacro^3 voxels; a sample whose value-tap cell lies
// in an empty macrocell has transfer-function alpha exactly 0.
constexpr int kMacroShift = 3;
constexpr int kMacro = 1 << kMacroShift;

// One brick as the kernels see it (72 bytes).
struct DevBrick {
  const float* base;     // voxel (0,0,0) of the voxel range inside the padded array
  const uint8_t* empty;  // [mz][my][mx] 1 = every sample there has alpha 0 (null: no skipping)
  int sy, sz;            // padded row and slice pitch, in floats
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
  int pad[2];
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
  uint32_t* pixel_samples;      // [H*W] or null
  unsigned long long* counter;  // total samples (atomic) or null
};

// Batched launch: a list of (view, output) pairs processed by one persistent
// kernel, ray tiles handed out through an atomic work counter.
struct BatchArgs {
  FrameArgs f;
  const int* view_ids;       // [n_items] view of each batch item
  uint32_t* const* fbs;      // [n_items] output frame buffers (device)
  const int* tile_prefix;    // [n_items+1] prefix sum of ray tiles per item
  int n_items;
  int total_tiles;
  unsigned int* work_counter;
};

cudaError_t launch_render(const FrameArgs& a, int view, int width, int height, cudaStream_t s);
cudaError_t launch_composite_f32(const float4* imgs, const int* order, int n_ranks, int npx, int mode, uint32_t* fb,
                                 cudaStream_t s);
cudaError_t launch_composite_u8(const uint32_t* imgs, const int* order, int n_ranks, int npx, uint32_t* fb,
                                cudaStream_t s);
cudaError_t launch_pad_brick(const float* src, int nx, int ny, int nz, float* dst_alloc, int px, int py, int pz,
                             int* nonfinite_flag, cudaStream_t s);
cudaError_t launch_render_batch(const BatchArgs& a, int tile_w, int tile_h, int grid, cudaStream_t s);
cudaError_t launch_macrocell_range(const DevBrick& b, float2* out, cudaStream_t s);
cudaError_t launch_macrocell_empty(const float2* ranges, int count, const int* prefix, int n, uint8_t* empty,
                                   cudaStream_t s);
inline int macrocells(const DevBrick& b) {
  return ((b.n[0] + kMacro - 1) >> kMacroShift) * ((b.n[1] + kMacro - 1) >> kMacroShift) *
         ((b.n[2] + kMacro - 1) >> kMacroShift);
}
// CTAs of the batched kernel that fit on one SM for a tile shape (0 if the shape is unknown).
int batch_blocks_per_sm(int tile_w, int tile_h, int n_tf);

}  // namespace aloha
