// adjoint.h -- structures of the differentiable form (forward with
// checkpoints, segment-parallel backward).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "internal.h"

namespace aloha {

// March state before sample m*K of a pixel (32 bytes).
struct Checkpoint {
  float r, g, b, a;  // colour before the sample
  float t;           // ray parameter of the sample
  float tmin;        // ray tmin at the start of the current brick
  uint32_t jd;       // brick walk position (low 16 bits) | next jitter draw (high 16 bits)
  uint32_t nb;       // samples already taken in the current brick
};

// One view of a training forward or backward launch.
struct TrainView {
  Checkpoint* ckpt;           // [npx][ckpt_cap]
  float4* final_rgba;         // [npx] final colour of the forward
  float4* out_rgba;           // forward: [npx] caller's image, or null
  const float4* dl_drgba;     // backward: [npx] dL/dRGBA
  uint2* work;                // [work_cap] (pixel, segment) items the forward appends
  unsigned* work_count;       // [0] items appended
  int* overflow;              // set when a pixel needs more checkpoints than ckpt_cap
  const int* chunk_order;     // forward: 8x4 chunk ids in the order to march them, or null (ring order)
  unsigned ckpt_cap;          // checkpoints per pixel
  unsigned work_cap;
  int n_chunks;               // forward: chunk positions of the view (chunk_order entries or ring slots)
  int view;                   // index into views
};

// A run of forward positions: positions [p0, next run's p0) of the `active`
// first views of run_views, items [item0, next run's item0).
struct TrainRun {
  int p0, active;
  unsigned item0, pad;
};

struct TrainArgs {
  const DevBrick* bricks;
  const DevView* views;
  const int* sched;
  const float4* tf;
  int n_tf;
  float dt, et_alpha;
  int jitter_mode;
  float jitter_value;
  int accum_id;
  unsigned k;                 // checkpoint interval (samples) of every view of the launch
  const TrainView* tv;        // [n_views] the launch's views
  int n_views;
  // Forward: the views in run_views (by chunk positions, descending) are
  // marched position-major: position p of every view that has one, then
  // p + 1, so every view's first (costliest, or central) chunks start first.
  // runs[0..n_runs] (the last one a sentinel holding the item count).
  const TrainRun* runs;
  int n_runs;
  const int* run_views;
  // Backward: items [item_base[v], item_base[v+1]) are view slot v's
  // (pixel, segment) items; item_base[n_views] is the launch's item count.
  const unsigned* item_base;
  unsigned* grab;             // the launch's item counter (zero before it)
  // Backward of one view (n_views == 1): the view itself and its item count,
  // in the launch parameters instead of tv / item_base.
  TrainView one;
  unsigned one_items;
  float* dtf;                 // [n_tf*4] accumulated
  float4* dgrid4;             // density gradient in x-quads: element (x,y,z) holds the
                              // contributions to voxels x, x+1, x+2 (w unused)
  const int4* brick_grid_origin;  // per brick: voxelRange.lower - grid_lo
  int grid_dims[3];
  unsigned long long* counter;
};

// One persistent training forward over the launch's views (a.tv, a.runs).
// `many` selects the instance for launches of many chunks per resident warp
// (kTrainForwardBlocksMany CTAs per SM instead of kTrainForwardBlocks).
cudaError_t launch_forward_train(const TrainArgs& a, unsigned items, int max_grid, bool many, cudaStream_t s);
int forward_train_blocks_per_sm(int n_tf, bool many);
// One persistent backward over the launch's views' items (a.tv, a.item_base).
cudaError_t launch_backward(const TrainArgs& a, int grid, cudaStream_t s);
// out[v] += quads[v].x + quads[v-1].y + quads[v-2].z along x, for a grid of
// dims; every quad of the grid is zero afterwards.
cudaError_t launch_fold_quads(float4* quads, float* out, const int dims[3], cudaStream_t s);
int backward_blocks_per_sm(int n_tf);

}  // namespace aloha
