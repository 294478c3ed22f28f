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
  unsigned k;                 // checkpoint interval (samples)
  unsigned ckpt_cap;          // checkpoints per pixel
  Checkpoint* ckpt;           // [npx][ckpt_cap]
  float4* final_rgba;         // [npx] final colour of the forward
  float4* out_rgba;           // [npx] caller's image (forward) or null
  uint2* work;                // [work_cap] (pixel, segment)
  unsigned work_cap;
  unsigned* work_count;        // [0] segments appended, [1] chunk counter of the forward,
                               // [2] item counter of the backward
  int* overflow;              // set when a pixel needs more checkpoints than ckpt_cap
  const float4* dl_drgba;     // [npx] backward input
  float* dtf;                 // [n_tf*4] accumulated
  float4* dgrid4;             // density gradient in x-quads: element (x,y,z) holds the
                              // contributions to voxels x, x+1, x+2 (w unused)
  const int4* brick_grid_origin;  // per brick: voxelRange.lower - grid_lo
  int grid_dims[3];
  unsigned long long* counter;
  const int* chunk_order;     // forward: 8x4 chunk ids in the order to march them, or null (ring order)
  int n_chunks;               // entries of chunk_order
};

cudaError_t launch_forward_train(const TrainArgs& a, int view, int width, int height, int max_grid, cudaStream_t s);
int forward_train_blocks_per_sm(int n_tf);
cudaError_t launch_backward(const TrainArgs& a, int view, int grid, cudaStream_t s);
// out[v] += quads[v].x + quads[v-1].y + quads[v-2].z along x, for a grid of dims.
cudaError_t launch_fold_quads(const float4* quads, float* out, const int dims[3], cudaStream_t s);
int backward_blocks_per_sm(int n_tf);

}  // namespace aloha
