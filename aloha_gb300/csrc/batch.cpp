// batch.cpp -- batched form: many views in one persistent launch, CUDA-graph
// capture and the autotuner over ray-tile shape and stencil staging.  No reference counterpart: the reference
// renders one camera per owlLaunch2D (waikikiRenderer.cpp:1028).
#include <cuda_runtime.h>

#include <cstring>
#include <new>
#include <vector>

#include "batch_internal.h"

using namespace aloha;

struct aloha_batch {
  aloha_ctx* ctx = nullptr;
  std::vector<int> views;
  std::vector<uint32_t*> fbs;
  int tile_w = 16, tile_h = 8, ctas_per_sm = 0;
  int stage = ALOHA_STAGING_NONE;
  int steps = 1;  // march steps per loop trip (2 only with direct loads)
  int* d_view_ids = nullptr;
  uint32_t** d_fbs = nullptr;
  int* d_prefix = nullptr;
  unsigned int* d_work = nullptr;
  int total_tiles = 0;
  int grid = 0;
  cudaStream_t capture_stream = nullptr;
  cudaGraph_t graph = nullptr;
  cudaGraphExec_t exec = nullptr;
};

namespace {

void drop_graph(aloha_batch* b) {
  if (b->exec) cudaGraphExecDestroy(b->exec);
  if (b->graph) cudaGraphDestroy(b->graph);
  b->exec = nullptr;
  b->graph = nullptr;
}

// The render kernel's stage for the batch's staging and unroll settings
// (two steps per trip exist for direct loads only).
int kernel_stage(const aloha_batch* b) {
  return b->stage == ALOHA_STAGING_NONE && b->steps == 2 ? kStageUnroll2 : b->stage;
}

// Tile prefix sums and the grid for the current tile shape.
int configure(aloha_batch* b) {
  aloha_ctx* c = b->ctx;
  std::vector<int> prefix(b->views.size() + 1, 0);
  for (size_t i = 0; i < b->views.size(); ++i) {
    int w = 0, h = 0;
    ctx_view_size(c, b->views[i], &w, &h);
    const long long next = (long long)prefix[i] + ring_slots(w, h, b->tile_w, b->tile_h);
    if (next > 0x7fffffffll) return ctx_fail(c, ALOHA_ERR_UNSUPPORTED, "batch: more than 2^31 - 1 tiles in all views");
    prefix[i + 1] = (int)next;
  }
  b->total_tiles = prefix.back();
  if (cudaMemcpy(b->d_prefix, prefix.data(), sizeof(int) * prefix.size(), cudaMemcpyHostToDevice) != cudaSuccess)
    return ctx_fail(c, ALOHA_ERR_CUDA, "batch: uploading tile prefix failed");
  int per_sm = render_blocks_per_sm(b->tile_w, b->tile_h, ctx_n_tf(c), true, kernel_stage(b));
  if (per_sm <= 0) return ctx_fail(c, ALOHA_ERR_CUDA, "batch: occupancy query failed");
  if (b->ctas_per_sm > 0 && b->ctas_per_sm < per_sm) per_sm = b->ctas_per_sm;
  b->grid = ctx_num_sms(c) * per_sm;
  drop_graph(b);
  return ALOHA_OK;
}

int enqueue(aloha_batch* b, cudaStream_t s) {
  aloha_ctx* c = b->ctx;
  BatchArgs a{};
  ctx_frame_args(c, &a.f);
  a.view_ids = b->d_view_ids;
  a.fbs = b->d_fbs;
  a.tile_prefix = b->d_prefix;
  a.n_items = (int)b->views.size();
  a.total_tiles = b->total_tiles;
  a.work_counter = b->d_work;
  if (cudaMemsetAsync(b->d_work, 0, sizeof(unsigned int), s) != cudaSuccess ||
      cudaMemsetAsync(a.f.counter, 0, sizeof(unsigned long long), s) != cudaSuccess)
    return ctx_fail(c, ALOHA_ERR_CUDA, "batch: memset failed");
  cudaError_t e = launch_render_warps(a, b->tile_w, b->tile_h, b->grid, true, s, kernel_stage(b));
  if (e != cudaSuccess) return ctx_fail(c, ALOHA_ERR_CUDA, "batch launch: %s", cudaGetErrorString(e));
  ctx_mark_samples(c);
  return ALOHA_OK;
}

// Brings every view of the batch up to date (schedules, cameras) on `s`.
int refresh(aloha_batch* b, cudaStream_t s) {
  for (int v : b->views) {
    int rc = ctx_prepare_view(b->ctx, v, s);
    if (rc) return rc;
  }
  return ALOHA_OK;
}

}  // namespace

extern "C" {

int aloha_batch_create(aloha_ctx* c, const int* views, int n_items, uint32_t* const* fbs, aloha_batch** out) {
  if (!c || !views || !fbs || !out) return ALOHA_ERR_NULL_POINTER;
  *out = nullptr;
  if (n_items < 1 || n_items > kMaxViews) return ctx_fail(c, ALOHA_ERR_INVALID_ARGUMENT, "batch of %d items", n_items);
  if (cudaSetDevice(ctx_device(c)) != cudaSuccess) return ctx_fail(c, ALOHA_ERR_CUDA, "cudaSetDevice failed");
  for (int i = 0; i < n_items; ++i) {
    if (!fbs[i]) return ctx_fail(c, ALOHA_ERR_NULL_POINTER, "batch frame buffer %d is null", i);
    if (!ctx_is_device_pointer(fbs[i]))
      return ctx_fail(c, ALOHA_ERR_INVALID_ARGUMENT, "batch frame buffer %d is not device memory", i);
    int rc = ctx_prepare_view(c, views[i], 0);
    if (rc) return rc;
  }
  aloha_batch* b = new (std::nothrow) aloha_batch();
  if (!b) return ALOHA_ERR_OUT_OF_MEMORY;
  b->ctx = c;
  b->views.assign(views, views + n_items);
  b->fbs.assign(fbs, fbs + n_items);
  bool ok = cudaMalloc(&b->d_view_ids, sizeof(int) * n_items) == cudaSuccess &&
            cudaMalloc(&b->d_fbs, sizeof(uint32_t*) * n_items) == cudaSuccess &&
            cudaMalloc(&b->d_prefix, sizeof(int) * (n_items + 1)) == cudaSuccess &&
            cudaMalloc(&b->d_work, sizeof(unsigned int)) == cudaSuccess &&
            cudaStreamCreateWithFlags(&b->capture_stream, cudaStreamNonBlocking) == cudaSuccess;
  ok = ok && cudaMemcpy(b->d_view_ids, views, sizeof(int) * n_items, cudaMemcpyHostToDevice) == cudaSuccess &&
       cudaMemcpy(b->d_fbs, fbs, sizeof(uint32_t*) * n_items, cudaMemcpyHostToDevice) == cudaSuccess &&
       cudaDeviceSynchronize() == cudaSuccess;
  if (!ok) {
    aloha_batch_destroy(b);
    return ctx_fail(c, ALOHA_ERR_OUT_OF_MEMORY, "batch: device allocation failed");
  }
  int rc = configure(b);
  if (rc) {
    aloha_batch_destroy(b);
    return rc;
  }
  *out = b;
  return ALOHA_OK;
}

int aloha_batch_set_config(aloha_batch* b, int tile_w, int tile_h, int ctas_per_sm) {
  if (!b) return ALOHA_ERR_NULL_POINTER;
  const bool known = known_chunk(tile_w, tile_h);
  if (!known || ctas_per_sm < 0)
    return ctx_fail(b->ctx, ALOHA_ERR_INVALID_ARGUMENT, "tile %dx%d not one of 8x4, 8x8, 16x8, 32x4", tile_w, tile_h);
  b->tile_w = tile_w;
  b->tile_h = tile_h;
  b->ctas_per_sm = ctas_per_sm;
  return configure(b);
}

int aloha_batch_set_staging(aloha_batch* b, int stage) {
  if (!b) return ALOHA_ERR_NULL_POINTER;
  if (stage != ALOHA_STAGING_NONE && stage != ALOHA_STAGING_NEXT_SAMPLE)
    return ctx_fail(b->ctx, ALOHA_ERR_INVALID_ARGUMENT, "staging %d not NONE (0) or NEXT_SAMPLE (1)", stage);
  b->stage = stage;
  return configure(b);
}

int aloha_batch_get_staging(const aloha_batch* b, int* stage) {
  if (!b || !stage) return ALOHA_ERR_NULL_POINTER;
  *stage = b->stage;
  return ALOHA_OK;
}

int aloha_batch_set_unroll(aloha_batch* b, int steps) {
  if (!b) return ALOHA_ERR_NULL_POINTER;
  if (steps != 1 && steps != 2) return ctx_fail(b->ctx, ALOHA_ERR_INVALID_ARGUMENT, "unroll %d not 1 or 2", steps);
  b->steps = steps;
  return configure(b);
}

int aloha_batch_get_unroll(const aloha_batch* b, int* steps) {
  if (!b || !steps) return ALOHA_ERR_NULL_POINTER;
  *steps = b->steps;
  return ALOHA_OK;
}

int aloha_batch_get_config(const aloha_batch* b, int* tile_w, int* tile_h, int* ctas_per_sm) {
  if (!b || !tile_w || !tile_h || !ctas_per_sm) return ALOHA_ERR_NULL_POINTER;
  *tile_w = b->tile_w;
  *tile_h = b->tile_h;
  *ctas_per_sm = b->ctas_per_sm;
  return ALOHA_OK;
}

int aloha_batch_launch(aloha_batch* b, void* stream) {
  if (!b) return ALOHA_ERR_NULL_POINTER;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
  cudaStreamIsCapturing(s, &st);
  if (st == cudaStreamCaptureStatusNone) {
    int rc = refresh(b, s);
    if (rc) return rc;
  }
  return enqueue(b, s);
}

int aloha_batch_launch_graph(aloha_batch* b, void* stream) {
  if (!b) return ALOHA_ERR_NULL_POINTER;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  int rc = refresh(b, s);
  if (rc) return rc;
  if (!b->exec) {
    // capture on a private stream ordered after the caller's work
    if (cudaStreamSynchronize(s) != cudaSuccess) return ctx_fail(b->ctx, ALOHA_ERR_CUDA, "sync before capture");
    if (cudaStreamBeginCapture(b->capture_stream, cudaStreamCaptureModeThreadLocal) != cudaSuccess)
      return ctx_fail(b->ctx, ALOHA_ERR_CUDA, "cudaStreamBeginCapture failed");
    rc = enqueue(b, b->capture_stream);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(b->capture_stream, &g);
    if (rc) {
      if (g) cudaGraphDestroy(g);
      return rc;
    }
    if (e != cudaSuccess) return ctx_fail(b->ctx, ALOHA_ERR_CUDA, "cudaStreamEndCapture: %s", cudaGetErrorString(e));
    b->graph = g;
    if (cudaGraphInstantiate(&b->exec, g, 0) != cudaSuccess) {
      drop_graph(b);
      return ctx_fail(b->ctx, ALOHA_ERR_CUDA, "cudaGraphInstantiate failed");
    }
  }
  if (cudaGraphLaunch(b->exec, s) != cudaSuccess) return ctx_fail(b->ctx, ALOHA_ERR_CUDA, "cudaGraphLaunch failed");
  ctx_mark_samples(b->ctx);
  return ALOHA_OK;
}

int aloha_batch_autotune(aloha_batch* b, void* stream, int reps, int* tile_w, int* tile_h, float* ms) {
  if (!b || !tile_w || !tile_h || !ms) return ALOHA_ERR_NULL_POINTER;
  if (reps < 1) reps = 1;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  static const int shapes[4][2] = {{8, 4}, {8, 8}, {16, 8}, {32, 4}};
  cudaEvent_t e0, e1;
  if (cudaEventCreate(&e0) != cudaSuccess || cudaEventCreate(&e1) != cudaSuccess)
    return ctx_fail(b->ctx, ALOHA_ERR_CUDA, "cudaEventCreate failed");
  // the loads and loop forms: direct, direct two steps per trip, staged
  static const int forms[3][2] = {{ALOHA_STAGING_NONE, 1}, {ALOHA_STAGING_NONE, 2}, {ALOHA_STAGING_NEXT_SAMPLE, 1}};
  float best = -1.f;
  int bw = b->tile_w, bh = b->tile_h, bs = b->stage, bu = b->steps;
  int rc = ALOHA_OK;
  for (int k = 0; k < 12 && !rc; ++k) {
    const int* sh = shapes[k % 4];
    const int stage = forms[k / 4][0], steps = forms[k / 4][1];
    b->stage = stage;
    b->steps = steps;
    rc = aloha_batch_set_config(b, sh[0], sh[1], 0);
    if (rc) break;
    rc = aloha_batch_launch(b, stream);  // warm-up
    if (rc) break;
    cudaEventRecord(e0, s);
    for (int r = 0; r < reps && !rc; ++r) rc = aloha_batch_launch(b, stream);
    cudaEventRecord(e1, s);
    if (rc) break;
    if (cudaEventSynchronize(e1) != cudaSuccess) {
      rc = ctx_fail(b->ctx, ALOHA_ERR_CUDA, "autotune: launch failed");
      break;
    }
    float t = 0.f;
    cudaEventElapsedTime(&t, e0, e1);
    t /= (float)reps;
    if (best < 0.f || t < best) {
      best = t;
      bw = sh[0];
      bh = sh[1];
      bs = stage;
      bu = steps;
    }
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  if (rc) return rc;
  b->stage = bs;
  b->steps = bu;
  rc = aloha_batch_set_config(b, bw, bh, 0);
  if (rc) return rc;
  *tile_w = bw;
  *tile_h = bh;
  *ms = best;
  return ALOHA_OK;
}

int aloha_batch_destroy(aloha_batch* b) {
  if (!b) return ALOHA_ERR_NULL_POINTER;
  if (b->capture_stream) cudaStreamSynchronize(b->capture_stream);
  cudaDeviceSynchronize();
  drop_graph(b);
  if (b->d_view_ids) cudaFree(b->d_view_ids);
  if (b->d_fbs) cudaFree(b->d_fbs);
  if (b->d_prefix) cudaFree(b->d_prefix);
  if (b->d_work) cudaFree(b->d_work);
  if (b->capture_stream) cudaStreamDestroy(b->capture_stream);
  delete b;
  return ALOHA_OK;
}

int aloha_render_batch(aloha_ctx* c, const int* views, int n_items, uint32_t* const* fbs, void* stream) {
  if (!c || !views || !fbs) return ALOHA_ERR_NULL_POINTER;
  if (n_items < 1 || n_items > kMaxViews) return ctx_fail(c, ALOHA_ERR_INVALID_ARGUMENT, "batch of %d items", n_items);
  if (cudaSetDevice(ctx_device(c)) != cudaSuccess) return ctx_fail(c, ALOHA_ERR_CUDA, "cudaSetDevice failed");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  // host frame buffers go through one device staging block
  std::vector<uint32_t*> dev_fbs(n_items);
  std::vector<size_t> sizes(n_items);
  size_t stage_elems = 0;
  for (int i = 0; i < n_items; ++i) {
    if (!fbs[i]) return ctx_fail(c, ALOHA_ERR_NULL_POINTER, "frame buffer %d is null", i);
    int rc = ctx_prepare_view(c, views[i], s);
    if (rc) return rc;
    int w = 0, h = 0;
    ctx_view_size(c, views[i], &w, &h);
    sizes[i] = (size_t)w * h;
    if (!ctx_is_device_pointer(fbs[i])) stage_elems += sizes[i];
  }
  uint32_t* stage = nullptr;
  if (stage_elems && cudaMalloc(&stage, stage_elems * sizeof(uint32_t)) != cudaSuccess)
    return ctx_fail(c, ALOHA_ERR_OUT_OF_MEMORY, "batch staging of %zu bytes", stage_elems * 4);
  size_t off = 0;
  for (int i = 0; i < n_items; ++i) {
    if (ctx_is_device_pointer(fbs[i])) {
      dev_fbs[i] = fbs[i];
    } else {
      dev_fbs[i] = stage + off;
      off += sizes[i];
    }
  }
  aloha_batch* b = nullptr;
  int rc = aloha_batch_create(c, views, n_items, dev_fbs.data(), &b);
  if (!rc) rc = aloha_batch_launch(b, stream);
  for (int i = 0; i < n_items && !rc; ++i)
    if (dev_fbs[i] != fbs[i] &&
        cudaMemcpyAsync(fbs[i], dev_fbs[i], sizes[i] * sizeof(uint32_t), cudaMemcpyDeviceToHost, s) != cudaSuccess)
      rc = ctx_fail(c, ALOHA_ERR_CUDA, "batch: copy to host failed");
  if (cudaStreamSynchronize(s) != cudaSuccess && !rc) rc = ctx_fail(c, ALOHA_ERR_CUDA, "batch: stream failed");
  if (b) aloha_batch_destroy(b);
  if (stage) cudaFree(stage);
  return rc;
}

}  // extern "C"
