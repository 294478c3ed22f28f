// api.cpp -- the C ABI (include/aloha.h): context, bricks, transfer function,
// virtual ranks, views and the render entry points.
//
// The context replaces maui::Renderer (waikikiRenderer.cpp:344-1080) for the
// volume path on one GPU: bricks are kept resident in HBM in a padded layout,
// every camera change recomputes the per-view schedule (rank order and each
// rank's front-to-back brick list), and render() launches one fused kernel.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdint>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "adjoint.h"
#include "batch_internal.h"
#include "internal.h"
#include "order.h"

using namespace aloha;

namespace {

// Scratch of the differentiable form for one view (checkpoints, final
// colours, the segment work list).
struct TrainState {
  Checkpoint* ckpt = nullptr;
  float4* final_rgba = nullptr;
  uint2* work = nullptr;
  unsigned* work_count = nullptr;
  int* overflow = nullptr;
  size_t bytes = 0;
  unsigned k = 0, cap = 0;
  size_t npx = 0;
  bool valid = false;
  void release() {
    for (void* p : {(void*)ckpt, (void*)final_rgba, (void*)work, (void*)work_count, (void*)overflow})
      if (p) cudaFree(p);
    *this = TrainState();
  }
};

struct ViewState {
  bool has_camera = false, has_size = false, dirty = true;
  float org[3], dir_00[3], dir_du[3], dir_dv[3];
  int width = 0, height = 0;
  Schedule sched;
  float4* accum = nullptr;  // [n_ranks][H*W]
  size_t accum_elems = 0;
  TrainState train;
};

struct DeviceBuffer {
  void* ptr = nullptr;
  size_t bytes = 0;
  cudaError_t ensure(size_t want) {
    if (want <= bytes) return cudaSuccess;
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
    cudaError_t e = cudaMalloc(&ptr, want);
    if (e == cudaSuccess) bytes = want;
    return e;
  }
  void release() {
    if (ptr) cudaFree(ptr);
    ptr = nullptr;
    bytes = 0;
  }
};

bool finite3(const float* v) { return std::isfinite(v[0]) && std::isfinite(v[1]) && std::isfinite(v[2]); }

bool is_device_pointer(const void* p) {
  cudaPointerAttributes attr;
  if (cudaPointerGetAttributes(&attr, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return attr.type == cudaMemoryTypeDevice || attr.type == cudaMemoryTypeManaged;
}

// Where an output buffer lives, from one pointer query: device memory, or
// host memory with the device address of page-locked memory registered with
// CUDA (e.g. cudaHostAlloc / cudaMallocHost; null for pageable memory).
// Kernels on GB300 write page-locked memory directly over NVLink-C2C.
bool classify_output(void* p, void** pinned_alias) {
  *pinned_alias = nullptr;
  cudaPointerAttributes attr;
  if (cudaPointerGetAttributes(&attr, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (attr.type == cudaMemoryTypeDevice || attr.type == cudaMemoryTypeManaged) return true;
  if (attr.type == cudaMemoryTypeHost) *pinned_alias = attr.devicePointer;
  return false;
}

}  // namespace

struct aloha_ctx {
  int device = 0;
  int num_sms = 0;
  std::string last_error;
  // bricks
  std::vector<aloha_brick_desc> descs;
  std::vector<Box> boxes;
  std::vector<DevBrick> dev_bricks;
  std::vector<char> brick_present;
  std::vector<size_t> brick_offset;  // quad offset of each padded brick in `voxels`
  DeviceBuffer voxels, bricks_dev, staging_in;
  float bounds_lo[3] = {0, 0, 0}, bounds_hi[3] = {0, 0, 0};
  // transfer function
  DeviceBuffer tf;
  int n_tf = 0;
  // empty-space macrocells: value range per macrocell (per brick) and the
  // per-transfer-function empty mask, refreshed before the next render
  DeviceBuffer mc_ranges, mc_empty, tf_prefix;
  std::vector<size_t> mc_offset;
  size_t mc_total = 0;
  bool empty_dirty = true;
  // virtual ranks
  int n_ranks = 0;
  std::vector<int> brick_rank;
  std::vector<KdNode> tree;
  OrderCache order_cache;  // eye-independent part of the visibility orders
  bool order_cache_valid = false;
  // views
  std::vector<ViewState> views;
  DeviceBuffer views_dev, sched_dev;
  int sched_stride = 0;  // ints per view slot
  // params, scratch
  aloha_render_params params;
  DeviceBuffer counter, flag, staging_out, work, grad4;
  DeviceBuffer train_tables;  // per launch of the differentiable form: item counter, views, runs
  // every byte of grad4 is zero once the stream reaches the last fold (the
  // fold clears the quads it reads); false after a reallocation or a backward
  // that returned before its fold was enqueued
  bool grad4_zero = false;
  // persistent render of one view: chunk shape and grid (occupancy depends on
  // the transfer-function size through shared memory)
  int chunk_w = 0, chunk_h = 0;  // 0 = automatic
  int grid_n_tf = -1, grid_blocks = 0, grid_cw = 0, grid_ch = 0;
  // cost-ordered chunks of single-view renders: mode, probe costs | max | order
  int chunk_order_mode = ALOHA_CHUNKS_AUTO;
  DeviceBuffer chunk_order;
  // rank-split render: mode, scratch rank images, per-chunk tickets, grid
  int split_mode = ALOHA_SPLIT_AUTO;
  int staging = ALOHA_STAGING_NONE;  // stencil loads of the single-view render kernel
  int grid_stage = -1;
  int lane_group_permille = 0;       // share of the cost order rendered by lane groups
  int grid_blocks_lg = 0, grid_lg_n_tf = -1;
  DeviceBuffer split_images, split_masks, split_items, split_done;
  int split_grid_n_tf = -1, split_grid_blocks = 0;
  int chunk_order_slots = -1;  // slot count of the chunk-order buffer's current layout
  bool split_grid_many = false;
  uint64_t last_samples = 0;
  bool samples_valid = false;

  int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    last_error = buf;
    return code;
  }
  int cuda_fail(cudaError_t e, const char* what) {
    return fail(ALOHA_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
  }
};

#define CUDA_TRY(ctx, call)                                 \
  do {                                                      \
    cudaError_t _e = (call);                                \
    if (_e != cudaSuccess) return (ctx)->cuda_fail(_e, #call); \
  } while (0)

namespace {

// Any change of scene, parameters or partition invalidates stored checkpoints.
void invalidate_training(aloha_ctx* c) {
  for (auto& v : c->views) v.train.valid = false;
}

// Conservative screen rectangle of every virtual rank, in 8x4-pixel chunks
// (inclusive [cx0, cy0, cx1, cy1]; cx0 > cx1 when no pixel ray can enter the
// rank's bricks).  A brick corner P projects to the continuous pixel
// coordinates (su, sv) solving P - org = a (dir_00 + su du + sv dv); the box
// projects into the hull of its corners when all of them lie in front of the
// camera (a > 0), else the rank gets the whole frame.  The margin covers the
// ray generation's rounding and its clamp of tiny direction components
// (up to 2e-5 per component of the unit direction).
std::vector<int> rank_screen_rects(const aloha_ctx* c, const ViewState& v) {
  const int R = c->n_ranks;
  const int cxn = (v.width + 7) / 8, cyn = (v.height + 3) / 4;
  std::vector<double> x0(R, 1e300), y0(R, 1e300), x1(R, -1e300), y1(R, -1e300);
  std::vector<char> full(R, 0);
  const double d00[3] = {v.dir_00[0], v.dir_00[1], v.dir_00[2]};
  const double du[3] = {v.dir_du[0], v.dir_du[1], v.dir_du[2]};
  const double dv[3] = {v.dir_dv[0], v.dir_dv[1], v.dir_dv[2]};
  // det [d00 du dv] and the cofactor rows for Cramer's rule
  auto det3 = [](const double a[3], const double b[3], const double cc[3]) {
    return a[0] * (b[1] * cc[2] - b[2] * cc[1]) - b[0] * (a[1] * cc[2] - a[2] * cc[1]) +
           cc[0] * (a[1] * b[2] - a[2] * b[1]);
  };
  const double det = det3(d00, du, dv);
  // angle of one pixel (smallest over the frame corners) for the margin
  double dmax = 0.0;
  for (int cy = 0; cy < 2; ++cy)
    for (int cx = 0; cx < 2; ++cx) {
      double n2 = 0.0;
      for (int a = 0; a < 3; ++a) {
        const double d = d00[a] + cx * v.width * du[a] + cy * v.height * dv[a];
        n2 += d * d;
      }
      dmax = std::max(dmax, std::sqrt(n2));
    }
  const double lu = std::sqrt(du[0] * du[0] + du[1] * du[1] + du[2] * du[2]);
  const double lv = std::sqrt(dv[0] * dv[0] + dv[1] * dv[1] + dv[2] * dv[2]);
  const double pix_angle = dmax > 0.0 ? std::min(lu, lv) / dmax : 0.0;
  const bool degenerate = !(std::fabs(det) > 1e-30) || !(pix_angle > 1e-12);
  const double margin = degenerate ? 0.0 : 2.0 + 6e-5 / pix_angle;
  for (size_t b = 0; b < c->boxes.size(); ++b) {
    const int r = c->brick_rank[b];
    if (r < 0 || r >= R || full[r]) continue;
    if (degenerate) {
      full[r] = 1;
      continue;
    }
    for (int k = 0; k < 8; ++k) {
      double rhs[3];
      for (int a = 0; a < 3; ++a)
        rhs[a] = (double)((k >> a) & 1 ? c->boxes[b].hi[a] : c->boxes[b].lo[a]) - (double)v.org[a];
      const double A = det3(rhs, du, dv) / det, B = det3(d00, rhs, dv) / det, C = det3(d00, du, rhs) / det;
      double scale = 0.0;
      for (int a = 0; a < 3; ++a) scale = std::max(scale, std::fabs(rhs[a]));
      if (!(A > 1e-6 * (scale + 1.0) / (dmax + 1e-300))) {
        full[r] = 1;
        break;
      }
      const double su = B / A - 0.5, sv = C / A - 0.5;  // pixel index whose centre the corner meets
      x0[r] = std::min(x0[r], su);
      x1[r] = std::max(x1[r], su);
      y0[r] = std::min(y0[r], sv);
      y1[r] = std::max(y1[r], sv);
    }
  }
  std::vector<int> rects(4 * (size_t)R);
  for (int r = 0; r < R; ++r) {
    int* q = &rects[4 * (size_t)r];
    if (full[r]) {
      q[0] = 0, q[1] = 0, q[2] = cxn - 1, q[3] = cyn - 1;
      continue;
    }
    if (x0[r] > x1[r]) {  // no bricks
      q[0] = 1, q[1] = 1, q[2] = 0, q[3] = 0;
      continue;
    }
    auto clampd = [](double t, double lo, double hi) { return t < lo ? lo : (t > hi ? hi : t); };
    const double px0 = clampd(std::floor(x0[r] - margin), -8.0, v.width + 8.0);
    const double px1 = clampd(std::ceil(x1[r] + margin), -8.0, v.width + 8.0);
    const double py0 = clampd(std::floor(y0[r] - margin), -8.0, v.height + 8.0);
    const double py1 = clampd(std::ceil(y1[r] + margin), -8.0, v.height + 8.0);
    q[0] = std::max(0, (int)std::floor(px0 / 8.0));
    q[2] = std::min(cxn - 1, (int)std::floor(px1 / 8.0));
    q[1] = std::max(0, (int)std::floor(py0 / 4.0));
    q[3] = std::min(cyn - 1, (int)std::floor(py1 / 4.0));
    if (px1 < 0.0 || py1 < 0.0 || px0 >= v.width || py0 >= v.height) q[0] = 1, q[1] = 1, q[2] = 0, q[3] = 0;
  }
  return rects;
}

// Upload dirty view state (camera, size, schedule) for `view` on `s`.
int prepare_view(aloha_ctx* c, int view, cudaStream_t s) {
  if (c->descs.empty()) return c->fail(ALOHA_ERR_NOT_READY, "no bricks uploaded");
  if (c->n_tf == 0) return c->fail(ALOHA_ERR_NOT_READY, "no transfer function set");
  if (view < 0 || view >= (int)c->views.size()) return c->fail(ALOHA_ERR_OUT_OF_RANGE, "view %d has no state", view);
  ViewState& v = c->views[view];
  if (!v.has_camera) return c->fail(ALOHA_ERR_NOT_READY, "view %d has no camera", view);
  if (!v.has_size) return c->fail(ALOHA_ERR_NOT_READY, "view %d has no size", view);
  for (size_t b = 0; b < c->brick_present.size(); ++b)
    if (!c->brick_present[b]) return c->fail(ALOHA_ERR_MISSING_BRICK, "brick %zu has no data (dropped)", b);
  if (c->empty_dirty) {
    CUDA_TRY(c, launch_macrocell_empty(static_cast<const float2*>(c->mc_ranges.ptr), (int)c->mc_total,
                                       static_cast<const int*>(c->tf_prefix.ptr), c->n_tf,
                                       static_cast<uint8_t*>(c->mc_empty.ptr), s));
    c->empty_dirty = false;
  }
  const int nb = (int)c->descs.size();
  const int stride = 2 * c->n_ranks + 1 + nb + 4 * c->n_ranks;
  if (stride != c->sched_stride) {
    CUDA_TRY(c, c->sched_dev.ensure(sizeof(int) * (size_t)stride * kMaxViews));
    c->sched_stride = stride;
    for (auto& vv : c->views) vv.dirty = true;
  }
  if (!v.dirty) return ALOHA_OK;
  if (!c->order_cache_valid) {
    c->order_cache = build_order_cache(c->boxes, c->brick_rank, c->n_ranks);
    c->order_cache_valid = true;
  }
  v.sched = make_schedule(c->boxes, c->brick_rank, c->n_ranks, c->tree, c->params.order_mode, v.org, c->order_cache);
  // every rank appears exactly once in the composite order
  std::vector<char> seen(c->n_ranks, 0);
  std::vector<int> order;
  for (int r : v.sched.rank_order)
    if (r >= 0 && r < c->n_ranks && !seen[r]) {
      seen[r] = 1;
      order.push_back(r);
    }
  for (int r = 0; r < c->n_ranks; ++r)
    if (!seen[r]) order.push_back(r);
  v.sched.rank_order = order;
  std::vector<int> slot;
  slot.reserve(stride);
  slot.insert(slot.end(), order.begin(), order.end());
  slot.insert(slot.end(), v.sched.rank_start.begin(), v.sched.rank_start.end());
  slot.insert(slot.end(), v.sched.rank_bricks.begin(), v.sched.rank_bricks.end());
  slot.resize(2 * c->n_ranks + 1 + nb, 0);
  const std::vector<int> rects = rank_screen_rects(c, v);
  slot.insert(slot.end(), rects.begin(), rects.end());
  DevView dv{};
  for (int a = 0; a < 3; ++a) {
    dv.org[a] = v.org[a];
    dv.dir_00[a] = v.dir_00[a];
    dv.dir_du[a] = v.dir_du[a];
    dv.dir_dv[a] = v.dir_dv[a];
  }
  dv.width = v.width;
  dv.height = v.height;
  // maxDepth as handleCameraEvent computes it (waikikiRenderer.cpp:858-859)
  {
    float ctr[3], s1 = 0.f, s2 = 0.f;
    for (int a = 0; a < 3; ++a) ctr[a] = (c->bounds_lo[a] + c->bounds_hi[a]) / 2.f;
    for (int a = 0; a < 3; ++a) {
      const float q = ctr[a] + c->bounds_hi[a];
      s1 = s1 + q * q;
      const float o = v.org[a] + ctr[a];
      s2 = s2 + o * o;
    }
    dv.max_depth = std::sqrt(s2) + std::sqrt(s1);
  }
  dv.n_ranks = c->n_ranks;
  dv.sched = view * stride;
  dv.rects = view * stride + 2 * c->n_ranks + 1 + nb;
  int* sched_dst = static_cast<int*>(c->sched_dev.ptr) + (size_t)view * stride;
  CUDA_TRY(c, cudaMemcpyAsync(sched_dst, slot.data(), sizeof(int) * stride, cudaMemcpyHostToDevice, s));
  CUDA_TRY(c, cudaMemcpyAsync(static_cast<DevView*>(c->views_dev.ptr) + view, &dv, sizeof dv,
                              cudaMemcpyHostToDevice, s));
  v.dirty = false;
  return ALOHA_OK;
}

// Per-view accumulation buffer when the parameters ask for it.
int prepare_accum(aloha_ctx* c, int view, cudaStream_t s, float4** out) {
  *out = nullptr;
  const aloha_render_params& p = c->params;
  if (!p.accumulate && p.accum_id == 0) return ALOHA_OK;
  ViewState& v = c->views[view];
  const size_t elems = (size_t)c->n_ranks * v.width * v.height;
  if (v.accum_elems != elems) {
    if (p.accum_id > 0)
      return c->fail(ALOHA_ERR_NOT_READY, "accum_id > 0 but view %d has no accumulation buffer of this size", view);
    if (v.accum) cudaFree(v.accum);
    v.accum = nullptr;
    v.accum_elems = 0;
    CUDA_TRY(c, cudaMalloc(&v.accum, elems * sizeof(float4)));
    CUDA_TRY(c, cudaMemsetAsync(v.accum, 0, elems * sizeof(float4), s));
    v.accum_elems = elems;
  }
  *out = v.accum;
  return ALOHA_OK;
}

constexpr size_t kSplitScratchCap = size_t(16) << 30;  // rank split scratch limit

// Bytes of scratch the rank split of `v` needs: rank image planes, masks,
// item list, tickets.
size_t split_scratch_bytes(const aloha_ctx* c, const ViewState& v) {
  const size_t slots = (size_t)ring_slots(v.width, v.height, 8, 4);
  return (size_t)c->n_ranks * v.width * v.height * sizeof(float4) + slots * (8 + 4 + 4 + 4 * (size_t)c->n_ranks);
}

// The rank split serves aloha_render (a frame buffer, no rank planes wanted)
// with 1 < n_ranks <= kSplitMaxRanks.
bool rank_split_possible(const aloha_ctx* c, const FrameArgs& f, const ViewState& v) {
  return f.fb && !f.rank_images && !f.rank_depth && c->n_ranks >= 2 && c->n_ranks <= kSplitMaxRanks &&
         ring_slots(v.width, v.height, 8, 4) < (1 << 25);
}

// Automatic mode: the pixel split for few ranks, the rank split for many.
// 8 bricks of a 512^3 volume at 1024^2: pixels 0.99 ms, ranks 1.15 ms (the
// longest chunks spend most of their samples inside one brick).  64 bricks of
// a 1024^3 volume at 2048^2: pixels 7.08 ms, ranks 6.58 ms (each pixel walks
// 64 ranks in the pixel split; most chunks are covered by few of them).
constexpr int kAutoRankSplitRanks = 32;

bool use_rank_split(const aloha_ctx* c, const FrameArgs& f, const ViewState& v) {
  if (c->split_mode == ALOHA_SPLIT_PIXELS || !rank_split_possible(c, f, v)) return false;
  if (c->split_mode == ALOHA_SPLIT_AUTO && c->n_ranks < kAutoRankSplitRanks) return false;
  return split_scratch_bytes(c, v) <= kSplitScratchCap;
}

int plan_chunk_order(aloha_ctx* c, const FrameArgs& f, int view, int cw, int ch, cudaStream_t s, const int** order,
                     int* chunks, bool auto_order = true, unsigned int* zero_work = nullptr,
                     unsigned long long* zero_samples = nullptr);

// Rank-split launch of a single view (mask, plan and render kernels).
int launch_split(aloha_ctx* c, const FrameArgs& f, int view, cudaStream_t s) {
  const ViewState& v = c->views[view];
  const int R = c->n_ranks;
  SplitArgs a{};
  a.f = f;
  a.view = view;
  a.n_slots = ring_slots(v.width, v.height, 8, 4);
  {  // cost order of the 8x4 chunks (positions are then chunks, not ring slots)
    int chunks = 0;
    // automatic ordering only below the automatic rank-split range: with many
    // ranks the (chunk, rank) items are short already (64 bricks at 2048^2:
    // 6.29 ms in ring order, 6.47 ms cost-ordered)
    const int rc = plan_chunk_order(c, f, view, 8, 4, s, &a.chunk_order, &chunks, R < kAutoRankSplitRanks);
    if (rc) return rc;
    if (a.chunk_order) a.n_slots = chunks;
  }
  CUDA_TRY(c, c->split_images.ensure((size_t)R * v.width * v.height * sizeof(float4)));
  a.f.rank_images = static_cast<float4*>(c->split_images.ptr);
  const size_t scan_blocks = ((size_t)a.n_slots + 1023) / 1024;
  CUDA_TRY(c, c->split_masks.ensure((size_t)a.n_slots * (sizeof(unsigned long long) + sizeof(uint32_t)) +
                                    scan_blocks * sizeof(uint32_t)));
  a.masks = static_cast<unsigned long long*>(c->split_masks.ptr);
  a.offsets = reinterpret_cast<uint32_t*>(a.masks + a.n_slots);
  a.block_sums = a.offsets + a.n_slots;
  CUDA_TRY(c, c->split_items.ensure((size_t)a.n_slots * R * sizeof(uint32_t) + 16));
  a.items = static_cast<uint32_t*>(c->split_items.ptr);
  a.n_items = reinterpret_cast<uint32_t*>(static_cast<char*>(c->split_items.ptr) + (size_t)a.n_slots * R * 4);
  const size_t before = c->split_done.bytes;
  CUDA_TRY(c, c->split_done.ensure((size_t)a.n_slots * sizeof(unsigned int)));
  if (c->split_done.bytes != before) CUDA_TRY(c, cudaMemsetAsync(c->split_done.ptr, 0, c->split_done.bytes, s));
  a.chunk_done = static_cast<unsigned int*>(c->split_done.ptr);
  a.work_counter = static_cast<unsigned int*>(c->work.ptr);
  const bool many = R >= kAutoRankSplitRanks;
  if (c->split_grid_n_tf != c->n_tf || c->split_grid_many != many) {
    const int per_sm = render_split_blocks_per_sm(c->n_tf, many);
    if (per_sm <= 0) return c->fail(ALOHA_ERR_CUDA, "render occupancy query failed");
    c->split_grid_blocks = per_sm * c->num_sms;
    c->split_grid_n_tf = c->n_tf;
    c->split_grid_many = many;
  }
  CUDA_TRY(c, launch_render_split(a, c->split_grid_blocks, many, s));
  return ALOHA_OK;
}

// The cost-ordered chunk list of a single view when the chunk-order mode asks
// for one (probe and sort kernels on `s`); *order stays null for ring order.
// Automatic mode orders frames of 512^2 pixels or more when auto_order is set.
// The probe also zeroes the given counters (only when *order is set).
int plan_chunk_order(aloha_ctx* c, const FrameArgs& f, int view, int cw, int ch, cudaStream_t s, const int** order,
                     int* chunks, bool auto_order, unsigned int* zero_work, unsigned long long* zero_samples) {
  const ViewState& v = c->views[view];
  *order = nullptr;
  const bool probed = c->chunk_order_mode == ALOHA_CHUNKS_PROBED ||
                      (c->chunk_order_mode == ALOHA_CHUNKS_AUTO && auto_order &&
                       (long long)v.width * v.height >= 512ll * 512ll);
  if (!probed) return ALOHA_OK;
  ChunkOrderArgs o{};
  o.f = f;
  o.view = view;
  o.cw = cw;
  o.ch = ch;
  o.n_slots = ring_slots(v.width, v.height, cw, ch);
  const size_t n_chunks = (size_t)((v.width + cw - 1) / cw) * ((v.height + ch - 1) / ch);
  const size_t slots = (size_t)o.n_slots, hist = (size_t)kOrderClasses * chunk_order_blocks(o.n_slots);
  const size_t key_words = (slots + 3) / 4;  // uint8 keys, padded to whole words
  const size_t before = c->chunk_order.bytes;
  CUDA_TRY(c, c->chunk_order.ensure((key_words + slots + hist + n_chunks) * sizeof(uint32_t)));
  uint32_t* w = static_cast<uint32_t*>(c->chunk_order.ptr);
  o.key = reinterpret_cast<uint8_t*>(w);
  o.cid = reinterpret_cast<int*>(w + key_words);
  o.hist = w + key_words + slots;
  o.order = reinterpret_cast<int*>(w + key_words + slots + hist);
  o.n_chunks = (int)n_chunks;
  // the histogram is zero between launches of one layout (the scatter clears
  // it); a new buffer or another slot count puts it elsewhere
  if (c->chunk_order.bytes != before || c->chunk_order_slots != o.n_slots) {
    CUDA_TRY(c, cudaMemsetAsync(o.hist, 0, hist * sizeof(uint32_t), s));
    c->chunk_order_slots = o.n_slots;
  }
  o.zero_work = zero_work;
  o.zero_samples = zero_samples;
  CUDA_TRY(c, launch_chunk_order(o, s));
  *order = o.order;
  *chunks = (int)n_chunks;
  return ALOHA_OK;
}

// One persistent render launch of a single view (resets the work counter).
// Zeroes the sample counter f.counter and the work counter itself (in the
// chunk probe when there is one).
int launch_single(aloha_ctx* c, const FrameArgs& f, int view, cudaStream_t s) {
  const ViewState& v = c->views[view];
  if (use_rank_split(c, f, v)) {
    CUDA_TRY(c, cudaMemsetAsync(f.counter, 0, sizeof(unsigned long long), s));
    return launch_split(c, f, view, s);
  }
  if (c->split_mode == ALOHA_SPLIT_RANKS && f.fb && !f.rank_images && !f.rank_depth && c->n_ranks > 1) {
    if (c->n_ranks > kSplitMaxRanks)
      return c->fail(ALOHA_ERR_UNSUPPORTED, "rank split: %d ranks exceed %d", c->n_ranks, kSplitMaxRanks);
    if (split_scratch_bytes(c, v) > kSplitScratchCap)
      return c->fail(ALOHA_ERR_UNSUPPORTED, "rank split: scratch of %zu bytes exceeds 16 GiB", split_scratch_bytes(c, v));
  }
  // automatic chunk: single 8x4 sub-tiles.  A frame ends with its slowest
  // chunk (a few long rays), so the smallest chunk ends it soonest: at 1024^2
  // on 512^3 in 8 bricks, 8x4 took 1.11 ms and 8x8 1.43 ms.
  int cw = c->chunk_w, ch = c->chunk_h;
  if (cw == 0) {
    cw = 8;
    ch = 4;
  }
  if (c->grid_n_tf != c->n_tf || c->grid_cw != cw || c->grid_ch != ch || c->grid_stage != c->staging) {
    const int per_sm = render_blocks_per_sm(cw, ch, c->n_tf, false, c->staging);
    if (per_sm <= 0) return c->fail(ALOHA_ERR_CUDA, "render occupancy query failed");
    c->grid_blocks = per_sm * c->num_sms;
    c->grid_n_tf = c->n_tf;
    c->grid_cw = cw;
    c->grid_ch = ch;
    c->grid_stage = c->staging;
  }
  BatchArgs b{};
  b.f = f;
  b.n_items = 1;
  b.single_view = view;
  b.total_tiles = ring_slots(v.width, v.height, cw, ch);
  b.work_counter = static_cast<unsigned int*>(c->work.ptr);
  int chunks = 0;
  const int* order = nullptr;
  int rc = plan_chunk_order(c, f, view, cw, ch, s, &order, &chunks, true, b.work_counter, f.counter);
  if (rc) return rc;
  if (order) {
    b.chunk_order = order;
    b.total_tiles = chunks;
  } else {
    CUDA_TRY(c, cudaMemsetAsync(c->work.ptr, 0, sizeof(unsigned int), s));
    CUDA_TRY(c, cudaMemsetAsync(f.counter, 0, sizeof(unsigned long long), s));
  }
  // lane groups for the costliest chunks (cost order, 8x4, direct loads, frame buffer only)
  bool lane_groups = false;
  if (c->lane_group_permille > 0 && order && cw == 8 && ch == 4 && c->staging == ALOHA_STAGING_NONE && f.fb &&
      !f.rank_images && !f.rank_depth && !f.accum) {
    b.group_chunks = (int)(((long long)chunks * c->lane_group_permille + 999) / 1000);
    b.total_tiles = chunks + b.group_chunks * (kLaneGroup - 1);
    lane_groups = true;
    if (c->grid_lg_n_tf != c->n_tf) {
      const int per_sm = render_blocks_per_sm(8, 4, c->n_tf, false, ALOHA_STAGING_NONE, true);
      if (per_sm <= 0) return c->fail(ALOHA_ERR_CUDA, "render occupancy query failed");
      c->grid_blocks_lg = per_sm * c->num_sms;
      c->grid_lg_n_tf = c->n_tf;
    }
  }
  const int warps_per_block = kRenderThreads / 32;
  const int grid = std::max(1, std::min(lane_groups ? c->grid_blocks_lg : c->grid_blocks,
                                        (b.total_tiles + warps_per_block - 1) / warps_per_block));
  CUDA_TRY(c, launch_render_warps(b, cw, ch, grid, false, s, c->staging, lane_groups));
  return ALOHA_OK;
}

FrameArgs frame_args(aloha_ctx* c) {
  const aloha_render_params& p = c->params;
  FrameArgs a{};
  a.bricks = static_cast<const DevBrick*>(c->bricks_dev.ptr);
  a.views = static_cast<const DevView*>(c->views_dev.ptr);
  a.sched = static_cast<const int*>(c->sched_dev.ptr);
  a.tf = static_cast<const float4*>(c->tf.ptr);
  a.n_tf = c->n_tf;
  a.dt = p.dt;
  a.et_alpha = p.et_alpha;
  a.jitter_mode = p.jitter_mode;
  a.jitter_value = p.jitter_value;
  a.crosshair = p.crosshair;
  a.spp = p.spp;
  a.accum_id = p.accum_id;
  a.accumulate = p.accumulate;
  a.heat_map = p.heat_map;
  a.heat_map_scale = p.heat_map_scale;
  a.composite_mode = p.composite_mode;
  a.island_id = p.island_id;
  a.num_islands = p.num_islands;
  a.counter = static_cast<unsigned long long*>(c->counter.ptr);
  return a;
}

int check_params(aloha_ctx* c, const aloha_render_params* p) {
  if (!(std::isfinite(p->dt) && p->dt > 0.f)) return c->fail(ALOHA_ERR_INVALID_ARGUMENT, "dt must be finite and > 0");
  if (!(std::isfinite(p->et_alpha) && p->et_alpha > 0.f))
    return c->fail(ALOHA_ERR_INVALID_ARGUMENT, "et_alpha must be finite and > 0");
  if (p->jitter_mode < 0 || p->jitter_mode > 2) return c->fail(ALOHA_ERR_INVALID_ARGUMENT, "bad jitter_mode");
  if (!std::isfinite(p->jitter_value)) return c->fail(ALOHA_ERR_INVALID_ARGUMENT, "jitter_value must be finite");
  if (p->spp < 1 || p->spp > 4096) return c->fail(ALOHA_ERR_INVALID_ARGUMENT, "spp must be in [1, 4096]");
  if (p->accum_id < 0) return c->fail(ALOHA_ERR_INVALID_ARGUMENT, "accum_id must be >= 0");
  if (p->composite_mode != ALOHA_COMPOSITE_FP32 && p->composite_mode != ALOHA_COMPOSITE_UBYTE)
    return c->fail(ALOHA_ERR_INVALID_ARGUMENT, "bad composite_mode");
  if (p->order_mode != ALOHA_ORDER_FACES && p->order_mode != ALOHA_ORDER_REFERENCE_KD)
    return c->fail(ALOHA_ERR_INVALID_ARGUMENT, "bad order_mode");
  if (p->num_islands < 1 || p->island_id < 0 || p->island_id >= p->num_islands)
    return c->fail(ALOHA_ERR_INVALID_ARGUMENT, "need num_islands >= 1 and 0 <= island_id < num_islands");
  if (!std::isfinite(p->heat_map_scale)) return c->fail(ALOHA_ERR_INVALID_ARGUMENT, "heat_map_scale not finite");
  return ALOHA_OK;
}

// partitionKD over n_ranks ranks.  It splits a group at the midplane of its
// bounds' longest axis, so bricks that are separated only along a shorter
// axis cannot be split (the reference repeats that split forever): an
// error, unless `identity_fallback` (one rank per brick, as set_bricks
// resets it), where brick b then goes to rank b without a KD tree, like an
// explicit assignment.  With one brick per rank either numbering gives the
// same frames.
int set_partition(aloha_ctx* c, int n_ranks, bool identity_fallback = false) {
  std::vector<int> br;
  std::vector<KdNode> tree;
  if (!partition_kd(c->boxes, n_ranks, br, tree)) {
    if (!identity_fallback || n_ranks != (int)c->boxes.size())
      return c->fail(ALOHA_ERR_INVALID_ARGUMENT, "partitionKD made no progress for %d ranks", n_ranks);
    br.resize(n_ranks);
    for (int b = 0; b < n_ranks; ++b) br[b] = b;
    tree.clear();
  }
  c->n_ranks = n_ranks;
  c->brick_rank = br;
  c->tree = tree;
  c->order_cache_valid = false;
  for (auto& v : c->views) v.dirty = true;
  invalidate_training(c);
  return ALOHA_OK;
}

// Copies host output bytes back after the stream finished.
int finish_host_output(aloha_ctx* c, void* host_dst, const void* dev_src, size_t bytes, cudaStream_t s) {
  CUDA_TRY(c, cudaMemcpyAsync(host_dst, dev_src, bytes, cudaMemcpyDeviceToHost, s));
  CUDA_TRY(c, cudaStreamSynchronize(s));
  return ALOHA_OK;
}

}  // namespace

namespace aloha {

int ctx_fail(aloha_ctx* c, int code, const char* fmt, ...) {
  char buf[512];
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(buf, sizeof buf, fmt, ap);
  va_end(ap);
  c->last_error = buf;
  return code;
}
int ctx_device(const aloha_ctx* c) { return c->device; }
int ctx_num_sms(const aloha_ctx* c) { return c->num_sms; }
int ctx_n_tf(const aloha_ctx* c) { return c->n_tf; }
void ctx_view_size(const aloha_ctx* c, int view, int* w, int* h) {
  *w = c->views[view].width;
  *h = c->views[view].height;
}
void ctx_frame_args(aloha_ctx* c, FrameArgs* a) { *a = frame_args(c); }
int ctx_prepare_view(aloha_ctx* c, int view, cudaStream_t s) { return prepare_view(c, view, s); }
void ctx_mark_samples(aloha_ctx* c) { c->samples_valid = true; }
bool ctx_is_device_pointer(const void* p) { return is_device_pointer(p); }
bool device_pointer_on(const void* p, int device) {
  cudaPointerAttributes attr;
  if (cudaPointerGetAttributes(&attr, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (attr.type == cudaMemoryTypeManaged) return true;
  return attr.type == cudaMemoryTypeDevice && attr.device == device;
}

}  // namespace aloha

extern "C" {

int aloha_abi_version(void) { return ALOHA_ABI_VERSION; }

const char* aloha_status_string(int status) {
  switch (status) {
    case ALOHA_OK: return "ok";
    case ALOHA_ERR_INVALID_ARGUMENT: return "invalid argument";
    case ALOHA_ERR_NULL_POINTER: return "null pointer";
    case ALOHA_ERR_OUT_OF_RANGE: return "index out of range";
    case ALOHA_ERR_NOT_READY: return "not ready";
    case ALOHA_ERR_OUT_OF_MEMORY: return "out of device memory";
    case ALOHA_ERR_CUDA: return "CUDA error";
    case ALOHA_ERR_TIMEOUT: return "device wait timed out";
    case ALOHA_ERR_MISSING_BRICK: return "missing brick";
    case ALOHA_ERR_UNSUPPORTED: return "unsupported";
    default: return "unknown status";
  }
}

int aloha_default_render_params(aloha_render_params* out) {
  if (!out) return ALOHA_ERR_NULL_POINTER;
  std::memset(out, 0, sizeof *out);
  out->dt = 0.5f;
  out->et_alpha = 0.99f;
  out->jitter_mode = ALOHA_JITTER_HASH;
  out->jitter_value = 0.f;
  out->crosshair = 0;
  out->spp = 1;
  out->accum_id = 0;
  out->accumulate = 0;
  out->heat_map = 0;
  out->heat_map_scale = 1e-5f;
  out->composite_mode = ALOHA_COMPOSITE_FP32;
  out->island_id = 0;
  out->num_islands = 1;
  out->order_mode = ALOHA_ORDER_FACES;
  return ALOHA_OK;
}

int aloha_create(int device, aloha_ctx** out) {
  if (!out) return ALOHA_ERR_NULL_POINTER;
  *out = nullptr;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
    cudaGetLastError();
    return ALOHA_ERR_CUDA;
  }
  if (device < 0 || device >= count) return ALOHA_ERR_OUT_OF_RANGE;
  cudaDeviceProp prop;
  if (cudaGetDeviceProperties(&prop, device) != cudaSuccess) return ALOHA_ERR_CUDA;
  // kernels are built for sm_103a only
  if (prop.major != 10 || prop.minor != 3) return ALOHA_ERR_UNSUPPORTED;
  if (cudaSetDevice(device) != cudaSuccess) return ALOHA_ERR_CUDA;
  aloha_ctx* c = new (std::nothrow) aloha_ctx();
  if (!c) return ALOHA_ERR_OUT_OF_MEMORY;
  c->device = device;
  c->num_sms = prop.multiProcessorCount;
  aloha_default_render_params(&c->params);
  if (c->views_dev.ensure(sizeof(DevView) * kMaxViews) != cudaSuccess ||
      c->counter.ensure(sizeof(unsigned long long)) != cudaSuccess || c->flag.ensure(sizeof(int)) != cudaSuccess ||
      c->work.ensure(sizeof(unsigned int)) != cudaSuccess) {
    delete c;
    return ALOHA_ERR_OUT_OF_MEMORY;
  }
  *out = c;
  return ALOHA_OK;
}

int aloha_destroy(aloha_ctx* c) {
  if (!c) return ALOHA_ERR_NULL_POINTER;
  cudaSetDevice(c->device);
  cudaDeviceSynchronize();
  for (auto& v : c->views) {
    if (v.accum) cudaFree(v.accum);
    v.train.release();
  }
  for (DeviceBuffer* b : {&c->voxels, &c->bricks_dev, &c->staging_in, &c->tf, &c->views_dev, &c->sched_dev,
                          &c->counter, &c->flag, &c->staging_out, &c->mc_ranges, &c->mc_empty, &c->tf_prefix,
                          &c->work, &c->grad4, &c->split_images, &c->split_masks, &c->split_items,
                          &c->split_done, &c->chunk_order})
    b->release();
  delete c;
  return ALOHA_OK;
}

const char* aloha_last_error(const aloha_ctx* c) { return c ? c->last_error.c_str() : "null context"; }

int aloha_set_render_params(aloha_ctx* c, const aloha_render_params* p) {
  if (!c || !p) return ALOHA_ERR_NULL_POINTER;
  int rc = check_params(c, p);
  if (rc) return rc;
  if (p->order_mode != c->params.order_mode)
    for (auto& v : c->views) v.dirty = true;
  c->params = *p;
  invalidate_training(c);
  return ALOHA_OK;
}

// Uploads one brick's voxels into its padded slot.
static int upload_brick(aloha_ctx* c, int b, const float* src) {
  const aloha_brick_desc& d = c->descs[b];
  const int nx = d.voxel_hi[0] - d.voxel_lo[0], ny = d.voxel_hi[1] - d.voxel_lo[1], nz = d.voxel_hi[2] - d.voxel_lo[2];
  const size_t raw = (size_t)nx * ny * nz;
  const float* dsrc = src;
  if (!is_device_pointer(src)) {
    CUDA_TRY(c, c->staging_in.ensure(raw * sizeof(float)));
    CUDA_TRY(c, cudaMemcpy(c->staging_in.ptr, src, raw * sizeof(float), cudaMemcpyHostToDevice));
    dsrc = static_cast<const float*>(c->staging_in.ptr);
  }
  const DevBrick& db = c->dev_bricks[b];
  float4* alloc = static_cast<float4*>(c->voxels.ptr) + c->brick_offset[b];
  CUDA_TRY(c, cudaMemset(c->flag.ptr, 0, sizeof(int)));
  CUDA_TRY(c, launch_pad_brick(dsrc, nx, ny, nz, alloc, db.sy, db.sz / db.sy, nz + 2 * kApron,
                               static_cast<int*>(c->flag.ptr), 0));
  CUDA_TRY(c, launch_macrocell_range(db, static_cast<float2*>(c->mc_ranges.ptr) + c->mc_offset[b], 0));
  c->empty_dirty = true;
  int bad = 0;  // this copy also waits for the two kernels above
  CUDA_TRY(c, cudaMemcpy(&bad, c->flag.ptr, sizeof(int), cudaMemcpyDeviceToHost));
  if (bad) return c->fail(ALOHA_ERR_INVALID_ARGUMENT, "brick %d holds a non-finite voxel", b);
  c->brick_present[b] = 1;
  invalidate_training(c);
  return ALOHA_OK;
}

int aloha_set_bricks(aloha_ctx* c, const aloha_brick_desc* descs, const float* const* voxels, int n) {
  if (!c || !descs || !voxels) return ALOHA_ERR_NULL_POINTER;
  if (n <= 0 || n > 65536) return c->fail(ALOHA_ERR_INVALID_ARGUMENT, "brick count %d not in [1, 65536]", n);
  CUDA_TRY(c, cudaSetDevice(c->device));
  size_t total = 0;
  std::vector<size_t> offs(n);
  std::vector<DevBrick> db(n);
  for (int b = 0; b < n; ++b) {
    const aloha_brick_desc& d = descs[b];
    if (!voxels[b]) return c->fail(ALOHA_ERR_NULL_POINTER, "voxels[%d] is null", b);
    int nsz[3];
    for (int a = 0; a < 3; ++a) {
      const long long size = (long long)d.voxel_hi[a] - d.voxel_lo[a];
      if (size <= 0 || size > 16384)
        return c->fail(ALOHA_ERR_INVALID_ARGUMENT, "brick %d: voxel range size %lld on axis %d", b, size, a);
      nsz[a] = (int)size;
      if (!(std::isfinite(d.space_lo[a]) && std::isfinite(d.space_hi[a]) && d.space_lo[a] < d.space_hi[a]))
        return c->fail(ALOHA_ERR_INVALID_ARGUMENT, "brick %d: empty or non-finite space range", b);
    }
    // rows padded to an even number of quads (32-byte aligned rows)
    const int px = ((nsz[0] + 2 * kApron) + 1) & ~1, py = nsz[1] + 2 * kApron, pz = nsz[2] + 2 * kApron;
    const size_t elems = (size_t)px * py * pz;
    if (elems >= (size_t)1 << 31)
      return c->fail(ALOHA_ERR_INVALID_ARGUMENT, "brick %d too large for 32-bit voxel offsets; split it", b);
    offs[b] = total;
    total += (elems + 15) & ~(size_t)15;  // 256-byte aligned bricks (in quads)
    db[b].sy = px;
    db[b].sz = px * py;
    for (int a = 0; a < 3; ++a) {
      db[b].n[a] = nsz[a];
      db[b].lo[a] = (float)d.voxel_lo[a];
      db[b].space_lo[a] = d.space_lo[a];
      db[b].space_hi[a] = d.space_hi[a];
    }
  }
  size_t free_b = 0, total_b = 0;
  CUDA_TRY(c, cudaMemGetInfo(&free_b, &total_b));
  if (total * sizeof(float4) > free_b + c->voxels.bytes)
    return c->fail(ALOHA_ERR_OUT_OF_MEMORY, "bricks need %zu bytes, %zu free", total * sizeof(float4), free_b);
  CUDA_TRY(c, cudaDeviceSynchronize());
  CUDA_TRY(c, c->voxels.ensure(total * sizeof(float4)));
  for (int b = 0; b < n; ++b)
    db[b].base = static_cast<const float4*>(c->voxels.ptr) + offs[b] + (size_t)kApron * db[b].sz +
                 (size_t)kApron * db[b].sy + kApron;
  std::vector<size_t> mc_off(n);
  size_t mc_total = 0;
  for (int b = 0; b < n; ++b) {
    mc_off[b] = mc_total;
    mc_total += (size_t)macrocells(db[b]);
  }
  CUDA_TRY(c, c->mc_ranges.ensure(mc_total * sizeof(float2)));
  CUDA_TRY(c, c->mc_empty.ensure(mc_total));
  for (int b = 0; b < n; ++b) db[b].empty = static_cast<const uint8_t*>(c->mc_empty.ptr) + mc_off[b];
  c->mc_offset = mc_off;
  c->mc_total = mc_total;
  c->empty_dirty = true;
  c->descs.assign(descs, descs + n);
  c->dev_bricks = db;
  c->brick_offset = offs;
  c->brick_present.assign(n, 0);
  c->boxes.resize(n);
  for (int a = 0; a < 3; ++a) {
    c->bounds_lo[a] = 1e30f;
    c->bounds_hi[a] = -1e30f;
  }
  for (int b = 0; b < n; ++b)
    for (int a = 0; a < 3; ++a) {
      c->boxes[b].lo[a] = descs[b].space_lo[a];
      c->boxes[b].hi[a] = descs[b].space_hi[a];
      c->bounds_lo[a] = std::min(c->bounds_lo[a], descs[b].space_lo[a]);
      c->bounds_hi[a] = std::max(c->bounds_hi[a], descs[b].space_hi[a]);
    }
  CUDA_TRY(c, c->bricks_dev.ensure(sizeof(DevBrick) * n));
  CUDA_TRY(c, cudaMemcpy(c->bricks_dev.ptr, db.data(), sizeof(DevBrick) * n, cudaMemcpyHostToDevice));
  for (int b = 0; b < n; ++b) {
    int rc = upload_brick(c, b, voxels[b]);
    if (rc) {
      c->descs.clear();
      return rc;
    }
  }
  c->staging_in.release();
  c->sched_stride = 0;
  return set_partition(c, n, true);
}

int aloha_update_brick(aloha_ctx* c, int brick, const float* voxels) {
  if (!c || !voxels) return ALOHA_ERR_NULL_POINTER;
  if (brick < 0 || brick >= (int)c->descs.size()) return c->fail(ALOHA_ERR_OUT_OF_RANGE, "brick %d", brick);
  CUDA_TRY(c, cudaSetDevice(c->device));
  CUDA_TRY(c, cudaDeviceSynchronize());
  return upload_brick(c, brick, voxels);
}

int aloha_drop_brick(aloha_ctx* c, int brick) {
  if (!c) return ALOHA_ERR_NULL_POINTER;
  if (brick < 0 || brick >= (int)c->descs.size()) return c->fail(ALOHA_ERR_OUT_OF_RANGE, "brick %d", brick);
  c->brick_present[brick] = 0;
  return ALOHA_OK;
}

int aloha_set_transfer_function(aloha_ctx* c, const float* rgba, int n) {
  if (!c || !rgba) return ALOHA_ERR_NULL_POINTER;
  if (n < 1 || n > kMaxTF) return c->fail(ALOHA_ERR_INVALID_ARGUMENT, "transfer function size %d not in [1, %d]", n, kMaxTF);
  CUDA_TRY(c, cudaSetDevice(c->device));
  std::vector<float> h((size_t)n * 4);
  if (is_device_pointer(rgba))
    CUDA_TRY(c, cudaMemcpy(h.data(), rgba, h.size() * sizeof(float), cudaMemcpyDeviceToHost));
  else
    std::memcpy(h.data(), rgba, h.size() * sizeof(float));
  for (float v : h)
    if (!std::isfinite(v)) return c->fail(ALOHA_ERR_INVALID_ARGUMENT, "transfer function holds a non-finite value");
  CUDA_TRY(c, cudaDeviceSynchronize());
  CUDA_TRY(c, c->tf.ensure(h.size() * sizeof(float)));
  CUDA_TRY(c, cudaMemcpy(c->tf.ptr, h.data(), h.size() * sizeof(float), cudaMemcpyHostToDevice));
  // prefix counts of entries with non-zero alpha, for the empty-space masks
  std::vector<int> prefix(n + 1, 0);
  for (int i = 0; i < n; ++i) prefix[i + 1] = prefix[i] + (h[(size_t)i * 4 + 3] != 0.0f ? 1 : 0);
  CUDA_TRY(c, c->tf_prefix.ensure(prefix.size() * sizeof(int)));
  CUDA_TRY(c, cudaMemcpy(c->tf_prefix.ptr, prefix.data(), prefix.size() * sizeof(int), cudaMemcpyHostToDevice));
  c->empty_dirty = true;
  c->n_tf = n;
  invalidate_training(c);
  return ALOHA_OK;
}

int aloha_set_ranks(aloha_ctx* c, int n_ranks) {
  if (!c) return ALOHA_ERR_NULL_POINTER;
  if (c->descs.empty()) return c->fail(ALOHA_ERR_NOT_READY, "no bricks uploaded");
  if (n_ranks < 1 || n_ranks > (int)c->descs.size())
    return c->fail(ALOHA_ERR_INVALID_ARGUMENT, "n_ranks %d not in [1, %zu]", n_ranks, c->descs.size());
  return set_partition(c, n_ranks);
}

int aloha_set_rank_assignment(aloha_ctx* c, const int* brick_rank, int n_bricks, int n_ranks) {
  if (!c || !brick_rank) return ALOHA_ERR_NULL_POINTER;
  if (n_bricks != (int)c->descs.size())
    return c->fail(ALOHA_ERR_INVALID_ARGUMENT, "assignment covers %d bricks, context has %zu", n_bricks, c->descs.size());
  if (n_ranks < 1 || n_ranks > n_bricks) return c->fail(ALOHA_ERR_INVALID_ARGUMENT, "bad n_ranks %d", n_ranks);
  for (int b = 0; b < n_bricks; ++b)
    if (brick_rank[b] < 0 || brick_rank[b] >= n_ranks)
      return c->fail(ALOHA_ERR_MISSING_BRICK, "brick %d is assigned to no rank", b);
  c->n_ranks = n_ranks;
  c->brick_rank.assign(brick_rank, brick_rank + n_bricks);
  c->tree.clear();
  c->order_cache_valid = false;
  for (auto& v : c->views) v.dirty = true;
  invalidate_training(c);
  return ALOHA_OK;
}

int aloha_set_camera(aloha_ctx* c, int view, const float* org, const float* dir_00, const float* dir_du,
                     const float* dir_dv) {
  if (!c || !org || !dir_00 || !dir_du || !dir_dv) return ALOHA_ERR_NULL_POINTER;
  if (view < 0 || view >= kMaxViews) return c->fail(ALOHA_ERR_OUT_OF_RANGE, "view %d not in [0, %d)", view, kMaxViews);
  if (!finite3(org) || !finite3(dir_00) || !finite3(dir_du) || !finite3(dir_dv))
    return c->fail(ALOHA_ERR_INVALID_ARGUMENT, "camera holds a non-finite value");
  if ((int)c->views.size() <= view) c->views.resize(view + 1);
  ViewState& v = c->views[view];
  std::memcpy(v.org, org, 12);
  std::memcpy(v.dir_00, dir_00, 12);
  std::memcpy(v.dir_du, dir_du, 12);
  std::memcpy(v.dir_dv, dir_dv, 12);
  v.has_camera = true;
  v.train.valid = false;
  v.dirty = true;
  return ALOHA_OK;
}

int aloha_resize(aloha_ctx* c, int view, int width, int height) {
  if (!c) return ALOHA_ERR_NULL_POINTER;
  if (view < 0 || view >= kMaxViews) return c->fail(ALOHA_ERR_OUT_OF_RANGE, "view %d not in [0, %d)", view, kMaxViews);
  if (width < 1 || height < 1 || width > 32768 || height > 32768 || (long long)width * height > (1ll << 30))
    return c->fail(ALOHA_ERR_INVALID_ARGUMENT, "frame size %dx%d out of range", width, height);
  if ((int)c->views.size() <= view) c->views.resize(view + 1);
  ViewState& v = c->views[view];
  if (v.width != width || v.height != height) {
    if (v.accum) cudaFree(v.accum);
    v.accum = nullptr;
    v.accum_elems = 0;
  }
  v.width = width;
  v.height = height;
  v.has_size = true;
  v.train.valid = false;
  v.dirty = true;
  return ALOHA_OK;
}

int aloha_get_composite_order(aloha_ctx* c, int view, int* rank_order, int max_ranks, int* n_ranks) {
  if (!c || !rank_order || !n_ranks) return ALOHA_ERR_NULL_POINTER;
  CUDA_TRY(c, cudaSetDevice(c->device));
  int rc = prepare_view(c, view, 0);
  if (rc) return rc;
  CUDA_TRY(c, cudaStreamSynchronize(0));
  const std::vector<int>& o = c->views[view].sched.rank_order;
  if ((int)o.size() > max_ranks) return c->fail(ALOHA_ERR_INVALID_ARGUMENT, "order needs %zu entries", o.size());
  std::copy(o.begin(), o.end(), rank_order);
  *n_ranks = (int)o.size();
  return ALOHA_OK;
}

int aloha_set_render_tile(aloha_ctx* c, int tile_w, int tile_h) {
  if (!c) return ALOHA_ERR_NULL_POINTER;
  if (!(tile_w == 0 && tile_h == 0) && !known_chunk(tile_w, tile_h))
    return c->fail(ALOHA_ERR_INVALID_ARGUMENT, "tile %dx%d not one of 0x0 (auto), 8x4, 8x8, 16x8, 32x4", tile_w,
                   tile_h);
  c->chunk_w = tile_w;
  c->chunk_h = tile_h;
  return ALOHA_OK;
}

int aloha_set_chunk_order(aloha_ctx* c, int mode) {
  if (!c) return ALOHA_ERR_NULL_POINTER;
  if (mode != ALOHA_CHUNKS_AUTO && mode != ALOHA_CHUNKS_RING && mode != ALOHA_CHUNKS_PROBED)
    return c->fail(ALOHA_ERR_INVALID_ARGUMENT, "chunk order %d not AUTO (0), RING (1) or PROBED (2)", mode);
  c->chunk_order_mode = mode;
  return ALOHA_OK;
}

int aloha_set_render_staging(aloha_ctx* c, int mode) {
  if (!c) return ALOHA_ERR_NULL_POINTER;
  if (mode != ALOHA_STAGING_NONE && mode != ALOHA_STAGING_NEXT_SAMPLE)
    return c->fail(ALOHA_ERR_INVALID_ARGUMENT, "staging %d not NONE (0) or NEXT_SAMPLE (1)", mode);
  c->staging = mode;
  return ALOHA_OK;
}

int aloha_set_lane_groups(aloha_ctx* c, int permille) {
  if (!c) return ALOHA_ERR_NULL_POINTER;
  if (permille < 0 || permille > 1000)
    return c->fail(ALOHA_ERR_INVALID_ARGUMENT, "lane-group share %d not in [0, 1000] per mille", permille);
  c->lane_group_permille = permille;
  return ALOHA_OK;
}

int aloha_set_render_split(aloha_ctx* c, int mode) {
  if (!c) return ALOHA_ERR_NULL_POINTER;
  if (mode != ALOHA_SPLIT_AUTO && mode != ALOHA_SPLIT_PIXELS && mode != ALOHA_SPLIT_RANKS)
    return c->fail(ALOHA_ERR_INVALID_ARGUMENT, "split mode %d not AUTO (0), PIXELS (1) or RANKS (2)", mode);
  c->split_mode = mode;
  return ALOHA_OK;
}

int aloha_render(aloha_ctx* c, int view, uint32_t* fb, void* stream) {
  if (!c || !fb) return ALOHA_ERR_NULL_POINTER;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  CUDA_TRY(c, cudaSetDevice(c->device));
  int rc = prepare_view(c, view, s);
  if (rc) return rc;
  const ViewState& v = c->views[view];
  FrameArgs a = frame_args(c);
  rc = prepare_accum(c, view, s, &a.accum);
  if (rc) return rc;
  const size_t npx = (size_t)v.width * v.height;
  // A pinned host frame buffer is written by the kernel directly; pageable
  // host memory goes through a device staging buffer.
  void* pinned = nullptr;
  const bool host = !classify_output(fb, &pinned);
  if (pinned) {
    a.fb = static_cast<uint32_t*>(pinned);
  } else if (host) {
    CUDA_TRY(c, c->staging_out.ensure(npx * sizeof(uint32_t)));
    a.fb = static_cast<uint32_t*>(c->staging_out.ptr);
  } else {
    a.fb = fb;
  }
  rc = launch_single(c, a, view, s);
  if (rc) return rc;
  c->samples_valid = true;
  if (pinned) {
    CUDA_TRY(c, cudaStreamSynchronize(s));
    return ALOHA_OK;
  }
  if (host) return finish_host_output(c, fb, a.fb, npx * sizeof(uint32_t), s);
  return ALOHA_OK;
}

int aloha_render_partials(aloha_ctx* c, int view, float* rank_images, float* rank_depth, void* stream) {
  if (!c || !rank_images) return ALOHA_ERR_NULL_POINTER;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  CUDA_TRY(c, cudaSetDevice(c->device));
  int rc = prepare_view(c, view, s);
  if (rc) return rc;
  const ViewState& v = c->views[view];
  FrameArgs a = frame_args(c);
  rc = prepare_accum(c, view, s, &a.accum);
  if (rc) return rc;
  const size_t npx = (size_t)v.width * v.height;
  const size_t img_bytes = (size_t)c->n_ranks * npx * sizeof(float4);
  const size_t depth_bytes = rank_depth ? (size_t)c->n_ranks * npx * sizeof(float) : 0;
  const bool host_img = !is_device_pointer(rank_images);
  const bool host_depth = rank_depth && !is_device_pointer(rank_depth);
  if (host_img || host_depth) CUDA_TRY(c, c->staging_out.ensure(img_bytes + depth_bytes));
  char* stage = static_cast<char*>(c->staging_out.ptr);
  a.rank_images = host_img ? reinterpret_cast<float4*>(stage) : reinterpret_cast<float4*>(rank_images);
  a.rank_depth = rank_depth ? (host_depth ? reinterpret_cast<float*>(stage + img_bytes) : rank_depth) : nullptr;
  a.fb = nullptr;
  rc = launch_single(c, a, view, s);
  if (rc) return rc;
  c->samples_valid = true;
  if (host_img) CUDA_TRY(c, cudaMemcpyAsync(rank_images, a.rank_images, img_bytes, cudaMemcpyDeviceToHost, s));
  if (host_depth) CUDA_TRY(c, cudaMemcpyAsync(rank_depth, a.rank_depth, depth_bytes, cudaMemcpyDeviceToHost, s));
  if (host_img || host_depth) CUDA_TRY(c, cudaStreamSynchronize(s));
  return ALOHA_OK;
}

int aloha_get_stats(aloha_ctx* c, aloha_stats* out) {
  if (!c || !out) return ALOHA_ERR_NULL_POINTER;
  CUDA_TRY(c, cudaSetDevice(c->device));
  std::memset(out, 0, sizeof *out);
  if (c->samples_valid) {
    // renders may run on any stream: wait for all of them
    CUDA_TRY(c, cudaDeviceSynchronize());
    unsigned long long n = 0;
    CUDA_TRY(c, cudaMemcpy(&n, c->counter.ptr, sizeof n, cudaMemcpyDeviceToHost));
    out->samples = n;
  }
  out->n_bricks = (int)c->descs.size();
  out->n_ranks = c->n_ranks;
  out->brick_bytes = c->voxels.bytes;
  return ALOHA_OK;
}

// ------------------------------------------------------------ composite

static int composite_common(const void* imgs, size_t img_bytes, const int* order, int n_ranks, int width, int height,
                            int mode, uint32_t* fb, void* stream, bool u8) {
  if (!imgs || !order || !fb) return ALOHA_ERR_NULL_POINTER;
  if (n_ranks < 1 || width < 1 || height < 1 || (long long)width * height > (1ll << 30))
    return ALOHA_ERR_INVALID_ARGUMENT;
  if (mode != ALOHA_COMPOSITE_FP32 && mode != ALOHA_COMPOSITE_UBYTE) return ALOHA_ERR_INVALID_ARGUMENT;
  std::vector<int> h_order(n_ranks);
  if (is_device_pointer(order)) {
    if (cudaMemcpy(h_order.data(), order, sizeof(int) * n_ranks, cudaMemcpyDeviceToHost) != cudaSuccess)
      return ALOHA_ERR_CUDA;
  } else {
    std::memcpy(h_order.data(), order, sizeof(int) * n_ranks);
  }
  for (int r : h_order)
    if (r < 0 || r >= n_ranks) return ALOHA_ERR_OUT_OF_RANGE;
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  const size_t npx = (size_t)width * height;
  const bool host_in = !is_device_pointer(imgs), host_out = !is_device_pointer(fb);
  void* d_in = nullptr;
  uint32_t* d_out = nullptr;
  int* d_order = nullptr;
  int rc = ALOHA_OK;
  auto fail = [&](int code) {
    rc = code;
    return code;
  };
  do {
    if (cudaMalloc(&d_order, sizeof(int) * n_ranks) != cudaSuccess) { fail(ALOHA_ERR_OUT_OF_MEMORY); break; }
    if (cudaMemcpyAsync(d_order, h_order.data(), sizeof(int) * n_ranks, cudaMemcpyHostToDevice, s) != cudaSuccess) {
      fail(ALOHA_ERR_CUDA);
      break;
    }
    const void* in = imgs;
    if (host_in) {
      if (cudaMalloc(&d_in, img_bytes) != cudaSuccess) { fail(ALOHA_ERR_OUT_OF_MEMORY); break; }
      if (cudaMemcpyAsync(d_in, imgs, img_bytes, cudaMemcpyHostToDevice, s) != cudaSuccess) { fail(ALOHA_ERR_CUDA); break; }
      in = d_in;
    }
    uint32_t* out = fb;
    if (host_out) {
      if (cudaMalloc(&d_out, npx * sizeof(uint32_t)) != cudaSuccess) { fail(ALOHA_ERR_OUT_OF_MEMORY); break; }
      out = d_out;
    }
    cudaError_t e = u8 ? launch_composite_u8(static_cast<const uint32_t*>(in), d_order, n_ranks, (int)npx, out, s)
                       : launch_composite_f32(static_cast<const float4*>(in), d_order, n_ranks, (int)npx, mode, out, s);
    if (e != cudaSuccess) { fail(ALOHA_ERR_CUDA); break; }
    if (host_out && cudaMemcpyAsync(fb, out, npx * sizeof(uint32_t), cudaMemcpyDeviceToHost, s) != cudaSuccess) {
      fail(ALOHA_ERR_CUDA);
      break;
    }
  } while (0);
  // temporaries: wait for the stream before freeing them
  if (cudaStreamSynchronize(s) != cudaSuccess && rc == ALOHA_OK) rc = ALOHA_ERR_CUDA;
  if (d_in) cudaFree(d_in);
  if (d_out) cudaFree(d_out);
  if (d_order) cudaFree(d_order);
  return rc;
}

int aloha_composite_over(const float* rank_images, const int* order, int n_ranks, int width, int height, int mode,
                         uint32_t* fb, void* stream) {
  const size_t bytes = (size_t)n_ranks * width * height * sizeof(float4);
  return composite_common(rank_images, bytes, order, n_ranks, width, height, mode, fb, stream, false);
}

int aloha_composite_over_rgba8(const uint32_t* rank_fbs, const int* order, int n_ranks, int width, int height,
                               uint32_t* fb, void* stream) {
  const size_t bytes = (size_t)n_ranks * width * height * sizeof(uint32_t);
  return composite_common(rank_fbs, bytes, order, n_ranks, width, height, ALOHA_COMPOSITE_UBYTE, fb, stream, true);
}

}  // extern "C"

// ------------------------------------------------------ differentiable form

namespace {

int check_trainable(aloha_ctx* c) {
  const aloha_render_params& p = c->params;
  if (c->n_ranks != 1)
    return c->fail(ALOHA_ERR_UNSUPPORTED, "the differentiable form needs one virtual rank (aloha_set_ranks(ctx, 1))");
  if (p.spp != 1 || p.accum_id != 0 || p.accumulate || p.crosshair || p.heat_map || p.num_islands != 1)
    return c->fail(ALOHA_ERR_UNSUPPORTED,
                   "the differentiable form needs spp 1, accum_id 0 and no accumulation, crosshair, heat map or islands");
  return ALOHA_OK;
}

// Checkpoints per pixel: samples along a ray are at most the chord through
// the bricks' union / dt plus one per brick (the lattice restarts in every
// brick), plus slack.
unsigned checkpoint_capacity(const aloha_ctx* c, unsigned k) {
  double d2 = 0;
  for (int a = 0; a < 3; ++a) d2 += (double)(c->bounds_hi[a] - c->bounds_lo[a]) * (c->bounds_hi[a] - c->bounds_lo[a]);
  const double bound = std::sqrt(d2) / c->params.dt + 2.0 * (double)c->descs.size() + 16.0;
  // saturated (a tiny dt): the segment-count check then refuses the view
  const double per_pixel = std::ceil(bound / k) + 1.0;
  return per_pixel < 4294967295.0 ? (unsigned)per_pixel : 0xffffffffu;
}

TrainArgs train_args(aloha_ctx* c) {
  const aloha_render_params& p = c->params;
  TrainArgs a{};
  a.bricks = static_cast<const DevBrick*>(c->bricks_dev.ptr);
  a.views = static_cast<const DevView*>(c->views_dev.ptr);
  a.sched = static_cast<const int*>(c->sched_dev.ptr);
  a.tf = static_cast<const float4*>(c->tf.ptr);
  a.n_tf = c->n_tf;
  a.dt = p.dt;
  a.et_alpha = p.et_alpha;
  a.jitter_mode = p.jitter_mode;
  a.jitter_value = p.jitter_value;
  a.accum_id = p.accum_id;
  a.counter = static_cast<unsigned long long*>(c->counter.ptr);
  return a;
}

TrainView train_view(const TrainState& t, int view) {
  TrainView tv{};
  tv.ckpt = t.ckpt;
  tv.final_rgba = t.final_rgba;
  tv.work = t.work;
  tv.work_count = t.work_count;
  tv.overflow = t.overflow;
  tv.ckpt_cap = t.cap;
  tv.work_cap = (unsigned)std::min<size_t>(t.npx * t.cap, 0xffffffffu);
  tv.view = view;
  return tv;
}

// Uploads a launch's tables (one block: the item counter, zeroed, then the
// parts at 16-byte aligned offsets) and returns their device addresses.
int upload_train_tables(aloha_ctx* c, const std::vector<std::pair<const void*, size_t>>& parts, cudaStream_t s,
                        std::vector<char*>& dev) {
  std::vector<size_t> off(parts.size());
  size_t total = 16;
  for (size_t i = 0; i < parts.size(); ++i) {
    off[i] = total;
    total += (parts[i].second + 15) & ~(size_t)15;
  }
  std::vector<char> host(total, 0);
  for (size_t i = 0; i < parts.size(); ++i)
    if (parts[i].second) std::memcpy(host.data() + off[i], parts[i].first, parts[i].second);
  CUDA_TRY(c, c->train_tables.ensure(total));
  char* base = static_cast<char*>(c->train_tables.ptr);
  // pageable source: staged by the runtime before the call returns
  CUDA_TRY(c, cudaMemcpyAsync(base, host.data(), total, cudaMemcpyHostToDevice, s));
  dev.assign(parts.size() + 1, nullptr);
  dev[0] = base;
  for (size_t i = 0; i < parts.size(); ++i) dev[i + 1] = base + off[i];
  return ALOHA_OK;
}

// The training forward of several views in one persistent launch: each
// view's checkpoints, final colour and segment list as aloha_forward keeps
// them.  One view keeps its cost-ordered chunks (frames of 512^2 and up);
// several march their chunks centre-out, position-major across the views.
int forward_views(aloha_ctx* c, int n_views, const int* view_ids, float* const* rgba, int checkpoint_every,
                  void* stream) {
  if (!c) return ALOHA_ERR_NULL_POINTER;
  if (n_views < 1) return c->fail(ALOHA_ERR_INVALID_ARGUMENT, "no views");
  if (!view_ids || !rgba) return c->fail(ALOHA_ERR_NULL_POINTER, "no view list");
  if (checkpoint_every < 1 || checkpoint_every > 65535)
    return c->fail(ALOHA_ERR_INVALID_ARGUMENT, "checkpoint_every %d not in [1, 65535]", checkpoint_every);
  for (int i = 0; i < n_views; ++i) {
    if (!rgba[i]) return c->fail(ALOHA_ERR_NULL_POINTER, "no image for view %d", view_ids[i]);
    for (int j = 0; j < i; ++j)
      if (view_ids[j] == view_ids[i]) return c->fail(ALOHA_ERR_INVALID_ARGUMENT, "view %d given twice", view_ids[i]);
  }
  int rc = check_trainable(c);
  if (rc) return rc;
  if ((int)c->descs.size() > 65535) return c->fail(ALOHA_ERR_UNSUPPORTED, "more than 65535 bricks");
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  CUDA_TRY(c, cudaSetDevice(c->device));
  const unsigned k = (unsigned)checkpoint_every;
  const unsigned cap = checkpoint_capacity(c, k);
  std::vector<TrainView> tvs(n_views);
  std::vector<char> host_out(n_views, 0);
  for (int i = 0; i < n_views; ++i) {
    const int view = view_ids[i];
    rc = prepare_view(c, view, s);
    if (rc) return rc;
    ViewState& v = c->views[view];
    TrainState& t = v.train;
    t.valid = false;
    const size_t npx = (size_t)v.width * v.height;
    if (npx * cap > 0xffffffffull)
      return c->fail(ALOHA_ERR_UNSUPPORTED, "too many checkpoint segments for view %d", view);
    const size_t need = npx * cap * (sizeof(Checkpoint) + sizeof(uint2)) + npx * sizeof(float4);
    if (t.npx != npx || t.cap != cap) {
      CUDA_TRY(c, cudaStreamSynchronize(s));
      t.release();
      size_t free_b = 0, total_b = 0;
      CUDA_TRY(c, cudaMemGetInfo(&free_b, &total_b));
      if (need > free_b)
        return c->fail(ALOHA_ERR_OUT_OF_MEMORY, "checkpoints of view %d need %zu bytes, %zu free", view, need, free_b);
      CUDA_TRY(c, cudaMalloc(&t.ckpt, npx * cap * sizeof(Checkpoint)));
      CUDA_TRY(c, cudaMalloc(&t.work, npx * cap * sizeof(uint2)));
      CUDA_TRY(c, cudaMalloc(&t.final_rgba, npx * sizeof(float4)));
      CUDA_TRY(c, cudaMalloc(&t.work_count, 4 * sizeof(unsigned)));
      CUDA_TRY(c, cudaMalloc(&t.overflow, sizeof(int)));
      t.npx = npx;
      t.cap = cap;
      t.bytes = need;
    }
    t.k = k;
    tvs[i] = train_view(t, view);
    host_out[i] = !is_device_pointer(rgba[i]);
    tvs[i].out_rgba = host_out[i] ? nullptr : reinterpret_cast<float4*>(rgba[i]);
    CUDA_TRY(c, cudaMemsetAsync(t.work_count, 0, 4 * sizeof(unsigned), s));
    CUDA_TRY(c, cudaMemsetAsync(t.overflow, 0, sizeof(int), s));
    tvs[i].n_chunks = ring_slots(v.width, v.height, 8, 4);
  }
  if (n_views == 1) {
    const int* order = nullptr;
    int chunks = 0;
    rc = plan_chunk_order(c, frame_args(c), view_ids[0], 8, 4, s, &order, &chunks);
    if (rc) return rc;
    if (order) {
      tvs[0].chunk_order = order;
      tvs[0].n_chunks = chunks;
    }
  }
  // position-major runs over the views sorted by positions, descending
  std::vector<int> by_size(n_views);
  for (int i = 0; i < n_views; ++i) by_size[i] = i;
  std::stable_sort(by_size.begin(), by_size.end(),
                   [&](int x, int y) { return tvs[x].n_chunks > tvs[y].n_chunks; });
  std::vector<TrainRun> runs;
  unsigned long long items = 0;
  int p = 0;
  for (int active = n_views; active > 0; --active) {
    const int p_end = tvs[by_size[active - 1]].n_chunks;  // views [0, active) have positions below p_end
    if (p_end <= p) continue;
    runs.push_back(TrainRun{p, active, (unsigned)items, 0u});
    items += (unsigned long long)(p_end - p) * (unsigned)active;
    p = p_end;
  }
  if (items >= 0xffffffffull) return c->fail(ALOHA_ERR_UNSUPPORTED, "too many chunks in one training forward");
  const int n_runs = (int)runs.size();
  runs.push_back(TrainRun{p, 1, (unsigned)items, 0u});
  std::vector<char*> dev;
  rc = upload_train_tables(c, {{tvs.data(), tvs.size() * sizeof(TrainView)},
                               {runs.data(), runs.size() * sizeof(TrainRun)},
                               {by_size.data(), by_size.size() * sizeof(int)}}, s, dev);
  if (rc) return rc;
  TrainArgs a = train_args(c);
  a.k = k;
  a.grab = reinterpret_cast<unsigned*>(dev[0]);
  a.tv = reinterpret_cast<const TrainView*>(dev[1]);
  a.n_views = n_views;
  a.runs = reinterpret_cast<const TrainRun*>(dev[2]);
  a.n_runs = n_runs;
  a.run_views = reinterpret_cast<const int*>(dev[3]);
  CUDA_TRY(c, cudaMemsetAsync(c->counter.ptr, 0, sizeof(unsigned long long), s));
  // few chunks per resident warp: the launch ends on its longest rays (fewer,
  // faster warps); many: throughput-bound (more warps)
  const int few_per_sm = forward_train_blocks_per_sm(c->n_tf, false);
  if (few_per_sm <= 0) return c->fail(ALOHA_ERR_CUDA, "forward occupancy query failed");
  const bool many = items >= (unsigned long long)kTrainManyChunksPerWarp * few_per_sm * c->num_sms * 4;
  const int per_sm = many ? forward_train_blocks_per_sm(c->n_tf, true) : few_per_sm;
  if (per_sm <= 0) return c->fail(ALOHA_ERR_CUDA, "forward occupancy query failed");
  CUDA_TRY(c, launch_forward_train(a, (unsigned)items, per_sm * c->num_sms, many, s));
  c->samples_valid = true;
  bool any_host = false;
  for (int i = 0; i < n_views; ++i) {
    TrainState& t = c->views[view_ids[i]].train;
    t.valid = true;
    if (host_out[i]) {
      CUDA_TRY(c, cudaMemcpyAsync(rgba[i], t.final_rgba, t.npx * sizeof(float4), cudaMemcpyDeviceToHost, s));
      any_host = true;
    }
  }
  if (any_host) CUDA_TRY(c, cudaStreamSynchronize(s));
  return ALOHA_OK;
}

// The backward of several views into one pair of gradients: the views'
// overflow flags are read with one host wait, their kernels accumulate into
// one x-quad buffer, and that buffer is cleared and folded into the density
// grid once.
int backward_views(aloha_ctx* c, int n_views, const int* view_ids, const float* const* dl_drgba, float* dl_dtf,
                   float* dl_ddensity, const int* grid_lo, const int* grid_dims, void* stream) {
  if (!c) return ALOHA_ERR_NULL_POINTER;
  if (n_views < 1) return c->fail(ALOHA_ERR_INVALID_ARGUMENT, "no views");
  if (!view_ids || !dl_drgba) return c->fail(ALOHA_ERR_NULL_POINTER, "no view list");
  if (!dl_dtf && !dl_ddensity) return c->fail(ALOHA_ERR_NULL_POINTER, "neither dl_dtf nor dl_ddensity given");
  if (dl_ddensity && (!grid_lo || !grid_dims)) return c->fail(ALOHA_ERR_NULL_POINTER, "dl_ddensity needs its grid");
  for (int i = 0; i < n_views; ++i) {
    const int view = view_ids[i];
    if (view < 0 || view >= (int)c->views.size()) return c->fail(ALOHA_ERR_OUT_OF_RANGE, "view %d", view);
    if (!dl_drgba[i]) return c->fail(ALOHA_ERR_NULL_POINTER, "no dL/dRGBA for view %d", view);
    for (int j = 0; j < i; ++j)
      if (view_ids[j] == view) return c->fail(ALOHA_ERR_INVALID_ARGUMENT, "view %d given twice", view);
  }
  int rc = check_trainable(c);
  if (rc) return rc;
  for (int i = 0; i < n_views; ++i)
    if (!c->views[view_ids[i]].train.valid)
      return c->fail(ALOHA_ERR_NOT_READY, "view %d has no forward checkpoints for the current scene and camera",
                     view_ids[i]);
  const bool with_density = dl_ddensity != nullptr;
  size_t grid_elems = 0;
  std::vector<int4> origin(with_density ? c->descs.size() : 0);
  if (with_density) {
    for (int a = 0; a < 3; ++a)
      if (grid_dims[a] < 1) return c->fail(ALOHA_ERR_INVALID_ARGUMENT, "grid dims must be positive");
    // products below 2^62, so none overflows; the fold takes the grid's (y, z)
    // rows as an int, and 2^40 voxels are far beyond any device's memory
    const unsigned long long gx = (unsigned)grid_dims[0], gy = (unsigned)grid_dims[1], gz = (unsigned)grid_dims[2];
    if (gy * gz > 0x7fffffffull || gx * (gy * gz) > (1ull << 40))
      return c->fail(ALOHA_ERR_OUT_OF_RANGE, "a gradient grid of %d x %d x %d voxels is too large", grid_dims[0],
                     grid_dims[1], grid_dims[2]);
    grid_elems = (size_t)(gx * gy * gz);
  }
  for (size_t b = 0; b < origin.size(); ++b) {
    const aloha_brick_desc& d = c->descs[b];
    for (int a = 0; a < 3; ++a)
      if (d.voxel_lo[a] < grid_lo[a] || (long long)d.voxel_hi[a] > (long long)grid_lo[a] + grid_dims[a])
        return c->fail(ALOHA_ERR_OUT_OF_RANGE, "brick %zu's voxel range leaves the gradient grid", b);
    origin[b] = make_int4(d.voxel_lo[0] - grid_lo[0], d.voxel_lo[1] - grid_lo[1], d.voxel_lo[2] - grid_lo[2], 0);
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  CUDA_TRY(c, cudaSetDevice(c->device));
  // every view's overflow flag and segment count, read with one wait
  std::vector<int> overflow(n_views, 0);
  std::vector<unsigned> segments(n_views, 0);
  for (int i = 0; i < n_views; ++i) {
    const TrainState& t = c->views[view_ids[i]].train;
    CUDA_TRY(c, cudaMemcpyAsync(&overflow[i], t.overflow, sizeof(int), cudaMemcpyDeviceToHost, s));
    CUDA_TRY(c, cudaMemcpyAsync(&segments[i], t.work_count, sizeof(unsigned), cudaMemcpyDeviceToHost, s));
  }
  CUDA_TRY(c, cudaStreamSynchronize(s));
  std::vector<unsigned> item_base(n_views + 1, 0);
  for (int i = 0; i < n_views; ++i) {
    if (overflow[i])
      return c->fail(ALOHA_ERR_OUT_OF_RANGE, "a ray of view %d needed more checkpoints than reserved", view_ids[i]);
    const TrainState& t = c->views[view_ids[i]].train;
    const unsigned long long n = std::min<unsigned long long>(segments[i], t.npx * t.cap);
    if (item_base[i] + n >= 0xffffffffull)
      return c->fail(ALOHA_ERR_UNSUPPORTED, "too many checkpoint segments in one backward");
    item_base[i + 1] = item_base[i] + (unsigned)n;
  }
  const size_t tf_bytes = (size_t)c->n_tf * 4 * sizeof(float), g_bytes = grid_elems * sizeof(float);
  const bool h_tf = dl_dtf && !is_device_pointer(dl_dtf), h_grid = with_density && !is_device_pointer(dl_ddensity);
  // device staging for host arguments, in one block: each host dL/dRGBA, dL/dtf, dL/ddensity, origins
  std::vector<size_t> off_dl(n_views, SIZE_MAX);
  size_t off = 0;
  for (int i = 0; i < n_views; ++i)
    if (!is_device_pointer(dl_drgba[i])) {
      off_dl[i] = off;
      off += c->views[view_ids[i]].train.npx * sizeof(float4);
    }
  const bool h_dl = off > 0;
  const size_t off_tf = off;
  const size_t off_grid = off_tf + (h_tf ? tf_bytes : 0);
  const size_t off_org = (off_grid + (h_grid ? g_bytes : 0) + 15) & ~(size_t)15;
  CUDA_TRY(c, c->staging_out.ensure(off_org + origin.size() * sizeof(int4)));
  char* st = static_cast<char*>(c->staging_out.ptr);
  float* dtf = h_tf ? reinterpret_cast<float*>(st + off_tf) : dl_dtf;
  float* grid_out = h_grid ? reinterpret_cast<float*>(st + off_grid) : dl_ddensity;
  float4* dgrid4 = nullptr;
  if (with_density) {
    // the kernels accumulate into x-quads (vector atomics), folded into the
    // grid afterwards; the fold leaves the buffer zero for the next call
    const size_t want = grid_elems * sizeof(float4);
    if (want > c->grad4.bytes) c->grad4_zero = false;
    CUDA_TRY(c, c->grad4.ensure(want));
    dgrid4 = static_cast<float4*>(c->grad4.ptr);
    if (!c->grad4_zero) CUDA_TRY(c, cudaMemsetAsync(dgrid4, 0, c->grad4.bytes, s));
    c->grad4_zero = false;
  }
  for (int i = 0; i < n_views; ++i)
    if (off_dl[i] != SIZE_MAX)
      CUDA_TRY(c, cudaMemcpyAsync(st + off_dl[i], dl_drgba[i], c->views[view_ids[i]].train.npx * sizeof(float4),
                                  cudaMemcpyHostToDevice, s));
  if (h_tf) CUDA_TRY(c, cudaMemcpyAsync(dtf, dl_dtf, tf_bytes, cudaMemcpyHostToDevice, s));
  if (h_grid) CUDA_TRY(c, cudaMemcpyAsync(grid_out, dl_ddensity, g_bytes, cudaMemcpyHostToDevice, s));
  if (with_density)
    CUDA_TRY(c, cudaMemcpyAsync(st + off_org, origin.data(), origin.size() * sizeof(int4), cudaMemcpyHostToDevice, s));
  const int per_sm = backward_blocks_per_sm(c->n_tf);
  if (per_sm <= 0) return c->fail(ALOHA_ERR_CUDA, "backward occupancy query failed");
  CUDA_TRY(c, cudaMemsetAsync(c->counter.ptr, 0, sizeof(unsigned long long), s));
  // one launch per checkpoint interval among the views (the interval is a
  // launch constant of the replay loop), all into the same gradients
  std::vector<char> done(n_views, 0);
  for (int first = 0; first < n_views; ++first) {
    if (done[first]) continue;
    const unsigned k = c->views[view_ids[first]].train.k;
    std::vector<TrainView> tvs;
    std::vector<unsigned> base{0};
    for (int i = first; i < n_views; ++i) {
      if (done[i] || c->views[view_ids[i]].train.k != k) continue;
      done[i] = 1;
      TrainView tv = train_view(c->views[view_ids[i]].train, view_ids[i]);
      tv.dl_drgba = off_dl[i] != SIZE_MAX ? reinterpret_cast<const float4*>(st + off_dl[i])
                                          : reinterpret_cast<const float4*>(dl_drgba[i]);
      tvs.push_back(tv);
      base.push_back(base.back() + (item_base[i + 1] - item_base[i]));
    }
    std::vector<char*> dev;
    rc = upload_train_tables(c, {{tvs.data(), tvs.size() * sizeof(TrainView)},
                                 {base.data(), base.size() * sizeof(unsigned)}}, s, dev);
    if (rc) return rc;
    TrainArgs a = train_args(c);
    a.k = k;
    a.grab = reinterpret_cast<unsigned*>(dev[0]);
    a.dtf = dtf;
    a.dgrid4 = dgrid4;
    a.brick_grid_origin = reinterpret_cast<const int4*>(st + off_org);
    if (with_density)
      for (int d = 0; d < 3; ++d) a.grid_dims[d] = grid_dims[d];
    // Views whose items give every resident thread many of them fill the GPU
    // alone: one launch each, with the view in the launch parameters (the
    // replay's registers then hold no per-view pointers).  Smaller views go
    // together into one launch, which fills the GPU with all of them.
    const unsigned long long resident = (unsigned long long)c->num_sms * per_sm * 128;
    bool all_large = true;
    for (size_t i = 0; i + 1 < base.size(); ++i)
      if ((unsigned long long)(base[i + 1] - base[i]) < 16 * resident) all_large = false;
    if (tvs.size() == 1 || all_large) {
      for (size_t i = 0; i < tvs.size(); ++i) {
        if (i > 0) CUDA_TRY(c, cudaMemsetAsync(a.grab, 0, sizeof(unsigned), s));
        a.n_views = 1;
        a.one = tvs[i];
        a.one_items = base[i + 1] - base[i];
        CUDA_TRY(c, launch_backward(a, c->num_sms * per_sm, s));
      }
    } else {
      a.tv = reinterpret_cast<const TrainView*>(dev[1]);
      a.n_views = (int)tvs.size();
      a.item_base = reinterpret_cast<const unsigned*>(dev[2]);
      CUDA_TRY(c, launch_backward(a, c->num_sms * per_sm, s));
    }
  }
  if (with_density) {
    CUDA_TRY(c, launch_fold_quads(dgrid4, grid_out, grid_dims, s));
    c->grad4_zero = true;
  }
  c->samples_valid = true;
  if (h_tf) CUDA_TRY(c, cudaMemcpyAsync(dl_dtf, dtf, tf_bytes, cudaMemcpyDeviceToHost, s));
  if (h_grid) CUDA_TRY(c, cudaMemcpyAsync(dl_ddensity, grid_out, g_bytes, cudaMemcpyDeviceToHost, s));
  if (h_dl || h_tf || h_grid) CUDA_TRY(c, cudaStreamSynchronize(s));
  return ALOHA_OK;
}

}  // namespace

extern "C" {

int aloha_forward(aloha_ctx* c, int view, float* rgba, int checkpoint_every, void* stream) {
  if (!c || !rgba) return ALOHA_ERR_NULL_POINTER;
  return forward_views(c, 1, &view, &rgba, checkpoint_every, stream);
}

int aloha_forward_views(aloha_ctx* c, int n_views, const int* views, float* const* rgba, int checkpoint_every,
                        void* stream) {
  return forward_views(c, n_views, views, rgba, checkpoint_every, stream);
}

int aloha_backward(aloha_ctx* c, int view, const float* dl_drgba, float* dl_dtf, float* dl_ddensity,
                   const int* grid_lo, const int* grid_dims, void* stream) {
  if (!c || !dl_drgba) return ALOHA_ERR_NULL_POINTER;
  return backward_views(c, 1, &view, &dl_drgba, dl_dtf, dl_ddensity, grid_lo, grid_dims, stream);
}

int aloha_backward_views(aloha_ctx* c, int n_views, const int* views, const float* const* dl_drgba, float* dl_dtf,
                         float* dl_ddensity, const int* grid_lo, const int* grid_dims, void* stream) {
  return backward_views(c, n_views, views, dl_drgba, dl_dtf, dl_ddensity, grid_lo, grid_dims, stream);
}

}  // extern "C"
