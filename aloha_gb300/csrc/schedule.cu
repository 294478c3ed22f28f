// schedule.cu -- cost-ordered chunks for single-view renders (both work
// divisions) and the differentiable forward.
//
// A frame ends with its slowest chunk (an 8x4 tile whose rays march far
// through translucent space), so the order in which warps take chunks sets
// the length of its tail: started last, a long chunk runs on an almost idle
// GPU.  Longest-first ordering needs the cost before the frame.  A coarse
// probe gives a good enough estimate: four rays of the chunk (a 2x2 sample),
// each stepped at 16 samples' stride through the bricks of every rank whose
// screen rectangle covers it, counting
// the strides that land in a non-empty macrocell (no voxel loads, no early
// termination); the chunk's cost is the largest of the four, as a warp runs
// as long as its longest ray.  The chunks are then sorted stably by cost
// class (a quarter octave each), most expensive first; ring order within a
// class keeps neighbouring chunks together.  The order only changes when a
// pixel is rendered, never how, so frames are bit-identical to ring order.
//
// Kernels: probe (4 threads per ring slot; each CTA also adds its class
// counts into its sort block's histogram column), one-CTA exclusive scan of
// the histogram table (class-major), stable scatter (which zeroes the table).
#include <cuda_runtime.h>
#include <stdint.h>

#include "internal.h"
#include "march.cuh"

namespace aloha {

namespace {

constexpr uint8_t kNoChunk = 0xff;
constexpr float kProbeStride = 16.0f;  // samples per probe step
constexpr int kProbeMaxSteps = 8192;   // per brick (the probe only estimates)
constexpr int kSortThreads = 1024;     // slots per sort block (histogram column, scatter CTA)
constexpr int kProbeThreads = 256;     // 4 per slot: 64 slots per probe CTA
constexpr int kScanThreads = 1024;

// Non-empty probe steps of one ray through every rank's bricks.
__device__ uint32_t probe_ray(const ChunkOrderArgs& a, const DevView& v, const int* __restrict__ order,
                              const int* __restrict__ rstart, const int* __restrict__ rbricks, int x, int y) {
  const Ray ray = generate_ray(v, x, y);
  const float stride = kProbeStride * a.f.dt;
  // ranks whose screen rectangle (in 8x4 chunks) misses the pixel cannot be hit
  const int* __restrict__ rects = a.f.sched + v.rects;
  const int qx = x >> 3, qy = y >> 2;
  uint32_t c = 0;
  for (int k = 0; k < v.n_ranks; ++k) {
    const int r = __ldg(order + k);
    const int* q = rects + 4 * r;
    if (qx < __ldg(q) || qy < __ldg(q + 1) || qx > __ldg(q + 2) || qy > __ldg(q + 3)) continue;
    float tmin = 0.0f;
    for (int j = __ldg(rstart + r); j < __ldg(rstart + r + 1); ++j) {
      const DevBrick b = a.f.bricks[__ldg(rbricks + j)];
      float t0, t1;
      if (!slab(ray, b.space_lo, b.space_hi, tmin, 1e10f, t0, t1)) continue;
      tmin = t1 + 1e-20f;
      const float span = (t1 - t0) / stride;
      const int steps = span < (float)kProbeMaxSteps ? (int)span + 1 : kProbeMaxSteps;
      if (!b.empty) {
        c += (uint32_t)steps;
        continue;
      }
      const int mnx = (b.n[0] + kMacro - 1) >> kMacroShift, mny = (b.n[1] + kMacro - 1) >> kMacroShift;
      for (int i = 0; i < steps; ++i) {
        const float t = fmaf((float)i, stride, t0);
        const int mx = min(max(__float2int_rd(fmaf(t, ray.d[0], ray.o[0]) - b.lo[0]), 0), b.n[0] - 1) >> kMacroShift;
        const int my = min(max(__float2int_rd(fmaf(t, ray.d[1], ray.o[1]) - b.lo[1]), 0), b.n[1] - 1) >> kMacroShift;
        const int mz = min(max(__float2int_rd(fmaf(t, ray.d[2], ray.o[2]) - b.lo[2]), 0), b.n[2] - 1) >> kMacroShift;
        c += __ldg(b.empty + (mz * mny + my) * mnx + mx) ? 0u : 1u;
      }
    }
  }
  return c;
}

// Cost class: 0 for the most expensive, one class per quarter octave.
__device__ __forceinline__ uint8_t cost_class(uint32_t c) {
  const int q = (int)(4.0f * log2f((float)c + 1.0f));
  return (uint8_t)(kOrderClasses - 1 - min(q, kOrderClasses - 1));
}

// Four threads per ring slot (lanes 4s..4s+3 of a warp): each probes one ray
// of the chunk's 2x2 sample; the slot's class comes from the largest.  A CTA
// covers kProbeThreads / 4 slots and adds its class counts into the histogram
// column of the sort block (kSortThreads slots) it belongs to.
__global__ void probe_chunks_kernel(ChunkOrderArgs a) {
  __shared__ uint32_t h[kOrderClasses];
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    if (a.zero_work) *a.zero_work = 0u;
    if (a.zero_samples) *a.zero_samples = 0ull;
  }
  for (int i = threadIdx.x; i < kOrderClasses; i += kProbeThreads) h[i] = 0;
  __syncthreads();
  const DevView& v = a.f.views[a.view];
  const int W = v.width, H = v.height, R = v.n_ranks;
  const int* __restrict__ order = a.f.sched + v.sched;
  const int cxn = (W + a.cw - 1) / a.cw, cyn = (H + a.ch - 1) / a.ch;
  const int gid = blockIdx.x * blockDim.x + threadIdx.x;
  const int slot = gid >> 2, q = gid & 3;
  uint32_t c = 0;
  bool valid = false;
  int cx = 0, cy = 0;
  if (slot < a.n_slots && ring_chunk(slot, cxn, cyn, cx, cy)) {
    valid = true;
    const int x = min(cx * a.cw + ((q & 1) ? (3 * a.cw) / 4 : a.cw / 4), W - 1);
    const int y = min(cy * a.ch + ((q & 2) ? (3 * a.ch) / 4 : a.ch / 4), H - 1);
    c = probe_ray(a, v, order, order + R, order + 2 * R + 1, x, y);
  }
  c = max(c, __shfl_xor_sync(0xffffffffu, c, 1));
  c = max(c, __shfl_xor_sync(0xffffffffu, c, 2));
  if (q == 0 && slot < a.n_slots) {
    const uint8_t k = valid ? cost_class(c) : kNoChunk;
    a.key[slot] = k;
    a.cid[slot] = cx + cxn * cy;
    if (valid) atomicAdd(&h[k], 1u);
  }
  __syncthreads();
  const int blocks = (a.n_slots + kSortThreads - 1) / kSortThreads;
  const int block = (int)(((long long)blockIdx.x * (kProbeThreads / 4)) / kSortThreads);
  for (int i = threadIdx.x; i < kOrderClasses; i += kProbeThreads)
    if (h[i]) atomicAdd(a.hist + i * blocks + block, h[i]);
}

// Exclusive scan of the histogram table in place (one CTA; each thread scans
// a contiguous range).
__global__ void __launch_bounds__(kScanThreads) class_scan_kernel(ChunkOrderArgs a, int n) {
  __shared__ uint32_t warp_sum[kScanThreads / 32];
  const int per = (n + kScanThreads - 1) / kScanThreads;
  const int lo = min(n, (int)threadIdx.x * per), hi = min(n, lo + per);
  uint32_t count = 0;
  for (int i = lo; i < hi; ++i) count += a.hist[i];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  uint32_t incl = count;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const uint32_t o = __shfl_up_sync(0xffffffffu, incl, d);
    if (lane >= d) incl += o;
  }
  if (lane == 31) warp_sum[wid] = incl;
  __syncthreads();
  if (wid == 0) {
    uint32_t w = warp_sum[lane];
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t o = __shfl_up_sync(0xffffffffu, w, d);
      if (lane >= d) w += o;
    }
    warp_sum[lane] = w;
  }
  __syncthreads();
  uint32_t at = incl - count + (wid > 0 ? warp_sum[wid - 1] : 0u);
  for (int i = lo; i < hi; ++i) {
    const uint32_t c = a.hist[i];
    a.hist[i] = at;
    at += c;
  }
}

// Stable scatter: a slot's position is its class's base for this CTA plus the
// slots of the same class before it in the CTA (earlier warps, then earlier
// lanes of its warp).
__global__ void __launch_bounds__(kSortThreads) class_scatter_kernel(ChunkOrderArgs a) {
  constexpr int kWarps = kSortThreads / 32;
  __shared__ uint32_t wc[kWarps][kOrderClasses];
  for (int i = threadIdx.x; i < kWarps * kOrderClasses; i += kSortThreads) (&wc[0][0])[i] = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int slot = blockIdx.x * kSortThreads + threadIdx.x;
  const uint8_t k = slot < a.n_slots ? a.key[slot] : kNoChunk;
  const unsigned peers = __match_any_sync(0xffffffffu, (unsigned)k);
  const unsigned rank = __popc(peers & ((1u << lane) - 1u));
  if (k != kNoChunk && lane == __ffs(peers) - 1) wc[w][k] = __popc(peers);
  __syncthreads();
  if (k != kNoChunk) {
    uint32_t pos = a.hist[k * gridDim.x + blockIdx.x] + rank;
    for (int e = 0; e < w; ++e) pos += wc[e][k];
    if (pos < (uint32_t)a.n_chunks) a.order[pos] = a.cid[slot];
  }
  // the block's histogram column is consumed: zero it for the next launch
  __syncthreads();
  for (int i = threadIdx.x; i < kOrderClasses; i += kSortThreads) a.hist[i * gridDim.x + blockIdx.x] = 0u;
}

}  // namespace

int chunk_order_blocks(int n_slots) { return (n_slots + kSortThreads - 1) / kSortThreads; }

// The histogram (a.hist, kOrderClasses x chunk_order_blocks(n_slots)) must be
// zero when this is called; the scatter leaves it zero again.
cudaError_t launch_chunk_order(const ChunkOrderArgs& a, cudaStream_t s) {
  static_assert(kSortThreads % (kProbeThreads / 4) == 0, "probe CTAs must tile sort blocks");
  const int probe_grid = (int)(((long long)a.n_slots * 4 + kProbeThreads - 1) / kProbeThreads);
  probe_chunks_kernel<<<probe_grid, kProbeThreads, 0, s>>>(a);
  const int blocks = chunk_order_blocks(a.n_slots);
  class_scan_kernel<<<1, kScanThreads, 0, s>>>(a, kOrderClasses * blocks);
  class_scatter_kernel<<<blocks, kSortThreads, 0, s>>>(a);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess)  // counts may stay behind: clear them for the next launch
    cudaMemsetAsync(a.hist, 0, (size_t)kOrderClasses * blocks * sizeof(uint32_t), s);
  return e;
}

}  // namespace aloha
