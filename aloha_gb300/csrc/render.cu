// render.cu -- forward kernels: fused per-view render, persistent batched
// render, ordered-over composite, brick padding.
#include <cuda_runtime.h>
#include <stdint.h>

#include <type_traits>

#include "internal.h"
#include "march.cuh"

namespace aloha {

// Persistent render: every warp pulls CW x CH pixel chunks of the launch's
// items (views) from one atomic counter -- a single view in cost order when
// b.chunk_order is set (schedule.cu), else centre-out per view -- and renders
// each chunk as 8 x 4-pixel sub-tiles, so the 32 rays of a warp start within
// a few voxels of each other.  Warps are independent (no barrier after the
// transfer function is staged): a warp with long rays never holds finished
// warps of its CTA, and views end without a per-launch tail.  Nothing waits
// on other warps or CTAs.
// MINB CTAs of 128 threads per SM: a single view ends with its slowest
// chunks, which run faster with more registers per thread (5 CTAs, 96
// registers); a batch of views is throughput-bound and runs faster with more
// resident warps (7 CTAs, 72 registers).
// STAGE selects the stencil loads: 0 direct, 1 the next sample's rows staged
// in shared memory with cp.async (StagedLoads; shared memory after the
// transfer function), kStageUnroll2 (batches) direct with the march loop
// written out two steps per trip.  LG > 1 (single view in cost order, 8x4 chunks, frame
// buffer only): work positions [0, LG * group_chunks) are the costliest
// group_chunks chunks, each as LG items of 32 / LG pixels rendered by lane
// groups of LG lanes per ray; the remaining positions are the other chunks of
// the cost order, rendered as usual.
template <int CW, int CH, int MINB, int STAGE, int LG = 1>
__global__ void __launch_bounds__(kRenderThreads, MINB) render_warps_kernel(BatchArgs b) {
  extern __shared__ float4 tf_s[];
  load_tf(tf_s, b.f.tf, b.f.n_tf);
  __syncthreads();
  using Loads = typename std::conditional<
      STAGE == 1, StagedLoads,
      typename std::conditional<STAGE == kStageUnroll2, UnrolledDirectLoads<2>, DirectLoads>::type>::type;
  Loads loads;
  if constexpr (STAGE == 1) loads.init(tf_s + (b.f.n_tf + 4));
  const int lane = threadIdx.x & 31;
  uint32_t n = 0;
  for (;;) {
    int chunk = 0;
    if (lane == 0) chunk = (int)atomicAdd(b.work_counter, 1u);
    chunk = __shfl_sync(0xffffffffu, chunk, 0);
    if (chunk >= b.total_tiles) break;
    int item = 0, first = 0;
    if (b.tile_prefix) {
      // item = last index with tile_prefix[item] <= chunk
      int lo = 0, hi = b.n_items - 1;
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(b.tile_prefix + mid) <= chunk)
          lo = mid;
        else
          hi = mid - 1;
      }
      item = lo;
      first = __ldg(b.tile_prefix + item);
    }
    const DevView v = b.f.views[b.view_ids ? __ldg(b.view_ids + item) : b.single_view];
    uint32_t* fb = b.fbs ? b.fbs[item] : b.f.fb;
    int ccx, ccy;
    const int cxn = (v.width + CW - 1) / CW;
    if constexpr (LG > 1) {
      if (chunk < b.group_chunks * LG) {
        const int id = __ldg(b.chunk_order + chunk / LG), part = chunk % LG;
        const int gl = lane % LG, p = part * (32 / LG) + lane / LG;
        const int x = (id % cxn) * 8 + (p & 7), y = (id / cxn) * 4 + (p >> 3);
        const LaneGroup g{gl, ((1u << LG) - 1u) << (lane - gl), lane - gl};
        // the group's lanes share x and y, so they take this branch together
        if (x < v.width && y < v.height) {
          const uint32_t ns =
              render_pixel<Loads, LG>(b.f, v, tf_s, x, y, fb, (size_t)x + (size_t)v.width * y, loads, g);
          if (gl == 0) n += ns;
        }
        continue;
      }
      chunk -= b.group_chunks * (LG - 1);  // position in the cost order of the remaining chunks
    }
    if (b.chunk_order) {
      const int id = __ldg(b.chunk_order + chunk);
      ccx = id % cxn;
      ccy = id / cxn;
    } else if (!ring_chunk(chunk - first, cxn, (v.height + CH - 1) / CH, ccx, ccy)) {
      continue;
    }
    const int x0 = ccx * CW, y0 = ccy * CH;
#pragma unroll 1
    for (int sub = 0; sub < (CW / 8) * (CH / 4); ++sub) {
      const int x = x0 + (sub % (CW / 8)) * 8 + (lane & 7);
      const int y = y0 + (sub / (CW / 8)) * 4 + (lane >> 3);
      if (x < v.width && y < v.height)
        n += render_pixel(b.f, v, tf_s, x, y, fb, (size_t)x + (size_t)v.width * y, loads);
    }
  }
  loads.finish();
  count_samples(b.f.counter, n);
}

// ---- Rank-split render of one view -------------------------------------
// A work item is one 8x4-pixel chunk for one virtual rank, so the bricks along
// a pixel's ray are marched by different warps at the same time.  The ranks
// of a pixel never interact before the composite (each has its own
// accumulator and early termination, like the reference's one process per
// rank), so this is render_pixel's arithmetic in another schedule.
//
// split_mask_kernel marks, per chunk slot, the ranks whose screen rectangle
// covers the chunk (bit k = k-th rank in visibility order); no pixel ray of
// an unmarked rank can enter its bricks, so its image is the output stage of
// an empty march.  The scan kernels and split_emit_kernel list the work items
// in position order (the cost order when s.chunk_order is set, else the
// centre-out ring): one per marked rank, or one compositing-only
// item for a chunk no rank covers.  render_split_kernel marches each item's rank into its
// image plane; the warp that completes a chunk's last marked rank (a ticket
// per chunk, taken after a fence) blends the chunk front to back, evaluating
// the unmarked ranks' images in place, and resets the ticket for the next
// launch.  No warp waits on another.

// Chunk of work position p: the p-th of the cost order when there is one,
// else ring slot p (false off the chunk grid).
__device__ __forceinline__ bool split_chunk(const SplitArgs& s, int p, int cxn, int cyn, int& cx, int& cy) {
  if (s.chunk_order) {
    const int id = __ldg(s.chunk_order + p);
    cx = id % cxn;
    cy = id / cxn;
    return true;
  }
  return ring_chunk(p, cxn, cyn, cx, cy);
}

__device__ __forceinline__ bool rect_covers(const int* __restrict__ q, int cx, int cy) {
  return cx >= __ldg(q) && cy >= __ldg(q + 1) && cx <= __ldg(q + 2) && cy <= __ldg(q + 3);
}

// Per slot: the mask of covering ranks and the number of items it lists
// (one per covering rank, one for a covered-by-none chunk, 0 off the grid).
__global__ void split_mask_kernel(SplitArgs s) {
  const DevView& v = s.f.views[s.view];
  const int W = v.width, H = v.height, R = v.n_ranks;
  const int* __restrict__ order = s.f.sched + v.sched;
  const int* __restrict__ rects = s.f.sched + v.rects;
  const int cxn = (W + 7) / 8, cyn = (H + 3) / 4;
  for (int slot = blockIdx.x * blockDim.x + threadIdx.x; slot < s.n_slots; slot += gridDim.x * blockDim.x) {
    int cx, cy;
    unsigned long long m = 0ull;
    uint32_t items = 0;
    if (split_chunk(s, slot, cxn, cyn, cx, cy)) {
      for (int k = 0; k < R; ++k)
        if (rect_covers(rects + 4 * __ldg(order + k), cx, cy)) m |= 1ull << k;
      items = m ? (uint32_t)__popcll(m) : 1u;
    }
    s.masks[slot] = m;
    s.offsets[slot] = items;
  }
}

// Exclusive scan of the per-slot item counts in place, and the item total,
// in two levels: per-block sums of kScanTile slots, a one-CTA scan of the
// block sums, then each block scans its tile and adds its base.
constexpr int kScanBlock = 256, kScanPer = 4, kScanTile = kScanBlock * kScanPer;

__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t* warp_sum, uint32_t& total) {
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5, nw = blockDim.x >> 5;
  uint32_t incl = v;
#pragma unroll
  for (int d = 1; d < 32; d <<= 1) {
    const uint32_t o = __shfl_up_sync(0xffffffffu, incl, d);
    if (lane >= d) incl += o;
  }
  if (lane == 31) warp_sum[wid] = incl;
  __syncthreads();
  if (wid == 0) {
    uint32_t w = lane < nw ? warp_sum[lane] : 0u;
#pragma unroll
    for (int d = 1; d < 32; d <<= 1) {
      const uint32_t o = __shfl_up_sync(0xffffffffu, w, d);
      if (lane >= d) w += o;
    }
    if (lane < nw) warp_sum[lane] = w;
  }
  __syncthreads();
  total = warp_sum[nw - 1];
  return incl - v + (wid > 0 ? warp_sum[wid - 1] : 0u);
}

__global__ void __launch_bounds__(kScanBlock) split_block_sums_kernel(SplitArgs s, uint32_t* sums) {
  __shared__ uint32_t warp_sum[kScanBlock / 32];
  const int base = blockIdx.x * kScanTile + threadIdx.x * kScanPer;
  uint32_t v = 0;
#pragma unroll
  for (int i = 0; i < kScanPer; ++i)
    if (base + i < s.n_slots) v += s.offsets[base + i];
  uint32_t total;
  block_exclusive_scan(v, warp_sum, total);
  if (threadIdx.x == 0) sums[blockIdx.x] = total;
}

// One CTA: exclusive scan of the block sums (contiguous ranges per thread).
__global__ void __launch_bounds__(1024) split_sums_scan_kernel(SplitArgs s, uint32_t* sums, int n) {
  __shared__ uint32_t warp_sum[1024 / 32];
  const int per = (n + 1023) / 1024;
  const int lo = min(n, (int)threadIdx.x * per), hi = min(n, lo + per);
  uint32_t v = 0;
  for (int i = lo; i < hi; ++i) v += sums[i];
  uint32_t total;
  uint32_t at = block_exclusive_scan(v, warp_sum, total);
  for (int i = lo; i < hi; ++i) {
    const uint32_t c = sums[i];
    sums[i] = at;
    at += c;
  }
  if (threadIdx.x == 0) *s.n_items = total;
}

__global__ void __launch_bounds__(kScanBlock) split_tile_scan_kernel(SplitArgs s, const uint32_t* sums) {
  __shared__ uint32_t warp_sum[kScanBlock / 32];
  const int base = blockIdx.x * kScanTile + threadIdx.x * kScanPer;
  uint32_t c[kScanPer], v = 0;
#pragma unroll
  for (int i = 0; i < kScanPer; ++i) {
    c[i] = base + i < s.n_slots ? s.offsets[base + i] : 0u;
    v += c[i];
  }
  uint32_t total;
  uint32_t at = block_exclusive_scan(v, warp_sum, total) + sums[blockIdx.x];
#pragma unroll
  for (int i = 0; i < kScanPer; ++i)
    if (base + i < s.n_slots) {
      s.offsets[base + i] = at;
      at += c[i];
    }
}

// Writes each slot's items at its offset: slot << 7 | rank position, or the
// compositing-only item of a chunk no rank covers.
__global__ void split_emit_kernel(SplitArgs s) {
  const DevView& v = s.f.views[s.view];
  const int cxn = (v.width + 7) / 8, cyn = (v.height + 3) / 4;
  for (int slot = blockIdx.x * blockDim.x + threadIdx.x; slot < s.n_slots; slot += gridDim.x * blockDim.x) {
    int cx, cy;
    if (!split_chunk(s, slot, cxn, cyn, cx, cy)) continue;
    uint32_t at = s.offsets[slot];
    unsigned long long m = s.masks[slot];
    const uint32_t base = (uint32_t)slot << 7;
    if (!m) {
      s.items[at] = base | kSplitBackground;
      continue;
    }
    while (m) {
      const int k = __ffsll((long long)m) - 1;
      m &= m - 1ull;
      s.items[at++] = base | (uint32_t)k;
    }
  }
}

template <int MINB>
__global__ void __launch_bounds__(kRenderThreads, MINB) render_split_kernel(SplitArgs s) {
  extern __shared__ float4 tf_s[];
  load_tf(tf_s, s.f.tf, s.f.n_tf);
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int W = s.f.views[s.view].width, H = s.f.views[s.view].height, R = s.f.views[s.view].n_ranks;
  const size_t npx = (size_t)W * H;
  const int* __restrict__ order = s.f.sched + s.f.views[s.view].sched;
  const int* __restrict__ rstart = order + R;
  const int* __restrict__ rbricks = rstart + R + 1;
  const int cxn = (W + 7) / 8, cyn = (H + 3) / 4;
  const uint32_t n_items = *s.n_items;
  float4* __restrict__ planes = s.f.rank_images;
  uint32_t n = 0;
  for (;;) {
    uint32_t item = 0;
    if (lane == 0) item = atomicAdd(s.work_counter, 1u);
    item = __shfl_sync(0xffffffffu, item, 0);
    if (item >= n_items) break;
    const uint32_t code = __ldg(s.items + item);
    const int slot = (int)(code >> 7), k = (int)(code & 127u);
    int cx, cy;
    split_chunk(s, slot, cxn, cyn, cx, cy);
    const int x = cx * 8 + (lane & 7), y = cy * 4 + (lane >> 3);
    const bool valid = x < W && y < H;
    const int pixel = x + W * y;
    const unsigned long long mask = __ldg(s.masks + slot);
    if (k != kSplitBackground) {
      if (valid) {
        const DevView v = s.f.views[s.view];
        const int r = __ldg(order + k);
        float z = 1.0f;
        uint32_t ns = 0;
        float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
        DirectLoads direct;
        const bool in_island = pixel_in_island(s.f, W, x, y);
        if (plain_output_stage(s.f)) {
          // the output stage is the identity: only the plane store is left,
          // so nothing else it needs stays live across the march
          if (in_island)
            acc = march_rank(s.f, v, tf_s, generate_ray(v, x, y), rbricks, __ldg(rstart + r), __ldg(rstart + r + 1),
                             pixel, z, ns, direct);
          planes[(size_t)r * npx + pixel] = acc;
        } else {
          if (in_island)
            acc = march_rank(s.f, v, tf_s, generate_ray(v, x, y), rbricks, __ldg(rstart + r), __ldg(rstart + r + 1),
                             pixel, z, ns, direct);
          rank_output(s.f, W, H, r, x, y, pixel, npx, acc, ns, z, planes, nullptr);
        }
        n += ns;
      }
      __threadfence();
      __syncwarp();
      unsigned ticket = 0;
      if (lane == 0) ticket = atomicAdd(s.chunk_done + slot, 1u);
      ticket = __shfl_sync(0xffffffffu, ticket, 0);
      if (ticket != (unsigned)(__popcll(mask) - 1)) continue;
      __threadfence();
    }
    if (valid) {
      OverBlend blend;
      for (int kk = 0; kk < R; ++kk) {
        const int r = __ldg(order + kk);
        const float4 img = (mask >> kk) & 1ull
                               ? __ldcg(planes + (size_t)r * npx + pixel)
                               : rank_output(s.f, W, H, r, x, y, pixel, npx, make_float4(0.f, 0.f, 0.f, 0.f), 0u,
                                             1.0f, nullptr, nullptr);
        blend.add(s.f.composite_mode, img);
      }
      s.f.fb[pixel] = blend.pack(s.f.composite_mode);
    }
    if (lane == 0 && k != kSplitBackground) s.chunk_done[slot] = 0u;
  }
  count_samples(s.f.counter, n);
}

// Ordered "over" of per-rank float images (IceT BLEND with ORDERED_COMPOSITE,
// waikikiRenderer.cpp:910-917,1042-1079), front to back.
__global__ void composite_f32_kernel(const float4* __restrict__ imgs, const int* __restrict__ order, int n_ranks,
                                     int npx, int mode, uint32_t* __restrict__ fb) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < npx; p += gridDim.x * blockDim.x) {
    OverBlend blend;
    for (int k = 0; k < n_ranks; ++k) blend.add(mode, __ldg(imgs + (size_t)__ldg(order + k) * npx + p));
    fb[p] = blend.pack(mode);
  }
}

// 8-bit ordered over of external RGBA8 rank images.
__global__ void composite_u8_kernel(const uint32_t* __restrict__ imgs, const int* __restrict__ order, int n_ranks,
                                    int npx, uint32_t* __restrict__ fb) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < npx; p += gridDim.x * blockDim.x) {
    uint32_t c8[4] = {0u, 0u, 0u, 0u};
    for (int k = 0; k < n_ranks; ++k) {
      const uint32_t q = __ldg(imgs + (size_t)__ldg(order + k) * npx + p);
      const uint32_t f = 255u - c8[3];
#pragma unroll
      for (int ch = 0; ch < 4; ++ch) c8[ch] = min(255u, c8[ch] + (((q >> (8 * ch)) & 255u) * f + 127u) / 255u);
    }
    fb[p] = c8[0] | (c8[1] << 8) | (c8[2] << 16) | (c8[3] << 24);
  }
}

// Copies a brick (x fastest) into its padded yz-quad array: element (x,y,z)
// holds V(x,y,z), V(x,y+1,z), V(x,y,z+1), V(x,y+1,z+1) with every index
// clamped to the brick (the apron and the quads' far rows and slices repeat
// edge values), and flags non-finite voxels.  CTAs take padded rows (y, z),
// their threads the row's elements, so the index arithmetic is one division
// per row; a row reads four source rows, each coalesced along x.
__global__ void pad_brick_kernel(const float* __restrict__ src, int nx, int ny, int nz, float4* __restrict__ dst,
                                 int px, int py, int pz, int* nonfinite) {
  const int rows = py * pz;
  bool bad = false;
  for (int r = blockIdx.x; r < rows; r += gridDim.x) {
    const int y = r % py, z = r / py;
    const int y0 = min(max(y - kApron, 0), ny - 1), y1 = min(max(y + 1 - kApron, 0), ny - 1);
    const int z0 = min(max(z - kApron, 0), nz - 1), z1 = min(max(z + 1 - kApron, 0), nz - 1);
    const float* __restrict__ r00 = src + ((size_t)z0 * ny + y0) * nx;
    const float* __restrict__ r10 = src + ((size_t)z0 * ny + y1) * nx;
    const float* __restrict__ r01 = src + ((size_t)z1 * ny + y0) * nx;
    const float* __restrict__ r11 = src + ((size_t)z1 * ny + y1) * nx;
    float4* __restrict__ out = dst + (size_t)r * px;
    for (int x = threadIdx.x; x < px; x += blockDim.x) {
      const int sx = min(max(x - kApron, 0), nx - 1);
      const float4 v = make_float4(__ldg(r00 + sx), __ldg(r10 + sx), __ldg(r01 + sx), __ldg(r11 + sx));
      bad |= !isfinite(v.x) || !isfinite(v.y) || !isfinite(v.z) || !isfinite(v.w);
      out[x] = v;
    }
  }
  if (bad) atomicOr(nonfinite, 1);
}

// Value range each macrocell's samples can read: a sample whose value-tap
// cell is c (c = clamp(floor(u), 0, n-1)) reads voxels c and c+1 (clamped), so
// macrocell m covers voxels [m*kMacro, m*kMacro + kMacro] per axis.  One warp
// per macrocell: its lanes split the macrocell's pairs of (y, z) rows, read
// each pair as yz-quads (four voxels per load, the components inside the
// range used), and combine their minima and maxima with shuffles.
__global__ void macrocell_range_kernel(const float4* __restrict__ base, int sy, int sz, int nx, int ny, int nz,
                                       int mnx, int mny, int mnz, float2* __restrict__ out) {
  const int total = mnx * mny * mnz;
  const int lane = threadIdx.x & 31;
  const int warps = (int)((gridDim.x * blockDim.x) >> 5);
  for (int i = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5); i < total; i += warps) {
    const int mx = i % mnx, my = (i / mnx) % mny, mz = i / (mnx * mny);
    const int x0 = mx * kMacro, y0 = my * kMacro, z0 = mz * kMacro;
    const int x1 = min(x0 + kMacro, nx - 1), y1 = min(y0 + kMacro, ny - 1), z1 = min(z0 + kMacro, nz - 1);
    const int pairs_y = (y1 - y0 + 2) >> 1, pairs = pairs_y * ((z1 - z0 + 2) >> 1);
    float lo = __int_as_float(0x7f800000), hi = -lo;
    for (int r = lane; r < pairs; r += 32) {
      const int y = y0 + 2 * (r % pairs_y), z = z0 + 2 * (r / pairs_y);
      const bool y_in = y + 1 <= y1, z_in = z + 1 <= z1;  // the quad's second row / slice inside the range
      const float4* row = base + (size_t)z * sz + (size_t)y * sy;
      for (int x = x0; x <= x1; ++x) {
        const float4 q = __ldg(row + x);
        lo = fminf(lo, q.x);
        hi = fmaxf(hi, q.x);
        if (y_in) {
          lo = fminf(lo, q.y);
          hi = fmaxf(hi, q.y);
        }
        if (z_in) {
          lo = fminf(lo, q.z);
          hi = fmaxf(hi, q.z);
        }
        if (y_in && z_in) {
          lo = fminf(lo, q.w);
          hi = fmaxf(hi, q.w);
        }
      }
    }
#pragma unroll
    for (int d = 16; d > 0; d >>= 1) {
      lo = fminf(lo, __shfl_xor_sync(0xffffffffu, lo, d));
      hi = fmaxf(hi, __shfl_xor_sync(0xffffffffu, hi, d));
    }
    if (lane == 0) out[i] = make_float2(lo, hi);
  }
}

// A macrocell is empty when every transfer-function entry its lookups can
// touch has alpha 0: indices floor(v*n - 1/2) and +1 for v in [lo, hi], with
// one index of margin on each side for rounding of the interpolated value.
// prefix[k] = number of entries below k with non-zero alpha.
__global__ void macrocell_empty_kernel(const float2* __restrict__ ranges, int count, const int* __restrict__ prefix,
                                       int n, uint8_t* __restrict__ empty) {
  const float nf = (float)n;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < count; i += gridDim.x * blockDim.x) {
    const float2 r = ranges[i];
    const float xl = fminf(fmaxf(r.x * nf - 0.5f, -8.0f), nf + 8.0f);
    const float xh = fminf(fmaxf(r.y * nf - 0.5f, -8.0f), nf + 8.0f);
    const int lo = max((int)floorf(xl) - 1, 0);
    const int hi = min((int)floorf(xh) + 2, n - 1);
    const int nonzero = lo <= hi ? __ldg(prefix + hi + 1) - __ldg(prefix + lo) : 0;
    empty[i] = nonzero == 0 ? 1 : 0;
  }
}

static size_t tf_smem(int n_tf) { return (size_t)(n_tf + 4) * sizeof(float4); }
static size_t render_smem(int n_tf, int stage) {
  return tf_smem(n_tf) + (stage == ALOHA_STAGING_NEXT_SAMPLE ? kStageBytes : 0);
}

cudaError_t launch_macrocell_range(const DevBrick& b, float2* out, cudaStream_t s) {
  const int mnx = (b.n[0] + kMacro - 1) >> kMacroShift, mny = (b.n[1] + kMacro - 1) >> kMacroShift,
            mnz = (b.n[2] + kMacro - 1) >> kMacroShift;
  const int total = mnx * mny * mnz;
  const int grid = min((total + 3) / 4, 152 * 32);  // 4 warps (macrocells) per CTA
  macrocell_range_kernel<<<grid, 128, 0, s>>>(b.base, b.sy, b.sz, b.n[0], b.n[1], b.n[2], mnx, mny, mnz, out);
  return cudaGetLastError();
}

cudaError_t launch_macrocell_empty(const float2* ranges, int count, const int* prefix, int n, uint8_t* empty,
                                   cudaStream_t s) {
  if (count <= 0) return cudaSuccess;
  const int grid = min((count + 255) / 256, 152 * 16);
  macrocell_empty_kernel<<<grid, 256, 0, s>>>(ranges, count, prefix, n, empty);
  return cudaGetLastError();
}

namespace {

// The kernel instance for a chunk shape, launch mode and staging, or null.
using RenderKernel = void (*)(BatchArgs);
template <int MINB, int STAGE>
RenderKernel render_kernel_for(int chunk_w, int chunk_h) {
  if (chunk_w == 8 && chunk_h == 4) return render_warps_kernel<8, 4, MINB, STAGE>;
  if (chunk_w == 8 && chunk_h == 8) return render_warps_kernel<8, 8, MINB, STAGE>;
  if (chunk_w == 16 && chunk_h == 8) return render_warps_kernel<16, 8, MINB, STAGE>;
  if (chunk_w == 32 && chunk_h == 4) return render_warps_kernel<32, 4, MINB, STAGE>;
  return nullptr;
}

RenderKernel render_kernel(int chunk_w, int chunk_h, bool batch, int stage, bool lane_groups) {
  if (lane_groups)
    return (!batch && stage == ALOHA_STAGING_NONE && chunk_w == 8 && chunk_h == 4)
               ? render_warps_kernel<8, 4, kSingleRenderBlocks, 0, kLaneGroup>
               : nullptr;
  if (stage == ALOHA_STAGING_NEXT_SAMPLE)
    return batch ? render_kernel_for<kBatchRenderBlocks, 1>(chunk_w, chunk_h)
                 : render_kernel_for<kSingleRenderBlocks, 1>(chunk_w, chunk_h);
  if (stage == kStageUnroll2) return batch ? render_kernel_for<kBatchRenderBlocks, kStageUnroll2>(chunk_w, chunk_h)
                                           : nullptr;
  if (stage != ALOHA_STAGING_NONE) return nullptr;
  return batch ? render_kernel_for<kBatchRenderBlocks, 0>(chunk_w, chunk_h)
               : render_kernel_for<kSingleRenderBlocks, 0>(chunk_w, chunk_h);
}

}  // namespace

cudaError_t launch_render_warps(const BatchArgs& b, int chunk_w, int chunk_h, int grid, bool batch, cudaStream_t s,
                                int stage, bool lane_groups) {
  if (lane_groups && (!b.chunk_order || b.f.rank_images || b.f.rank_depth || b.f.accum)) return cudaErrorInvalidValue;
  const RenderKernel k = render_kernel(chunk_w, chunk_h, batch, stage, lane_groups);
  if (!k) return cudaErrorInvalidValue;
  k<<<grid, kRenderThreads, render_smem(b.f.n_tf, stage), s>>>(b);
  return cudaGetLastError();
}

int render_blocks_per_sm(int chunk_w, int chunk_h, int n_tf, bool batch, int stage, bool lane_groups) {
  const RenderKernel k = render_kernel(chunk_w, chunk_h, batch, stage, lane_groups);
  int n = 0;
  if (!k || cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, kRenderThreads, render_smem(n_tf, stage)) !=
                cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

// Many ranks make short (chunk, rank) items, so the launch is throughput-bound
// and runs best with more resident warps (64 ranks of 1024^3 at 2048^2:
// 5.58 ms at 5 CTAs/SM, 5.26 ms at 7); with few ranks the longest items
// bound the frame and 5 CTAs/SM is best (8 ranks: 0.89 vs 0.96 ms).
using SplitKernel = void (*)(SplitArgs);
static SplitKernel split_kernel(bool many_ranks) {
  return many_ranks ? render_split_kernel<kManyRankSplitBlocks> : render_split_kernel<kSingleRenderBlocks>;
}

cudaError_t launch_render_split(const SplitArgs& a, int grid, bool many_ranks, cudaStream_t s) {
  int mg = (a.n_slots + 255) / 256;
  mg = mg < 1 ? 1 : (mg > 152 * 8 ? 152 * 8 : mg);
  split_mask_kernel<<<mg, 256, 0, s>>>(a);
  const int tiles = (a.n_slots + kScanTile - 1) / kScanTile;
  split_block_sums_kernel<<<tiles, kScanBlock, 0, s>>>(a, a.block_sums);
  split_sums_scan_kernel<<<1, 1024, 0, s>>>(a, a.block_sums, tiles);
  split_tile_scan_kernel<<<tiles, kScanBlock, 0, s>>>(a, a.block_sums);
  split_emit_kernel<<<mg, 256, 0, s>>>(a);
  cudaError_t e = cudaMemsetAsync(a.work_counter, 0, sizeof(unsigned int), s);
  if (e != cudaSuccess) return e;
  split_kernel(many_ranks)<<<grid, kRenderThreads, tf_smem(a.f.n_tf), s>>>(a);
  return cudaGetLastError();
}

int render_split_blocks_per_sm(int n_tf, bool many_ranks) {
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, split_kernel(many_ranks), kRenderThreads, tf_smem(n_tf)) !=
      cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

static int composite_grid(int npx) {
  int g = (npx + 255) / 256;
  return g < 1 ? 1 : (g > 152 * 16 ? 152 * 16 : g);
}

cudaError_t launch_composite_f32(const float4* imgs, const int* order, int n_ranks, int npx, int mode, uint32_t* fb,
                                 cudaStream_t s) {
  composite_f32_kernel<<<composite_grid(npx), 256, 0, s>>>(imgs, order, n_ranks, npx, mode, fb);
  return cudaGetLastError();
}

cudaError_t launch_composite_u8(const uint32_t* imgs, const int* order, int n_ranks, int npx, uint32_t* fb,
                                cudaStream_t s) {
  composite_u8_kernel<<<composite_grid(npx), 256, 0, s>>>(imgs, order, n_ranks, npx, fb);
  return cudaGetLastError();
}

cudaError_t launch_pad_brick(const float* src, int nx, int ny, int nz, float4* dst, int px, int py, int pz,
                             int* nonfinite, cudaStream_t s) {
  const int rows = py * pz;
  const int g = rows < 152 * 32 ? rows : 152 * 32;  // CTAs of 128 threads take rows
  pad_brick_kernel<<<g < 1 ? 1 : g, 128, 0, s>>>(src, nx, ny, nz, dst, px, py, pz, nonfinite);
  return cudaGetLastError();
}

}  // namespace aloha
