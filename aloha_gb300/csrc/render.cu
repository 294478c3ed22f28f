// render.cu -- forward kernels: fused per-view render, persistent batched
// render, ordered-over composite, brick padding.
#include <cuda_runtime.h>
#include <stdint.h>

#include "internal.h"
#include "march.cuh"

namespace aloha {

// Persistent render: every warp pulls CW x CH pixel chunks of the launch's
// items (views) from one atomic counter, centre-out per view, and renders
// each chunk as 8 x 4-pixel sub-tiles, so the 32 rays of a warp start within
// a few voxels of each other.  Warps are independent (no barrier after the
// transfer function is staged): a warp with long rays never holds finished
// warps of its CTA, and views end without a per-launch tail.  Nothing waits
// on other warps or CTAs.
// Six CTAs of 128 threads per SM (80 registers, no spills) keep 24 warps
// resident to hide the gather latency of the march.
template <int CW, int CH>
__global__ void __launch_bounds__(kRenderThreads, 6) render_warps_kernel(BatchArgs b) {
  extern __shared__ float4 tf_s[];
  load_tf(tf_s, b.f.tf, b.f.n_tf);
  __syncthreads();
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
    if (!ring_chunk(chunk - first, (v.width + CW - 1) / CW, (v.height + CH - 1) / CH, ccx, ccy)) continue;
    const int x0 = ccx * CW, y0 = ccy * CH;
#pragma unroll 1
    for (int sub = 0; sub < (CW / 8) * (CH / 4); ++sub) {
      const int x = x0 + (sub % (CW / 8)) * 8 + (lane & 7);
      const int y = y0 + (sub / (CW / 8)) * 4 + (lane >> 3);
      if (x < v.width && y < v.height) n += render_pixel(b.f, v, tf_s, x, y, fb, (size_t)x + (size_t)v.width * y);
    }
  }
  count_samples(b.f.counter, n);
}

// Ordered "over" of per-rank float images (IceT BLEND with ORDERED_COMPOSITE,
// waikikiRenderer.cpp:910-917,1042-1079), front to back.
__global__ void composite_f32_kernel(const float4* __restrict__ imgs, const int* __restrict__ order, int n_ranks,
                                     int npx, int mode, uint32_t* __restrict__ fb) {
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < npx; p += gridDim.x * blockDim.x) {
    float4 comp = make_float4(0.f, 0.f, 0.f, 0.f);
    uint32_t c8[4] = {0u, 0u, 0u, 0u};
    for (int k = 0; k < n_ranks; ++k) {
      const int r = __ldg(order + k);
      const float4 img = __ldg(imgs + (size_t)r * npx + p);
      if (mode == ALOHA_COMPOSITE_UBYTE) {
        const uint32_t q0 = quantize8(img.x), q1 = quantize8(img.y), q2 = quantize8(img.z), q3 = quantize8(img.w);
        const uint32_t f = 255u - c8[3];
        c8[0] = min(255u, c8[0] + (q0 * f + 127u) / 255u);
        c8[1] = min(255u, c8[1] + (q1 * f + 127u) / 255u);
        c8[2] = min(255u, c8[2] + (q2 * f + 127u) / 255u);
        c8[3] = min(255u, c8[3] + (q3 * f + 127u) / 255u);
      } else {
        const float oma = 1.0f - comp.w;
        comp.x = fmaf(oma, img.x, comp.x);
        comp.y = fmaf(oma, img.y, comp.y);
        comp.z = fmaf(oma, img.z, comp.z);
        comp.w = fmaf(oma, img.w, comp.w);
      }
    }
    fb[p] = (mode == ALOHA_COMPOSITE_UBYTE) ? (c8[0] | (c8[1] << 8) | (c8[2] << 16) | (c8[3] << 24))
                                            : pack_rgba(comp);
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

// Copies a brick (x fastest) into its padded x-quad array: element (x,y,z)
// holds V(x..x+3) with every index clamped to the brick (the apron and the
// quad tails repeat edge values), and flags non-finite voxels.
__global__ void pad_brick_kernel(const float* __restrict__ src, int nx, int ny, int nz, float4* __restrict__ dst,
                                 int px, int py, int pz, int* nonfinite) {
  const size_t total = (size_t)px * py * pz;
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += (size_t)gridDim.x * blockDim.x) {
    const int x = (int)(i % px);
    const int y = (int)((i / px) % py);
    const int z = (int)(i / ((size_t)px * py));
    const int sy = min(max(y - kApron, 0), ny - 1);
    const int sz = min(max(z - kApron, 0), nz - 1);
    const float* row = src + ((size_t)sz * ny + sy) * nx;
    float v[4];
#pragma unroll
    for (int k = 0; k < 4; ++k) v[k] = row[min(max(x - kApron + k, 0), nx - 1)];
    if (!isfinite(v[0]) || !isfinite(v[1]) || !isfinite(v[2]) || !isfinite(v[3])) atomicOr(nonfinite, 1);
    dst[i] = make_float4(v[0], v[1], v[2], v[3]);
  }
}

// Value range each macrocell's samples can read: a sample whose value-tap
// cell is c (c = clamp(floor(u), 0, n-1)) reads voxels c and c+1 (clamped), so
// macrocell m covers voxels [m*kMacro, m*kMacro + kMacro] per axis.
__global__ void macrocell_range_kernel(const float4* __restrict__ base, int sy, int sz, int nx, int ny, int nz,
                                       int mnx, int mny, int mnz, float2* __restrict__ out) {
  const int total = mnx * mny * mnz;
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < total; i += gridDim.x * blockDim.x) {
    const int mx = i % mnx, my = (i / mnx) % mny, mz = i / (mnx * mny);
    const int x0 = mx * kMacro, y0 = my * kMacro, z0 = mz * kMacro;
    const int x1 = min(x0 + kMacro, nx - 1), y1 = min(y0 + kMacro, ny - 1), z1 = min(z0 + kMacro, nz - 1);
    float lo = __int_as_float(0x7f800000), hi = -lo;
    for (int z = z0; z <= z1; ++z)
      for (int y = y0; y <= y1; ++y) {
        const float4* row = base + (size_t)z * sz + (size_t)y * sy;
        for (int x = x0; x <= x1; ++x) {
          const float v = __ldg(row + x).x;
          lo = fminf(lo, v);
          hi = fmaxf(hi, v);
        }
      }
    out[i] = make_float2(lo, hi);
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

cudaError_t launch_macrocell_range(const DevBrick& b, float2* out, cudaStream_t s) {
  const int mnx = (b.n[0] + kMacro - 1) >> kMacroShift, mny = (b.n[1] + kMacro - 1) >> kMacroShift,
            mnz = (b.n[2] + kMacro - 1) >> kMacroShift;
  const int total = mnx * mny * mnz;
  const int grid = total < 256 ? 1 : min((total + 127) / 128, 152 * 32);
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

cudaError_t launch_render_warps(const BatchArgs& b, int chunk_w, int chunk_h, int grid, cudaStream_t s) {
  const size_t smem = tf_smem(b.f.n_tf);
  if (chunk_w == 8 && chunk_h == 4)
    render_warps_kernel<8, 4><<<grid, kRenderThreads, smem, s>>>(b);
  else if (chunk_w == 8 && chunk_h == 8)
    render_warps_kernel<8, 8><<<grid, kRenderThreads, smem, s>>>(b);
  else if (chunk_w == 16 && chunk_h == 8)
    render_warps_kernel<16, 8><<<grid, kRenderThreads, smem, s>>>(b);
  else if (chunk_w == 32 && chunk_h == 4)
    render_warps_kernel<32, 4><<<grid, kRenderThreads, smem, s>>>(b);
  else
    return cudaErrorInvalidValue;
  return cudaGetLastError();
}

int render_blocks_per_sm(int chunk_w, int chunk_h, int n_tf) {
  int n = 0;
  const size_t smem = tf_smem(n_tf);
  cudaError_t e = cudaErrorInvalidValue;
  if (chunk_w == 8 && chunk_h == 4)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, render_warps_kernel<8, 4>, kRenderThreads, smem);
  else if (chunk_w == 8 && chunk_h == 8)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, render_warps_kernel<8, 8>, kRenderThreads, smem);
  else if (chunk_w == 16 && chunk_h == 8)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, render_warps_kernel<16, 8>, kRenderThreads, smem);
  else if (chunk_w == 32 && chunk_h == 4)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, render_warps_kernel<32, 4>, kRenderThreads, smem);
  if (e != cudaSuccess) {
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
  const size_t total = (size_t)px * py * pz;
  size_t g = (total + 255) / 256;
  if (g > 152 * 64) g = 152 * 64;
  if (g < 1) g = 1;
  pad_brick_kernel<<<(unsigned)g, 256, 0, s>>>(src, nx, ny, nz, dst, px, py, pz, nonfinite);
  return cudaGetLastError();
}

}  // namespace aloha
