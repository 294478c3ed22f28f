// adjoint.cu -- differentiable form of the march (no reference counterpart).
//
// Forward (training): every pixel marches the single virtual rank's bricks
// front to back exactly as render_pixel does (same arithmetic, so the image
// is bit-identical to a render with one rank) and stores the march state
// every K samples: colour, t, the brick walk position, tmin, the jitter draw
// index and the samples already taken in the brick.  It also appends one work
// item per K-sample segment.
//
// Backward: one thread per segment.  With front-to-back compositing the
// colour adjoint g_rgb = dL/dC_rgb is the same for every sample, and the
// adjoint of alpha after sample i has the closed form
//     gA_{i+1} = (g_a (1 - a_N) - g_rgb . (rgb_N - rgb_{i+1})) / (1 - a_{i+1})
// (a_N, rgb_N: the final state).  So every segment is independent: a thread
// replays its K samples from the checkpoint and scatters
//     dL/dalpha_i = (1-a_i)(s_i g.c_i + gA_{i+1}),  dL/dc_i = g (1-a_i) alpha_i s_i,
//     dL/ds_i = (1-a_i) alpha_i g.c_i
// through the transfer-function lookup (shared-memory accumulation, one flush
// per CTA), the shading and the seven-tap stencil (20 voxel weights, atomic
// adds into the density gradient on the caller's grid).  Early termination is
// held fixed, as usual for a discontinuity.
#include <cuda_runtime.h>
#include <stdint.h>

#include "adjoint.h"
#include "march.cuh"

namespace aloha {

namespace {

struct Walk {
  int j;          // position in the rank's brick list
  float tmin;     // ray tmin at the start of this brick
  uint32_t draw;  // next jitter draw index
};

// Schedule of the single virtual rank: [rank_order 1][rank_start 2][bricks].
__device__ __forceinline__ const int* rank_bricks(const TrainArgs& a, const DevView& v) { return a.sched + v.sched + 3; }

// Samples of one pixel along the single rank's bricks, starting at walk
// state `w` (and, when `resume`, inside brick w.j at t_resume with nb0
// samples already taken there).  Calls `visit` before compositing each
// sample; stops after max_samples.  The walk, jitter draws and sample
// arithmetic are those of render_pixel / march_brick.
template <class Visit>
__device__ __forceinline__ uint32_t walk_samples(const TrainArgs& a, const DevView& v, const float4* tf_s,
                                                 const Ray& ray, uint32_t pixel, Walk w, float t_resume,
                                                 uint32_t nb0, bool resume, float4& color, uint32_t max_samples,
                                                 Visit visit) {
  const int* __restrict__ rb = rank_bricks(a, v);
  const int j1 = __ldg(a.sched + v.sched + 2);
  const float nf = (float)a.n_tf;
  uint32_t n = 0;
  for (; w.j < j1; ++w.j) {
    const DevBrick b = a.bricks[__ldg(rb + w.j)];
    float t0, t1;
    if (!slab(ray, b.space_lo, b.space_hi, w.tmin, 1e10f, t0, t1)) continue;
    float t;
    uint32_t nb = 0;
    if (resume) {
      t = t_resume;
      nb = nb0;
      resume = false;
    } else {
      const float ils = jitter(a.jitter_mode, a.jitter_value, pixel, (uint32_t)a.accum_id, w.draw++);
      t = first_sample_t(t0, a.dt, ils);
    }
    const uint32_t cap = march_cap(t0, t1, a.dt);
    for (; t < t1 && color.w < a.et_alpha && nb < cap; t = t + a.dt) {
      if (n == max_samples) return n;
      const float ux = fmaf(t, ray.d[0], ray.o[0]) - b.lo[0];
      const float uy = fmaf(t, ray.d[1], ray.o[1]) - b.lo[1];
      const float uz = fmaf(t, ray.d[2], ray.o[2]) - b.lo[2];
      const StencilOut s = stencil(b.base, b.sy, b.sz, b.n[0], b.n[1], b.n[2], ux, uy, uz);
      const float shade = shade_factor(s, ray);
      const float4 c = tf_lookup(tf_s, a.n_tf, nf, s.value);
      visit(b, t, w, nb, ux, uy, uz, s, shade, c, color);
      composite_step(color, c, shade);
      ++n;
      ++nb;
    }
    w.tmin = t1 + 1e-20f;
    if (!(color.w < a.et_alpha)) break;
  }
  return n;
}

template <int TW, int TH>
__global__ void __launch_bounds__(TW* TH) forward_train_kernel(TrainArgs a, int view) {
  extern __shared__ float4 tf_s[];
  load_tf(tf_s, a.tf, a.n_tf);
  __syncthreads();
  const DevView v = a.views[view];
  const int wi = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int x = blockIdx.x * TW + (wi % (TW / 8)) * 8 + (lane & 7);
  const int y = blockIdx.y * TH + (wi / (TW / 8)) * 4 + (lane >> 3);
  const bool active = x < v.width && y < v.height;
  uint32_t n = 0, nseg = 0;
  uint32_t pixel = 0;
  if (active) {
    pixel = (uint32_t)x + (uint32_t)v.width * (uint32_t)y;
    const Ray ray = generate_ray(v, x, y);
    float4 color = make_float4(0.f, 0.f, 0.f, 0.f);
    Checkpoint* ck = a.ckpt + (size_t)pixel * a.ckpt_cap;
    const uint32_t K = a.k, cap = a.ckpt_cap;
    uint32_t idx = 0;
    n = walk_samples(a, v, tf_s, ray, pixel, Walk{0, 0.0f, 0u}, 0.f, 0u, false, color, 0xffffffffu,
                     [&](const DevBrick&, float t, const Walk& w, uint32_t nb, float, float, float,
                         const StencilOut&, float, const float4&, const float4& col) {
                       if (idx % K == 0) {
                         const uint32_t m = idx / K;
                         if (m < cap) {
                           Checkpoint c;
                           c.r = col.x;
                           c.g = col.y;
                           c.b = col.z;
                           c.a = col.w;
                           c.t = t;
                           c.tmin = w.tmin;
                           c.jd = (uint32_t)w.j | (w.draw << 16);
                           c.nb = nb;
                           ck[m] = c;
                         } else {
                           atomicOr(a.overflow, 1);
                         }
                       }
                       ++idx;
                     });
    a.final_rgba[pixel] = color;
    if (a.out_rgba) a.out_rgba[pixel] = color;
    nseg = min((n + K - 1) / K, cap);
  }
  // warp-aggregated append of (pixel, segment) items, ordered by segment then
  // lane so that a backward warp replays neighbouring rays together
  const unsigned full = 0xffffffffu;
  const unsigned total = __reduce_add_sync(full, nseg);
  const unsigned maxseg = __reduce_max_sync(full, nseg);
  unsigned base = 0;
  if (lane == 0 && total) base = atomicAdd(a.work_count, total);
  base = __shfl_sync(full, base, 0);
  unsigned off = 0;
  for (unsigned m = 0; m < maxseg; ++m) {
    const unsigned mask = __ballot_sync(full, m < nseg);
    if (m < nseg) {
      const unsigned slot = base + off + __popc(mask & ((1u << lane) - 1u));
      if (slot < a.work_cap) a.work[slot] = make_uint2(pixel, m);
    }
    off += __popc(mask);
  }
  count_samples(a.counter, n);
}

__device__ __forceinline__ void red_add(float* p, float v) {
  if (v != 0.f) atomicAdd(p, v);
}

// Density-gradient scatter of one sample: the 20 voxels of the stencil with
// their combined weights (value tap and the six gradient taps).  Indices are
// clamped to the brick (the derivative of clamp addressing) and mapped to the
// caller's grid, so ghost and apron copies accumulate into the shared voxel.
__device__ __forceinline__ void stencil_backward(const DevBrick& b, const TrainArgs& a, int brick, float ux,
                                                 float uy, float uz, float dv, float dgx, float dgy, float dgz) {
  const float mx = ux - 0.5f, my = uy - 0.5f, mz = uz - 0.5f;
  const float fmx = floorf(mx), fmy = floorf(my), fmz = floorf(mz);
  const float fcx = floorf(ux), fcy = floorf(uy), fcz = floorf(uz);
  const float fx = mx - fmx, fy = my - fmy, fz = mz - fmz;
  const float gx = ux - fcx, gy = uy - fcy, gz = uz - fcz;
  const bool hx = fcx != fmx, hy = fcy != fmy, hz = fcz != fmz;
  const int ix = min(max((int)fmx, -kApron), b.n[0] - 1);
  const int iy = min(max((int)fmy, -kApron), b.n[1] - 1);
  const int iz = min(max((int)fmz, -kApron), b.n[2] - 1);
  const int cx = min(max((int)fcx, -kApron), b.n[0]);
  const int cy = min(max((int)fcy, -kApron), b.n[1]);
  const int cz = min(max((int)fcz, -kApron), b.n[2]);
  const int4 org = a.brick_grid_origin[brick];
  const size_t sx = (size_t)a.grid_dims[0], sxy = sx * (size_t)a.grid_dims[1];
  float* __restrict__ G = a.dgrid;
  auto at = [&](int x, int y, int z) -> float* {
    x = min(max(x, 0), b.n[0] - 1) + org.x;
    y = min(max(y, 0), b.n[1] - 1) + org.y;
    z = min(max(z, 0), b.n[2] - 1) + org.z;
    return G + ((size_t)z * sxy + (size_t)y * sx + (size_t)x);
  };
  const float wx[2] = {1.f - gx, gx}, wy[2] = {1.f - gy, gy}, wz[2] = {1.f - gz, gz};
  const float wxg[3] = {-(1.f - fx), (1.f - fx) - fx, fx};
  const float wyg[3] = {-(1.f - fy), (1.f - fy) - fy, fy};
  const float wzg[3] = {-(1.f - fz), (1.f - fz) - fz, fz};
  const float wv[3] = {hx ? 0.f : wx[0], hx ? wx[0] : wx[1], hx ? wx[1] : 0.f};
  const int myc = hy ? 1 : 0, mzc = hz ? 1 : 0;
#pragma unroll
  for (int l = 0; l < 2; ++l)
#pragma unroll
    for (int j = 0; j < 2; ++j) {
      const float wyz = wy[j] * wz[l];
      const float side = dgy * wyg[myc + j] * wz[l] + dgz * wzg[mzc + l] * wy[j];
#pragma unroll
      for (int k = 0; k < 3; ++k)
        red_add(at(ix + k, cy + j, cz + l), wyz * (dgx * wxg[k] + dv * wv[k]) + wv[k] * side);
    }
  const int ye = hy ? iy : iy + 2, ze = hz ? iz : iz + 2;
  const float wye = dgy * wyg[hy ? 0 : 2], wze = dgz * wzg[hz ? 0 : 2];
#pragma unroll
  for (int l = 0; l < 2; ++l)
#pragma unroll
    for (int i = 0; i < 2; ++i) red_add(at(cx + i, ye, cz + l), wye * wx[i] * wz[l]);
#pragma unroll
  for (int j = 0; j < 2; ++j)
#pragma unroll
    for (int i = 0; i < 2; ++i) red_add(at(cx + i, cy + j, ze), wze * wx[i] * wy[j]);
}

__global__ void __launch_bounds__(128) backward_kernel(TrainArgs a, int view) {
  extern __shared__ float4 smem[];
  float4* tf_s = smem;                                         // n_tf + 4 entries
  float* dtf_s = reinterpret_cast<float*>(smem + a.n_tf + 4);  // n_tf * 4
  load_tf(tf_s, a.tf, a.n_tf);
  for (int i = threadIdx.x; i < a.n_tf * 4; i += blockDim.x) dtf_s[i] = 0.f;
  __syncthreads();
  const DevView v = a.views[view];
  const int* __restrict__ rb = rank_bricks(a, v);
  const unsigned count = min(*a.work_count, a.work_cap);
  const float nf = (float)a.n_tf;
  uint32_t nsamp = 0;
  for (unsigned item = blockIdx.x * blockDim.x + threadIdx.x; item < count; item += gridDim.x * blockDim.x) {
    const uint2 wk = a.work[item];
    const uint32_t pixel = wk.x, m = wk.y;
    const int x = (int)(pixel % (uint32_t)v.width), y = (int)(pixel / (uint32_t)v.width);
    const Ray ray = generate_ray(v, x, y);
    const Checkpoint ck = a.ckpt[(size_t)pixel * a.ckpt_cap + m];
    const float4 F = a.final_rgba[pixel];
    const float4 g = a.dl_drgba[pixel];
    const float gfin = g.w * (1.0f - F.w);
    float4 color = make_float4(ck.r, ck.g, ck.b, ck.a);
    const Walk w0{(int)(ck.jd & 0xffffu), ck.tmin, ck.jd >> 16};
    nsamp += walk_samples(
        a, v, tf_s, ray, pixel, w0, ck.t, ck.nb, true, color, a.k,
        [&](const DevBrick& b, float, const Walk& wcur, uint32_t, float ux, float uy, float uz, const StencilOut& s,
            float shade, const float4& c, const float4& col) {
          float4 nxt = col;  // state after this sample
          composite_step(nxt, c, shade);
          const float tn = fmaxf(1.0f - nxt.w, 1e-6f);
          const float gA = (gfin - (g.x * (F.x - nxt.x) + g.y * (F.y - nxt.y) + g.z * (F.z - nxt.z))) / tn;
          const float oma = 1.0f - col.w;
          const float gc = g.x * c.x + g.y * c.y + g.z * c.z;
          const float kc = oma * c.w * shade;
          const float dch[4] = {g.x * kc, g.y * kc, g.z * kc, oma * (shade * gc + gA)};
          const float ds = oma * c.w * gc;
          // transfer function lookup backward
          const float xb = s.value * nf - 0.5f;
          const float fl = floorf(xb);
          const float wt = xb - fl;
          const int i0 = (int)fl;
          const int ic = min(max(i0, -2), a.n_tf);
          const float4 e0 = tf_s[ic + 2], e1 = tf_s[ic + 3];
          const float de[4] = {e1.x - e0.x, e1.y - e0.y, e1.z - e0.z, e1.w - e0.w};
          float dv = 0.f;
#pragma unroll
          for (int ch = 0; ch < 4; ++ch) {
            if (i0 >= 0 && i0 < a.n_tf) atomicAdd(dtf_s + i0 * 4 + ch, (1.f - wt) * dch[ch]);
            if (i0 + 1 >= 0 && i0 + 1 < a.n_tf) atomicAdd(dtf_s + (i0 + 1) * 4 + ch, wt * dch[ch]);
            dv += dch[ch] * de[ch] * nf;
          }
          // shading backward: s = .1 + .9 |q|, q = (g.d)/|g + 1e-4|
          const float ex = s.gx + 1e-4f, ey = s.gy + 1e-4f, ez = s.gz + 1e-4f;
          const float len2 = ex * ex + ey * ey + ez * ez;
          const float len = sqrtf(len2);
          const float gd = s.gx * ray.d[0] + s.gy * ray.d[1] + s.gz * ray.d[2];
          const float q = gd / len;
          const float kk = ds * 0.9f * (q > 0.f ? 1.f : (q < 0.f ? -1.f : 0.f));
          const float inv = 1.0f / len, c3 = gd / (len2 * len);
          stencil_backward(b, a, __ldg(rb + wcur.j), ux, uy, uz, dv, kk * (ray.d[0] * inv - c3 * ex),
                           kk * (ray.d[1] * inv - c3 * ey), kk * (ray.d[2] * inv - c3 * ez));
        });
  }
  count_samples(a.counter, nsamp);
  __syncthreads();
  for (int i = threadIdx.x; i < a.n_tf * 4; i += blockDim.x) red_add(a.dtf + i, dtf_s[i]);
}

size_t backward_smem(int n_tf) { return (size_t)(n_tf + 4) * sizeof(float4) + (size_t)n_tf * 4 * sizeof(float); }

}  // namespace

cudaError_t launch_forward_train(const TrainArgs& a, int view, int width, int height, cudaStream_t s) {
  constexpr int TW = 16, TH = 8;
  dim3 grid((width + TW - 1) / TW, (height + TH - 1) / TH);
  forward_train_kernel<TW, TH><<<grid, TW * TH, (size_t)(a.n_tf + 4) * sizeof(float4), s>>>(a, view);
  return cudaGetLastError();
}

cudaError_t launch_backward(const TrainArgs& a, int view, int grid, cudaStream_t s) {
  const size_t smem = backward_smem(a.n_tf);
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(backward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  backward_kernel<<<grid, 128, smem, s>>>(a, view);
  return cudaGetLastError();
}

int backward_blocks_per_sm(int n_tf) {
  const size_t smem = backward_smem(n_tf);
  if (smem > 48 * 1024 &&
      cudaFuncSetAttribute(backward_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, backward_kernel, 128, smem) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

}  // namespace aloha
