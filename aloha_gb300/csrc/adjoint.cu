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
//
// One launch serves one view or many: the forward marches the chunks of all
// its views position-major (every view's first chunk, then every view's
// second, ...), and the backward replays the segments of all its views, each
// item finding its view in a prefix of the views' segment counts.  A launch
// of one view passes it in the kernel parameters instead (backward_kernel's
// MULTI = false), which keeps its pointers out of the replay's registers.
#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <climits>

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
//
// With SKIP, samples in empty macrocells (transfer-function alpha exactly 0,
// see march_brick) are counted and stepped over without a `visit` (in one
// jump when the steps are exact).  Only the density gradient may skip them: a
// zero-alpha sample still carries a gradient for the alpha entries.
//
// With CAN_STOP the walk also ends, before the next sample, once *stop is set
// (by the visitor).
template <bool SKIP, bool CAN_STOP = false, class Visit>
__device__ __forceinline__ uint32_t walk_samples(const TrainArgs& a, const DevView& v, const float4* tf_s,
                                                 const Ray& ray, uint32_t pixel, Walk w, float t_resume,
                                                 uint32_t nb0, bool resume, float4& color, uint32_t max_samples,
                                                 Visit visit, const bool* stop = nullptr) {
  const int* __restrict__ rb = rank_bricks(a, v);
  const int j1 = __ldg(a.sched + v.sched + 2);
  const float nf = (float)a.n_tf;
  const float dt = a.dt;
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
      t = first_sample_t(t0, dt, ils);
    }
    const uint32_t cap = march_cap(t0, t1, dt);
    const bool exact = SKIP && exact_steps(t, t1, dt);
    const int mnx = (b.n[0] + kMacro - 1) >> kMacroShift, mny = (b.n[1] + kMacro - 1) >> kMacroShift;
    const float mag = fmaxf(fmaxf(fabsf(ray.o[0]) + fabsf(b.lo[0]), fabsf(ray.o[1]) + fabsf(b.lo[1])),
                            fabsf(ray.o[2]) + fabsf(b.lo[2])) + fabsf(t1);
    const float eps = 2e-6f * mag + 1e-4f;
    float inv_d[3];  // 1 / direction, once per brick (the lookups below reuse it)
    float inv_dt = 0.0f;
    if (SKIP) {
#pragma unroll
      for (int ax = 0; ax < 3; ++ax) inv_d[ax] = 1.0f / ray.d[ax];
      inv_dt = 1.0f / dt;
    }
    float t_cell = t0;  // samples before it lie in a macrocell found non-empty
    while (t < t1 && color.w < a.et_alpha && nb < cap) {
      if (n == max_samples) return n;
      if (CAN_STOP && *stop) return n;
      const float ux = fmaf(t, ray.d[0], ray.o[0]) - b.lo[0];
      const float uy = fmaf(t, ray.d[1], ray.o[1]) - b.lo[1];
      const float uz = fmaf(t, ray.d[2], ray.o[2]) - b.lo[2];
      if (SKIP && b.empty && !(t < t_cell)) {
        const int mx = min(max(__float2int_rd(ux), 0), b.n[0] - 1) >> kMacroShift;
        const int my = min(max(__float2int_rd(uy), 0), b.n[1] - 1) >> kMacroShift;
        const int mz = min(max(__float2int_rd(uz), 0), b.n[2] - 1) >> kMacroShift;
        const float bnd[3] = {(float)(mx << kMacroShift), (float)(my << kMacroShift), (float)(mz << kMacroShift)};
        float tb = t1;
#pragma unroll
        for (int ax = 0; ax < 3; ++ax) {
          const float face = ray.d[ax] > 0.f ? bnd[ax] + (float)kMacro - eps : bnd[ax] + eps;
          tb = fminf(tb, (face - (ray.o[ax] - b.lo[ax])) * inv_d[ax]);
        }
        if (!__ldg(b.empty + (mz * mny + my) * mnx + mx)) {
          t_cell = tb;
        } else if (exact) {
          ++n;
          ++nb;
          t = t + dt;
          n += run_steps(t, nb, tb, cap, dt, inv_dt, max_samples - n);
          continue;
        } else {
          do {
            ++n;
            ++nb;
            t = t + dt;
          } while (t < tb && nb < cap && n != max_samples);
          continue;
        }
      }
      const StencilOut s = stencil<true>(b.base, b.sy, b.sz, b.n[0], b.n[1], b.n[2], ux, uy, uz);
      const float shade = shade_factor(s, ray);
      const float4 c = tf_lookup(tf_s, a.n_tf, nf, s.value);
      visit(b, t, w, nb, ux, uy, uz, s, shade, c, color);
      composite_step(color, c, shade);
      ++n;
      ++nb;
      t = t + dt;
    }
    w.tmin = t1 + 1e-20f;
    if (!(color.w < a.et_alpha)) break;
  }
  return n;
}

// Stores the march state before every K-th sample (evaluated or skipped):
// colour, t, the brick walk position, tmin, the jitter draw index and the
// samples already taken in the brick.  The brick loop sets j, tmin, draw.
struct CheckpointHook {
  static constexpr bool kActive = true;
  Checkpoint* ck;
  uint32_t K, cap;
  int* overflow;
  uint32_t left = 0, m = 0;  // samples to the next checkpoint, checkpoints so far
  int j = 0;
  float tmin = 0.0f;
  uint32_t draw = 0;
  __device__ __forceinline__ void operator()(float t, uint32_t nb, const float4& col) {
    if (left == 0) {
      left = K;
      if (m < cap) {
        Checkpoint c;
        c.r = col.x;
        c.g = col.y;
        c.b = col.z;
        c.a = col.w;
        c.t = t;
        c.tmin = tmin;
        c.jd = (uint32_t)j | (draw << 16);
        c.nb = nb;
        ck[m] = c;
      } else {
        atomicOr(overflow, 1);
      }
      ++m;
    }
    --left;
  }
};

// Training forward of one warp's 8 x 4 pixels at (x, y): the single rank's
// march (march_rank's brick walk with one draw, through march_brick, so the
// colour is the render's bit for bit), checkpoints, final colour, and the
// warp-aggregated append of (pixel, segment) items.  Returns the lane's
// sample count.
__device__ __forceinline__ uint32_t train_subtile(const TrainArgs& a, const TrainView& tv, const DevView& v,
                                                  const float4* tf_s, int x, int y, int lane) {
  const bool active = x < v.width && y < v.height;
  uint32_t n = 0, nseg = 0;
  uint32_t pixel = 0;
  if (active) {
    pixel = (uint32_t)x + (uint32_t)v.width * (uint32_t)y;
    const Ray ray = generate_ray(v, x, y);
    float4 color = make_float4(0.f, 0.f, 0.f, 0.f);
    CheckpointHook hook{tv.ckpt + (size_t)pixel * tv.ckpt_cap, a.k, tv.ckpt_cap, tv.overflow};
    const int* __restrict__ rb = rank_bricks(a, v);
    const int j1 = __ldg(a.sched + v.sched + 2);
    for (int j = 0; j < j1; ++j) {
      const DevBrick b = a.bricks[__ldg(rb + j)];
      float t0, t1;
      if (!slab(ray, b.space_lo, b.space_hi, hook.tmin, 1e10f, t0, t1)) continue;
      const float ils = jitter(a.jitter_mode, a.jitter_value, pixel, (uint32_t)a.accum_id, hook.draw++);
      hook.j = j;
      n += march_brick(b, tf_s, a.n_tf, ray, t0, t1, ils, a.dt, a.et_alpha, color, hook);
      hook.tmin = t1 + 1e-20f;
      if (!(color.w < a.et_alpha)) break;
    }
    tv.final_rgba[pixel] = color;
    if (tv.out_rgba) tv.out_rgba[pixel] = color;
    nseg = min((n + a.k - 1) / a.k, tv.ckpt_cap);
  }
  // warp-aggregated append of (pixel, segment) items, ordered by segment then
  // lane so that a backward warp replays neighbouring rays together
  const unsigned full = 0xffffffffu;
  const unsigned total = __reduce_add_sync(full, nseg);
  const unsigned maxseg = __reduce_max_sync(full, nseg);
  unsigned base = 0;
  if (lane == 0 && total) base = atomicAdd(tv.work_count, total);
  base = __shfl_sync(full, base, 0);
  unsigned off = 0;
  for (unsigned m = 0; m < maxseg; ++m) {
    const unsigned mask = __ballot_sync(full, m < nseg);
    if (m < nseg) {
      const unsigned slot = base + off + __popc(mask & ((1u << lane) - 1u));
      if (slot < tv.work_cap) tv.work[slot] = make_uint2(pixel, m);
    }
    off += __popc(mask);
  }
  return n;
}

// Item `item` of a forward launch -> (view slot, chunk position): the run
// holding it (binary search over the few runs), then position-major within
// the run.
__device__ __forceinline__ void forward_item(const TrainArgs& a, unsigned item, int& slot, int& pos) {
  int lo = 0, hi = a.n_runs - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (__ldg(&a.runs[mid].item0) <= item)
      lo = mid;
    else
      hi = mid - 1;
  }
  const int p0 = __ldg(&a.runs[lo].p0), active = __ldg(&a.runs[lo].active);
  const unsigned off = item - __ldg(&a.runs[lo].item0);
  pos = p0 + (int)(off / (unsigned)active);
  slot = __ldg(a.run_views + off % (unsigned)active);
}

// Persistent training forward over the launch's views: warps pull items
// (a view's 8 x 4 chunk, in its cost order when it has one, else
// centre-out, as the render does) from the launch's counter.
template <int MINB>
__global__ void __launch_bounds__(128, MINB) forward_train_kernel(TrainArgs a, unsigned items) {
  extern __shared__ float4 tf_s[];
  load_tf(tf_s, a.tf, a.n_tf);
  __syncthreads();
  const int lane = threadIdx.x & 31;
  uint32_t n = 0;
  for (;;) {
    unsigned item = 0;
    if (lane == 0) item = atomicAdd(a.grab, 1u);
    item = __shfl_sync(0xffffffffu, item, 0);
    if (item >= items) break;
    int slot, pos;
    forward_item(a, item, slot, pos);
    const TrainView& tv = a.tv[slot];
    const DevView v = a.views[tv.view];
    const int cxn = (v.width + 7) / 8, cyn = (v.height + 3) / 4;
    int ccx, ccy;
    if (tv.chunk_order) {
      const int id = __ldg(tv.chunk_order + pos);
      ccx = id % cxn;
      ccy = id / cxn;
    } else if (!ring_chunk(pos, cxn, cyn, ccx, ccy)) {
      continue;
    }
    n += train_subtile(a, tv, v, tf_s, ccx * 8 + (lane & 7), ccy * 4 + (lane >> 3), lane);
  }
  count_samples(a.counter, n);
}

__device__ __forceinline__ void red_add(float* p, float v) {
  if (v != 0.f) atomicAdd(p, v);
}

// Adds weights of brick voxels (x..x+2, y, z) (y, z already clamped to the
// brick) into the quad gradient: one float4 atomic when the three voxels are
// inside the brick, else one scalar atomic per clamped voxel.
__device__ __forceinline__ void scatter3(const TrainArgs& a, const DevBrick& b, const int4 org, int x, int y, int z,
                                         float w0, float w1, float w2) {
  if (w0 == 0.f && w1 == 0.f && w2 == 0.f) return;
  float4* row = a.dgrid4 + ((size_t)(z + org.z) * a.grid_dims[1] + (size_t)(y + org.y)) * a.grid_dims[0] + org.x;
  if (x >= 0 && x + 2 < b.n[0]) {
    atomicAdd(row + x, make_float4(w0, w1, w2, 0.f));
  } else {
    const int hi = b.n[0] - 1;
    red_add(&row[min(max(x, 0), hi)].x, w0);
    red_add(&row[min(max(x + 1, 0), hi)].x, w1);
    red_add(&row[min(max(x + 2, 0), hi)].x, w2);
  }
}

// The same for voxels (x, x+1): one float2 atomic on the quad's first half.
__device__ __forceinline__ void scatter2(const TrainArgs& a, const DevBrick& b, const int4 org, int x, int y, int z,
                                         float w0, float w1) {
  if (w0 == 0.f && w1 == 0.f) return;
  float4* row = a.dgrid4 + ((size_t)(z + org.z) * a.grid_dims[1] + (size_t)(y + org.y)) * a.grid_dims[0] + org.x;
  if (x >= 0 && x + 1 < b.n[0]) {
    atomicAdd(reinterpret_cast<float2*>(row + x), make_float2(w0, w1));
  } else {
    const int hi = b.n[0] - 1;
    red_add(&row[min(max(x, 0), hi)].x, w0);
    red_add(&row[min(max(x + 1, 0), hi)].x, w1);
  }
}

// Density-gradient scatter of one sample: the 20 voxels of the stencil with
// their combined weights (value tap and the six gradient taps), as 4 row
// quads and 4 row pairs.  Indices are clamped to the brick (the derivative of
// clamp addressing) and mapped to the caller's grid, so ghost and apron copies
// accumulate into the voxel they copy.
__device__ __forceinline__ void stencil_backward(const DevBrick& b, const TrainArgs& a, int brick, float ux,
                                                 float uy, float uz, float dv, float dgx, float dgy, float dgz) {
  // the forward stencil's coordinates (same indices and weights)
  const AxisCoord X = axis_coord(ux, b.n[0]), Y = axis_coord(uy, b.n[1]), Z = axis_coord(uz, b.n[2]);
  const float fx = X.f, fy = Y.f, fz = Z.f, gx = X.g, gy = Y.g, gz = Z.g;
  const bool hx = X.h, hy = Y.h, hz = Z.h;
  const int ix = X.i, iy = Y.i, iz = Z.i, cx = X.c, cy = Y.c, cz = Z.c;
  const int4 org = a.brick_grid_origin[brick];
  const int ny1 = b.n[1] - 1, nz1 = b.n[2] - 1;
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
      const float side = fmaf(dgy * wyg[myc + j], wz[l], dgz * wzg[mzc + l] * wy[j]);
      float w[3];
#pragma unroll
      for (int k = 0; k < 3; ++k) w[k] = fmaf(wyz, fmaf(dgx, wxg[k], dv * wv[k]), wv[k] * side);
      scatter3(a, b, org, ix, min(max(cy + j, 0), ny1), min(max(cz + l, 0), nz1), w[0], w[1], w[2]);
    }
  const int ye = min(max(hy ? iy : iy + 2, 0), ny1), ze = min(max(hz ? iz : iz + 2, 0), nz1);
  const float wye = dgy * wyg[hy ? 0 : 2], wze = dgz * wzg[hz ? 0 : 2];
#pragma unroll
  for (int l = 0; l < 2; ++l)
    scatter2(a, b, org, cx, ye, min(max(cz + l, 0), nz1), wye * wx[0] * wz[l], wye * wx[1] * wz[l]);
#pragma unroll
  for (int j = 0; j < 2; ++j)
    scatter2(a, b, org, cx, min(max(cy + j, 0), ny1), ze, wze * wx[0] * wy[j], wze * wx[1] * wy[j]);
}

// out[v] += q[v].x + q[v-1].y + q[v-2].z along x (each voxel written by one
// thread), leaving every quad it read zero again: a quad is rewritten only if
// it was nonzero, so a backward that touched part of the grid pays for that
// part only, and the next backward finds the buffer clear without a memset.
// CTAs take grid rows (y, z) and walk each in chunks of blockDim.x quads
// staged in shared memory behind the previous chunk's last two, so no quad
// is cleared before its three readers have it.
__global__ void fold_quads_kernel(float4* __restrict__ q, float* __restrict__ out, int dx, int rows) {
  extern __shared__ float4 sq[];  // [2 + blockDim.x]: q[x0-2], q[x0-1], then the chunk
  const int bd = (int)blockDim.x, i = (int)threadIdx.x;
  const float4 zero = make_float4(0.f, 0.f, 0.f, 0.f);
  for (int r = blockIdx.x; r < rows; r += gridDim.x) {
    float4* __restrict__ qr = q + (size_t)r * dx;
    float* __restrict__ orow = out + (size_t)r * dx;
    if (i < 2) sq[i] = zero;
    for (int x0 = 0; x0 < dx; x0 += bd) {
      const int x = x0 + i;
      const float4 v = x < dx ? qr[x] : zero;
      sq[2 + i] = v;
      __syncthreads();
      if (x < dx) {
        float s = v.x;
        if (x >= 1) s += sq[1 + i].y;
        if (x >= 2) s += sq[i].z;
        if (s != 0.f) orow[x] += s;
        if (v.x != 0.f || v.y != 0.f || v.z != 0.f || v.w != 0.f) qr[x] = zero;
      }
      __syncthreads();
      if (i < 2) sq[i] = sq[bd + i];
      __syncthreads();
    }
  }
}

// Adds a pending transfer-function gradient (entries i and i+1, four
// channels each) to the CTA's shared copy and clears it.
__device__ __forceinline__ void flush_tf(float* dtf_s, int n, int i, float pend[8]) {
#pragma unroll
  for (int k = 0; k < 2; ++k) {
    const int e = i + k;
    if (e >= 0 && e < n) {
#pragma unroll
      for (int ch = 0; ch < 4; ++ch)
        if (pend[4 * k + ch] != 0.f) atomicAdd(dtf_s + e * 4 + ch, pend[4 * k + ch]);
    }
  }
#pragma unroll
  for (int k = 0; k < 8; ++k) pend[k] = 0.f;
}

// Near-opaque samples.  The closed form for the adjoint of the accumulated
// alpha after sample i,
//     gA = (g_a (1 - a_N) - g_rgb . (rgb_N - rgb_{i+1})) / (1 - a_{i+1}),
// divides two vanishing quantities once a sample leaves almost no
// transmittance, and gives 0 for a sample of alpha exactly 1 (1 - a = 0),
// where the true value is g_a R_a - g_rgb . R_rgb with R the composite of the
// rest of the ray normalised to the transmittance after the sample:
//     R_a = prod_j (1 - alpha_j),  R_rgb = sum_j prod_{l<j} (1 - alpha_l) alpha_j s_j c_j.
// The replay records such a sample as an event (the closed form stands in
// for it meanwhile); after the segment, suffix_composite marches on from the
// sample after it and the event's alpha adjoint is corrected by the
// difference.  A ray has at most three events: each one cuts the
// transmittance by more than 256 from above kVisible.
constexpr float kOpaqueStep = 1.0f / 256.0f;  // alpha above 1 - 1/256
constexpr float kVisible = 1e-5f;             // ... and the sample not hidden already
constexpr int kMaxEvents = 3;

struct OpaqueEvent {
  Walk w;          // walk position of the sample (next jitter draw)
  float t_next;    // t and brick sample count of the sample after it
  uint32_t nb_next;
  float4 after;    // colour after the sample
  float oma;       // transmittance before it
  float gA;        // the closed form's value
  float value;     // interpolated value (transfer-function lookup)
  float ux, uy, uz;
  int brick;
};

// R after an event: the forward's following samples replayed from
// (w, t_next, nb_next) with the colour after the event (so that early
// termination ends the ray where the forward ended it), until R's
// transmittance is below 2^-24 (the rest cannot move the result) or the ray
// ends.  Skipped samples (alpha 0) leave R unchanged, so empty space is
// stepped over.  Returns (R_rgb, R_a).
__device__ __forceinline__ float4 suffix_composite(const TrainArgs& a, const DevView& v, const float4* tf_s,
                                                   const Ray& ray, uint32_t pixel, const OpaqueEvent& e) {
  float r0 = 0.f, r1 = 0.f, r2 = 0.f, tp = 1.0f;
  bool stop = false;
  float4 col = e.after;
  walk_samples<true, true>(
      a, v, tf_s, ray, pixel, e.w, e.t_next, e.nb_next, true, col, 0xffffffffu,
      [&](const DevBrick&, float, const Walk&, uint32_t, float, float, float, const StencilOut&, float shade,
          const float4& c, const float4&) {
        const float k = tp * c.w * shade;
        r0 = fmaf(k, c.x, r0);
        r1 = fmaf(k, c.y, r1);
        r2 = fmaf(k, c.z, r2);
        tp = tp * (1.0f - c.w);
        if (tp < 5.96e-8f) stop = true;
      },
      &stop);
  return make_float4(r0, r1, r2, tp);
}

constexpr unsigned kBackwardGrab = 256;  // most items a backward warp takes per grab (8 rows of 32)

// One backward item: the replay of segment (pixel, ck) of view v and its
// adjoint, added to dtf_s (shared, WITH_TF) and the x-quad density gradient
// (WITH_DENSITY).  Returns the samples replayed.
template <bool WITH_TF, bool WITH_DENSITY>
__device__ __forceinline__ uint32_t backward_item(const TrainArgs& a, const DevView& v, const int* __restrict__ rb,
                                                  const float4* tf_s, float* dtf_s, float nf, uint32_t pixel,
                                                  const Checkpoint& ck, const float4 F, const float4 g) {
  const int x = (int)(pixel % (uint32_t)v.width), y = (int)(pixel / (uint32_t)v.width);
  const Ray ray = generate_ray(v, x, y);
  const float gfin = g.w * (1.0f - F.w);
  float4 color = make_float4(ck.r, ck.g, ck.b, ck.a);
  const Walk w0{(int)(ck.jd & 0xffffu), ck.tmin, ck.jd >> 16};
  // transfer-function gradient of consecutive samples with the same lookup
  // index is summed in registers and added to shared memory once per index
  int pend_i = INT_MIN;
  float pend[8] = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
  OpaqueEvent events[kMaxEvents];
  int n_events = 0;
  const uint32_t n = walk_samples<!WITH_TF>(
      a, v, tf_s, ray, pixel, w0, ck.t, ck.nb, true, color, a.k,
      [&](const DevBrick& b, float t, const Walk& wcur, uint32_t nb, float ux, float uy, float uz,
          const StencilOut& s, float shade, const float4& c, const float4& col) {
        // Backward-only arithmetic below is free to contract and to use
        // approximate reciprocals (the gradient tolerance is relative); the
        // replay that feeds it is the exact forward.
        float4 nxt = col;  // state after this sample
        composite_step(nxt, c, shade);
        const float oma = 1.0f - col.w;
        const float tn1 = 1.0f - nxt.w;
        // dL/d(accumulated alpha after this sample), closed form
        const float gA =
            __fdividef(gfin - fmaf(g.x, F.x - nxt.x, fmaf(g.y, F.y - nxt.y, g.z * (F.z - nxt.z))),
                       fmaxf(tn1, 1e-6f));
        if (tn1 < kOpaqueStep * oma && oma > kVisible && n_events < kMaxEvents) {
          OpaqueEvent& e = events[n_events++];
          e.w = wcur;
          e.t_next = t + a.dt;
          e.nb_next = nb + 1;
          e.after = nxt;
          e.oma = oma;
          e.gA = gA;
          e.value = s.value;
          e.ux = ux;
          e.uy = uy;
          e.uz = uz;
          e.brick = __ldg(rb + wcur.j);
        }
        const float gc = fmaf(g.x, c.x, fmaf(g.y, c.y, g.z * c.z));
        const float dA = oma * fmaf(shade, gc, gA);  // dL/d(alpha of this sample)
        // transfer function lookup backward (the lookup of tf_lookup)
        const float xb = s.value * nf - 0.5f;
        const int i0 = __float2int_rd(xb);
        const float wt = xb - (float)i0;
        const int ic = min(max(i0, -2), a.n_tf);
        const float4 e0 = tf_s[ic + 2], e1 = tf_s[ic + 3];
        if (WITH_TF && i0 != pend_i) {
          flush_tf(dtf_s, a.n_tf, pend_i, pend);
          pend_i = i0;
        }
        if (e0.w == 0.f && e1.w == 0.f) {
          // Alpha is exactly 0 at this sample: only the two alpha entries of
          // the lookup receive gradient; the colour entries, the shading and
          // the density gradients all carry a factor alpha or d(alpha)/dv = 0.
          if (WITH_TF) {
            pend[3] = fmaf(1.f - wt, dA, pend[3]);
            pend[7] = fmaf(wt, dA, pend[7]);
          }
          return;
        }
        const float kc = oma * c.w * shade;
        const float dch[4] = {g.x * kc, g.y * kc, g.z * kc, dA};
        if (WITH_TF) {
  #pragma unroll
          for (int ch = 0; ch < 4; ++ch) {
            pend[ch] = fmaf(1.f - wt, dch[ch], pend[ch]);
            pend[4 + ch] = fmaf(wt, dch[ch], pend[4 + ch]);
          }
        }
        if (!WITH_DENSITY) return;
        const float ds = oma * c.w * gc;
        const float de[4] = {e1.x - e0.x, e1.y - e0.y, e1.z - e0.z, e1.w - e0.w};
        float dv = 0.f;
  #pragma unroll
        for (int ch = 0; ch < 4; ++ch) dv = fmaf(dch[ch], de[ch], dv);
        dv *= nf;
        // shading backward: s = .1 + .9 |q|, q = (g.d)/|g + 1e-4|
        const float ex = s.gx + 1e-4f, ey = s.gy + 1e-4f, ez = s.gz + 1e-4f;
        const float len2 = fmaf(ex, ex, fmaf(ey, ey, ez * ez));
        const float inv = rsqrtf(len2);
        const float gd = fmaf(s.gx, ray.d[0], fmaf(s.gy, ray.d[1], s.gz * ray.d[2]));
        const float kk = ds * 0.9f * (gd > 0.f ? 1.f : (gd < 0.f ? -1.f : 0.f));
        const float c3 = gd * inv * inv * inv;
        const float ki = kk * inv, kc3 = kk * c3;
        stencil_backward(b, a, __ldg(rb + wcur.j), ux, uy, uz, dv, fmaf(ki, ray.d[0], -kc3 * ex),
                         fmaf(ki, ray.d[1], -kc3 * ey), fmaf(ki, ray.d[2], -kc3 * ez));
      });
  if (WITH_TF) flush_tf(dtf_s, a.n_tf, pend_i, pend);
  // near-opaque samples: correct the alpha adjoint by the true one
  for (int k = 0; k < n_events; ++k) {
    const OpaqueEvent& e = events[k];
    const float4 R = suffix_composite(a, v, tf_s, ray, pixel, e);
    const float gtrue = fmaf(g.w, R.w, -fmaf(g.x, R.x, fmaf(g.y, R.y, g.z * R.z)));
    const float dd = e.oma * (gtrue - e.gA);  // change of dL/d(alpha of the sample)
    if (dd == 0.f) continue;
    const float xb = e.value * nf - 0.5f;
    const int i0 = __float2int_rd(xb);
    const float wt = xb - (float)i0;
    if (WITH_TF) {
      if (i0 >= 0 && i0 < a.n_tf) atomicAdd(dtf_s + i0 * 4 + 3, (1.f - wt) * dd);
      if (i0 + 1 >= 0 && i0 + 1 < a.n_tf) atomicAdd(dtf_s + (i0 + 1) * 4 + 3, wt * dd);
    }
    if (WITH_DENSITY) {
      const int ic = min(max(i0, -2), a.n_tf);
      const float dv = nf * dd * (tf_s[ic + 3].w - tf_s[ic + 2].w);
      if (dv != 0.f) {
        const DevBrick b = a.bricks[e.brick];
        stencil_backward(b, a, e.brick, e.ux, e.uy, e.uz, dv, 0.f, 0.f, 0.f);
      }
    }
  }
  return n;
}

// WITH_TF: the transfer-function gradient; WITH_DENSITY: the density
// gradient (at least one of them).  Without the transfer-function gradient
// the replay skips empty macrocells like the forward: a sample there has
// transfer-function alpha 0 at both lookup entries, so its density and
// shading gradients vanish and only the alpha entries would receive any.
// Without the density gradient the shading and stencil adjoints are skipped.
// MULTI: the launch's items belong to several views (item_base, tv), each
// item looks its view up; else to the one view passed in the parameters
// (a.one), whose pointers then stay in the constant bank, as the replay's
// register budget wants.
template <bool WITH_TF, bool WITH_DENSITY, bool MULTI>
__global__ void __launch_bounds__(128, 5) backward_kernel(TrainArgs a) {
  extern __shared__ float4 smem[];
  float4* tf_s = smem;                                         // n_tf + 4 entries
  float* dtf_s = reinterpret_cast<float*>(smem + a.n_tf + 4);  // n_tf * 4 (WITH_TF)
  load_tf(tf_s, a.tf, a.n_tf);
  if (WITH_TF)
    for (int i = threadIdx.x; i < a.n_tf * 4; i += blockDim.x) dtf_s[i] = 0.f;
  __syncthreads();
  const unsigned count = MULTI ? __ldg(a.item_base + a.n_views) : a.one_items;
  const float nf = (float)a.n_tf;
  uint32_t nsamp = 0;
  DevView v1{};
  const int* rb1 = nullptr;
  if constexpr (!MULTI) {
    v1 = a.views[a.one.view];
    rb1 = rank_bricks(a, v1);
  }
  // Warps take kBackwardGrab consecutive items at a time.  The forward lays
  // out each of its 8x4 tiles as rows of 32 (segment m of every lane, then
  // m + 1, ...), so a warp replays consecutive segments of the same rays and
  // finds the bricks warm in L1 from the previous segment.
  // The grab shrinks (to one row) when there are too few items to give every
  // warp several grabs.
  const unsigned lane = threadIdx.x & 31u;
  const unsigned warps = gridDim.x * (blockDim.x / 32u);
  const unsigned take = max(32u, min(kBackwardGrab, (count / (warps * 8u)) & ~31u));
  for (;;) {
    unsigned grab = 0;
    if (lane == 0) grab = atomicAdd(a.grab, take);
    grab = __shfl_sync(0xffffffffu, grab, 0);
    if (grab >= count) break;
    const unsigned end = min(grab + take, count);
    for (unsigned item = grab + lane; item < end; item += 32u) {
      if constexpr (MULTI) {
        int slot = 0;  // item_base[slot] <= item < item_base[slot + 1]
        for (int hi = a.n_views - 1; slot < hi;) {
          const int mid = (slot + hi + 1) >> 1;
          if (__ldg(a.item_base + mid) <= item)
            slot = mid;
          else
            hi = mid - 1;
        }
        const TrainView& tv = a.tv[slot];
        const DevView v = a.views[tv.view];
        const uint2 wk = tv.work[item - __ldg(a.item_base + slot)];
        const Checkpoint ck = tv.ckpt[(size_t)wk.x * tv.ckpt_cap + wk.y];
        nsamp += backward_item<WITH_TF, WITH_DENSITY>(a, v, rank_bricks(a, v), tf_s, dtf_s, nf, wk.x, ck,
                                                      tv.final_rgba[wk.x], tv.dl_drgba[wk.x]);
      } else {
        const uint2 wk = a.one.work[item];
        const Checkpoint ck = a.one.ckpt[(size_t)wk.x * a.one.ckpt_cap + wk.y];
        nsamp += backward_item<WITH_TF, WITH_DENSITY>(a, v1, rb1, tf_s, dtf_s, nf, wk.x, ck, a.one.final_rgba[wk.x],
                                                      a.one.dl_drgba[wk.x]);
      }
    }
  }
  count_samples(a.counter, nsamp);
  if (WITH_TF) {
    __syncthreads();
    for (int i = threadIdx.x; i < a.n_tf * 4; i += blockDim.x) red_add(a.dtf + i, dtf_s[i]);
  }
}

size_t backward_smem(int n_tf, bool with_tf) {
  return (size_t)(n_tf + 4) * sizeof(float4) + (with_tf ? (size_t)n_tf * 4 * sizeof(float) : 0);
}

}  // namespace

cudaError_t launch_forward_train(const TrainArgs& a, unsigned items, int max_grid, bool many, cudaStream_t s) {
  int grid = (int)std::min<unsigned>((items + 3) / 4, (unsigned)max_grid);
  if (grid < 1) grid = 1;
  const size_t smem = (size_t)(a.n_tf + 4) * sizeof(float4);
  if (many)
    forward_train_kernel<kTrainForwardBlocksMany><<<grid, 128, smem, s>>>(a, items);
  else
    forward_train_kernel<kTrainForwardBlocks><<<grid, 128, smem, s>>>(a, items);
  return cudaGetLastError();
}

int forward_train_blocks_per_sm(int n_tf, bool many) {
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(
          &n, many ? forward_train_kernel<kTrainForwardBlocksMany> : forward_train_kernel<kTrainForwardBlocks>, 128,
          (size_t)(n_tf + 4) * sizeof(float4)) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

cudaError_t launch_backward(const TrainArgs& a, int grid, cudaStream_t s) {
  const bool with_tf = a.dtf != nullptr, with_density = a.dgrid4 != nullptr;
  if (!with_tf && !with_density) return cudaErrorInvalidValue;
  const size_t smem = backward_smem(a.n_tf, with_tf);
  const bool multi = a.n_views > 1;
  void (*k)(TrainArgs) =
      multi ? (!with_tf ? backward_kernel<false, true, true>
                        : (with_density ? backward_kernel<true, true, true> : backward_kernel<true, false, true>))
            : (!with_tf ? backward_kernel<false, true, false>
                        : (with_density ? backward_kernel<true, true, false> : backward_kernel<true, false, false>));
  if (smem > 48 * 1024) {
    cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
    if (e != cudaSuccess) return e;
  }
  k<<<grid, 128, smem, s>>>(a);
  return cudaGetLastError();
}

cudaError_t launch_fold_quads(float4* quads, float* out, const int dims[3], cudaStream_t s) {
  const long long rows = (long long)dims[1] * dims[2];
  if (rows <= 0 || rows > 0x7fffffffll || dims[0] <= 0) return cudaErrorInvalidValue;
  const int threads = dims[0] >= 256 ? 256 : 128;
  const int grid = (int)(rows < 152 * 32 ? rows : 152 * 32);
  fold_quads_kernel<<<grid, threads, (threads + 2) * sizeof(float4), s>>>(quads, out, dims[0], (int)rows);
  return cudaGetLastError();
}

int backward_blocks_per_sm(int n_tf) {
  // the instance with the transfer-function gradient needs more shared memory
  const size_t smem = backward_smem(n_tf, true);
  if (smem > 48 * 1024 &&
      cudaFuncSetAttribute(backward_kernel<true, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem) !=
          cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  int n = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, backward_kernel<true, true, true>, 128, smem) != cudaSuccess) {
    cudaGetLastError();
    return 0;
  }
  return n;
}

}  // namespace aloha
