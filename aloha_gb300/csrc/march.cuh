// march.cuh -- device functions of the volume march (sm_103a).
//
// Restates the reference's per-pixel path (deviceCode.cpp:94-107 ray
// generation, 41-57 slab test, 245-254 firstSampleT, 256-298 integrateBrick,
// 354-416 output stage).  This file is compiled with -fmad=false: every fused
// multiply-add is an explicit fmaf, so the results are bit-identical to the
// CPU restatement, which fixes the same evaluation order.
//
// Sampling: voxel-unit coordinate u = o + t*d - voxelRange.lower; the value
// tap is the trilinear interpolation at u, the six gradient taps sit at
// u +- 1/2 (the reference's tc +- 0.5/N, deviceCode.cpp:278-284).  u - 1/2 and
// u + 1/2 differ by exactly 1, so all seven taps read one 20-voxel cross
// around the cell and share their fractional weights.  With the yz-quad brick
// layout (each element holds a voxel's 2x2 (y, z) neighbourhood) the cross is
// five 16-byte and two 8-byte loads per sample (56 texel fetches in the
// reference).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "internal.h"
#include "steps.h"

namespace aloha {

__device__ __forceinline__ float lerpf(float a, float b, float w) { return fmaf(w, b - a, a); }

__device__ __forceinline__ uint32_t pcg_hash(uint32_t v) {
  uint32_t state = v * 747796405u + 2891336453u;
  uint32_t word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
  return (word >> 22u) ^ word;
}

// Per-brick ray offset ils_t0 (deviceCode.cpp:386) from (pixel, accumID, draw).
__device__ __forceinline__ float jitter(int mode, float value, uint32_t pixel, uint32_t accum_id, uint32_t draw) {
  if (mode == ALOHA_JITTER_CONST) return value;
  if (mode == ALOHA_JITTER_HASH) {
    uint32_t h = pcg_hash(pixel ^ pcg_hash(accum_id ^ pcg_hash(draw)));
    return (float)(h >> 8) * (1.0f / 16777216.0f);
  }
  return 0.0f;
}

struct Ray {
  float o[3], d[3];
};

// generateRay (deviceCode.cpp:94-107).
__device__ __forceinline__ Ray generate_ray(const DevView& v, int x, int y) {
  Ray r;
  const float su = (float)x + 0.5f, sv = (float)y + 0.5f;
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    r.o[a] = v.org[a];
    r.d[a] = fmaf(sv, v.dir_dv[a], fmaf(su, v.dir_du[a], v.dir_00[a]));
  }
  const float len2 = fmaf(r.d[2], r.d[2], fmaf(r.d[1], r.d[1], r.d[0] * r.d[0]));
  const float inv = 1.0f / sqrtf(len2);
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    r.d[a] = r.d[a] * inv;
    if (fabsf(r.d[a]) < 1e-5f) r.d[a] = 1e-5f;
  }
  return r;
}

// Slab test (deviceCode.cpp:41-57) against a brick's space range.
__device__ __forceinline__ bool slab(const Ray& r, const float lo[3], const float hi[3], float tmin, float tmax,
                                     float& t0, float& t1) {
  float nr[3], fr[3];
#pragma unroll
  for (int a = 0; a < 3; ++a) {
    const float l = (lo[a] - r.o[a]) / r.d[a];
    const float h = (hi[a] - r.o[a]) / r.d[a];
    nr[a] = fminf(l, h);
    fr[a] = fmaxf(l, h);
  }
  t0 = fmaxf(tmin, fmaxf(fmaxf(nr[0], nr[1]), nr[2]));
  t1 = fminf(tmax, fminf(fminf(fr[0], fr[1]), fr[2]));
  return t0 < t1;
}

// Seven-tap stencil at voxel coordinate (ux, uy, uz) of a padded brick.
// Evaluation order (shared with the CPU restatement): taps displaced along an
// axis interpolate bilinearly across that axis first (x: y then z; y: x then
// z; z: x then y), then lerp along it; the value tap lerps the x-tap columns
// along x.  lerp(a, b, w) = fmaf(w, b - a, a).
struct StencilOut {
  float value, gx, gy, gz;
};

// One axis of the stencil's coordinates at voxel coordinate u: the weight of
// the centre (g = u - floor u) and of the displaced taps (f = m - floor m,
// m = u - 1/2), whether floor m = floor u - 1 (h), and the clamped indices
// i = floor m and c = floor u.  floor u comes from one round-down conversion
// to an integer k; for |u| < 2^22 (every coordinate of a sample inside a
// brick) k and k - 1 are exact floats and m = RN(u - 1/2) lies in
// [k - 1/2, k + 1/2], so floor m = k - (m < k): the same bits as floorf.  For
// a degenerate coordinate beyond that the indices still clamp into the apron,
// where every tap along the axis reads the same edge value, so the (finite)
// weights cannot change the result.
struct AxisCoord {
  int i, c;
  float f, g;
  bool h;
};

__device__ __forceinline__ AxisCoord axis_coord(float u, int n) {
  const float m = u - 0.5f;
  const int k = __float2int_rd(u);
  const float fc = (float)k;
  AxisCoord a;
  a.h = m < fc;
  a.f = m - (a.h ? fc - 1.0f : fc);
  a.g = u - fc;
  a.c = min(max(k, -kApron), n);
  a.i = min(max(a.c - (a.h ? 1 : 0), -kApron), n - 1);
  return a;
}

// The same coordinates from two float floors per axis (floor u, floor m),
// each converted to an index.  One more conversion per axis, but the weights
// do not wait for an integer-to-float conversion: the render's march, bound
// by the latency of its dependent chain, measured faster this way, the
// backward (which also scatters) the other way.
__device__ __forceinline__ AxisCoord axis_coord_floors(float u, int n) {
  const float m = u - 0.5f;
  const float fm = floorf(m), fc = floorf(u);
  AxisCoord a;
  a.h = fc != fm;
  a.f = m - fm;
  a.g = u - fc;
  a.c = min(max((int)fc, -kApron), n);
  a.i = min(max((int)fm, -kApron), n - 1);
  return a;
}

// The stencil's arithmetic from its eight loaded rows (shared by the direct
// loads of stencil() and the staged loads of StagedLoads, so both give the
// same bits).
__device__ __forceinline__ StencilOut stencil_rows(const float4 r00, const float4 r10, const float4 r01,
                                                   const float4 r11, const float2 e0, const float2 e1,
                                                   const float2 f0, const float2 f1, float fx, float fy, float fz,
                                                   float gx, float gy, float gz, bool hx, bool hy, bool hz) {
  const float a000 = r00.x, a100 = r00.y, a200 = r00.z;
  const float a010 = r10.x, a110 = r10.y, a210 = r10.z;
  const float a001 = r01.x, a101 = r01.y, a201 = r01.z;
  const float a011 = r11.x, a111 = r11.y, a211 = r11.z;
  const float b00 = e0.x, b10 = e0.y, b01 = e1.x, b11 = e1.y;
  const float c00 = f0.x, c10 = f0.y, c01 = f1.x, c11 = f1.y;

  // x taps: columns X_k = bilinear (y by gy, then z by gz) at x = ix + k.
  const float X0 = lerpf(lerpf(a000, a010, gy), lerpf(a001, a011, gy), gz);
  const float X1 = lerpf(lerpf(a100, a110, gy), lerpf(a101, a111, gy), gz);
  const float X2 = lerpf(lerpf(a200, a210, gy), lerpf(a201, a211, gy), gz);
  StencilOut s;
  s.value = lerpf(hx ? X1 : X0, hx ? X2 : X1, gx);
  s.gx = lerpf(X1, X2, fx) - lerpf(X0, X1, fx);

  // Voxels at x = cx, cx+1 of the four (y, z) rows of the X region.
  const float v000 = hx ? a100 : a000, v100 = hx ? a200 : a100;
  const float v010 = hx ? a110 : a010, v110 = hx ? a210 : a110;
  const float v001 = hx ? a101 : a001, v101 = hx ? a201 : a101;
  const float v011 = hx ? a111 : a011, v111 = hx ? a211 : a111;
  // x lerps shared by the y and z taps
  const float L00 = lerpf(v000, v100, gx);  // (cy,   cz)
  const float L10 = lerpf(v010, v110, gx);  // (cy+1, cz)
  const float L01 = lerpf(v001, v101, gx);  // (cy,   cz+1)
  const float L11 = lerpf(v011, v111, gx);  // (cy+1, cz+1)

  // y taps: rows bilinear (x by gx, then z by gz).
  const float Yc0 = lerpf(L00, L01, gz);
  const float Yc1 = lerpf(L10, L11, gz);
  const float Ye = lerpf(lerpf(b00, b10, gx), lerpf(b01, b11, gx), gz);
  const float Y0 = hy ? Ye : Yc0, Y1 = hy ? Yc0 : Yc1, Y2 = hy ? Yc1 : Ye;
  s.gy = lerpf(Y1, Y2, fy) - lerpf(Y0, Y1, fy);

  // z taps: slices bilinear (x by gx, then y by gy).
  const float Zc0 = lerpf(L00, L10, gy);
  const float Zc1 = lerpf(L01, L11, gy);
  const float Ze = lerpf(lerpf(c00, c10, gx), lerpf(c01, c11, gx), gy);
  const float Z0 = hz ? Ze : Zc0, Z1 = hz ? Zc0 : Zc1, Z2 = hz ? Zc1 : Ze;
  s.gz = lerpf(Z1, Z2, fz) - lerpf(Z0, Z1, fz);
  return s;
}

// The stencil from its seven loaded yz-quads (element (x,y,z) holds V(x,y,z),
// V(x,y+1,z), V(x,y,z+1), V(x,y+1,z+1)): q0..q2 at x = ix..ix+2 of row (cy,
// cz); e0, e1 at x = cx, cx+1 of row (ye, cz); the first halves f0, f1 at
// x = cx, cx+1 of row (cy, ze).  Regrouped into the x rows stencil_rows takes.
__device__ __forceinline__ StencilOut stencil_quads(const float4 q0, const float4 q1, const float4 q2,
                                                    const float4 e0, const float4 e1, const float2 f0,
                                                    const float2 f1, float fx, float fy, float fz, float gx, float gy,
                                                    float gz, bool hx, bool hy, bool hz) {
  return stencil_rows(make_float4(q0.x, q1.x, q2.x, 0.f), make_float4(q0.y, q1.y, q2.y, 0.f),
                      make_float4(q0.z, q1.z, q2.z, 0.f), make_float4(q0.w, q1.w, q2.w, 0.f), make_float2(e0.x, e1.x),
                      make_float2(e0.z, e1.z), make_float2(f0.x, f1.x), make_float2(f0.y, f1.y), fx, fy, fz, gx, gy,
                      gz, hx, hy, hz);
}

// ROUND_DOWN picks axis_coord (one conversion per axis) over
// axis_coord_floors; both give the same bits.
template <bool ROUND_DOWN = false>
__device__ __forceinline__ StencilOut stencil(const float4* __restrict__ base, int sy, int sz, int nx, int ny,
                                              int nz, float ux, float uy, float uz) {
  // Indices, clamped into the apron.  Every index the oracle clamps to the
  // edge maps to an apron voxel holding that edge value, so these clamps only
  // keep pathological coordinates in bounds and never change a value.
  const AxisCoord X = ROUND_DOWN ? axis_coord(ux, nx) : axis_coord_floors(ux, nx);
  const AxisCoord Y = ROUND_DOWN ? axis_coord(uy, ny) : axis_coord_floors(uy, ny);
  const AxisCoord Z = ROUND_DOWN ? axis_coord(uz, nz) : axis_coord_floors(uz, nz);
  const int ix = X.i, iy = Y.i, iz = Z.i, cx = X.c, cy = Y.c, cz = Z.c;
  const bool hx = X.h, hy = Y.h, hz = Z.h;  // floor(u) == floor(u - 1/2) + 1

  // X region: x in {ix, ix+1, ix+2}, y in {cy, cy+1}, z in {cz, cz+1}: one
  // yz-quad per x.
  const float4* p0 = base + (cz * sz + cy * sy + ix);
  const float4 q0 = __ldg(p0), q1 = __ldg(p0 + 1), q2 = __ldg(p0 + 2);
  // Extra y row (iy or iy+2) at z in {cz, cz+1} and extra z slice (iz or
  // iz+2) at y in {cy, cy+1}, both at x in {cx, cx+1}: two components of a
  // yz-quad each.
  const int ye = hy ? iy : iy + 2;
  const int ze = hz ? iz : iz + 2;
  const float4* p1 = base + (cz * sz + ye * sy + cx);
  const float4 e0 = __ldg(p1), e1 = __ldg(p1 + 1);
  const float4* p2 = base + (ze * sz + cy * sy + cx);  // only (y, y+1) at z: the quads' first halves
  const float2 f0 = __ldg(reinterpret_cast<const float2*>(p2)), f1 = __ldg(reinterpret_cast<const float2*>(p2 + 1));
  return stencil_quads(q0, q1, q2, e0, e1, f0, f1, X.f, Y.f, Z.f, X.g, Y.g, Z.g, hx, hy, hz);
}

// ---- Where the stencil's rows come from -----------------------------------
// DirectLoads: read-only loads from the brick when the sample is evaluated.
// StagedLoads: the rows of the next sample along the ray are copied into this
// thread's own shared-memory slots with cp.async while the current sample is
// evaluated (double buffering), so the gather's latency overlaps the
// arithmetic without holding registers.  Each thread stages only for itself,
// so no warp or CTA synchronisation is involved; a staged sample is used only
// when the march reaches exactly its t within the same brick march (t is
// strictly increasing there), else it is dropped.  The values are the same
// as the direct loads', so frames are bit-identical.
struct DirectLoads {
  static constexpr bool kStaged = false;
  static constexpr int kSteps = 1;  // march steps per loop trip
  __device__ __forceinline__ void begin_brick() {}
  __device__ __forceinline__ void finish() {}
};

// Direct loads with the march loop written out STEPS steps per trip (a
// step-unrolled march: the same steps in the same order, the same bits).
template <int STEPS>
struct UnrolledDirectLoads : DirectLoads {
  static constexpr int kSteps = STEPS;
};

__device__ __forceinline__ void cp_async16(void* smem, const void* gmem) {
  const unsigned a = (unsigned)__cvta_generic_to_shared(smem);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 16;\n" ::"r"(a), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N> __device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Shared memory of the staged loads: [2 slots][7 rows][kRenderThreads] float4
// (each thread's rows strided by the CTA size, so a warp's row reads are
// contiguous): the seven yz-quads of stencil(), in its order.
constexpr int kStageRows = 7;
constexpr size_t kStageBytes = (size_t)2 * kStageRows * kRenderThreads * sizeof(float4);

struct StagedLoads {
  static constexpr bool kStaged = true;
  static constexpr int kSteps = 1;
  float4* col;     // this thread's column: row e of slot k at col[(k * kStageRows + e) * kRenderThreads]
  float t_staged;  // t of the sample in slot `cur` (NaN: none)
  int cur;
  bool inflight;   // copies may be outstanding
  __device__ __forceinline__ void init(float4* stage_smem) {
    col = stage_smem + threadIdx.x;
    t_staged = __int_as_float(0x7fffffff);
    cur = 0;
    inflight = false;
  }
  __device__ __forceinline__ void begin_brick() { t_staged = __int_as_float(0x7fffffff); }
  // Outstanding copies must land before the CTA's shared memory is released.
  __device__ __forceinline__ void finish() {
    if (inflight) cp_async_wait_all();
    inflight = false;
  }
  __device__ __forceinline__ float4* row(int slot, int e) const { return col + (slot * kStageRows + e) * kRenderThreads; }

  // Starts the copies of the stencil rows at (ux, uy, uz) into `slot`: the
  // addresses of stencil(), clamped into the apron.
  __device__ __forceinline__ void issue(int slot, const float4* __restrict__ base, int sy, int sz, int nx, int ny,
                                        int nz, float ux, float uy, float uz) const {
    const AxisCoord X = axis_coord_floors(ux, nx), Y = axis_coord_floors(uy, ny), Z = axis_coord_floors(uz, nz);
    const int ix = X.i, iy = Y.i, iz = Z.i, cx = X.c, cy = Y.c, cz = Z.c;
    const int ye = Y.h ? iy : iy + 2;
    const int ze = Z.h ? iz : iz + 2;
    const float4* p0 = base + (cz * sz + cy * sy + ix);
    const float4* p1 = base + (cz * sz + ye * sy + cx);
    const float4* p2 = base + (ze * sz + cy * sy + cx);
    cp_async16(row(slot, 0), p0);
    cp_async16(row(slot, 1), p0 + 1);
    cp_async16(row(slot, 2), p0 + 2);
    cp_async16(row(slot, 3), p1);
    cp_async16(row(slot, 4), p1 + 1);
    cp_async16(row(slot, 5), p2);
    cp_async16(row(slot, 6), p2 + 1);
    cp_async_commit();
  }

  // The sample at t (voxel coordinate u): its rows from the slot it was
  // staged in (or loaded now), after starting the copies of the next sample
  // t + dt when that one lies before t1.
  __device__ __forceinline__ StencilOut sample(const float4* __restrict__ base, int sy, int sz, int nx, int ny, int nz,
                                               float ux, float uy, float uz, float t, float t1, float dt,
                                               const float o[3], const float d[3], float lox, float loy, float loz) {
    if (!(t_staged == t)) {
      if (inflight) cp_async_wait_all();  // a dropped copy may still be landing in `cur`
      issue(cur, base, sy, sz, nx, ny, nz, ux, uy, uz);
    }
    const float tn = t + dt;  // the march's next t, by the same addition
    const bool next = tn < t1;
    if (next) {
      issue(cur ^ 1, base, sy, sz, nx, ny, nz, fmaf(tn, d[0], o[0]) - lox, fmaf(tn, d[1], o[1]) - loy,
            fmaf(tn, d[2], o[2]) - loz);
      cp_async_wait<1>();
    } else {
      cp_async_wait<0>();
    }
    const AxisCoord X = axis_coord_floors(ux, nx), Y = axis_coord_floors(uy, ny), Z = axis_coord_floors(uz, nz);
    const float4 f0 = *row(cur, 5), f1 = *row(cur, 6);
    const StencilOut s = stencil_quads(*row(cur, 0), *row(cur, 1), *row(cur, 2), *row(cur, 3), *row(cur, 4),
                                       make_float2(f0.x, f0.y), make_float2(f1.x, f1.y), X.f, Y.f, Z.f, X.g, Y.g, Z.g,
                                       X.h, Y.h, Z.h);
    t_staged = next ? tn : __int_as_float(0x7fffffff);
    inflight = next;
    cur ^= 1;
    return s;
  }
};

// tex1D on the transfer function (linear, normalized coords, border 0;
// waikikiRenderer.cpp:990-1008).  tf_s holds the n entries at [2, n+2) with
// two zero entries on each side.
__device__ __forceinline__ float4 tf_lookup(const float4* __restrict__ tf_s, int n, float nf, float v) {
  const float xb = v * nf - 0.5f;
  const float fl = floorf(xb);
  const float w = xb - fl;
  const int i = min(max((int)fl, -2), n);
  const float4 e0 = tf_s[i + 2];
  const float4 e1 = tf_s[i + 3];
  return make_float4(lerpf(e0.x, e1.x, w), lerpf(e0.y, e1.y, w), lerpf(e0.z, e1.z, w), lerpf(e0.w, e1.w, w));
}

// Gradient shading .1 + .9 |N.d|, N = g / |g + 1e-4| (deviceCode.cpp:285,294),
// evaluated as (g.d) / |g + 1e-4|.
__device__ __forceinline__ float shade_factor(const StencilOut& s, const Ray& r) {
  const float ex = s.gx + 1e-4f, ey = s.gy + 1e-4f, ez = s.gz + 1e-4f;
  const float len = sqrtf(fmaf(ez, ez, fmaf(ey, ey, ex * ex)));
  const float gd = fmaf(s.gz, r.d[2], fmaf(s.gy, r.d[1], s.gx * r.d[0]));
  return fmaf(0.9f, fabsf(gd / len), 0.1f);
}

// Front-to-back compositing of one sample (deviceCode.cpp:292-296).
__device__ __forceinline__ void composite_step(float4& color, const float4 c, float shade) {
  const float oma = 1.0f - color.w;
  const float s1 = oma * c.w;
  color.x = fmaf(s1 * c.x, shade, color.x);
  color.y = fmaf(s1 * c.y, shade, color.y);
  color.z = fmaf(s1 * c.z, shade, color.z);
  color.w = fmaf(oma, c.w, color.w);
}

// A march hook sees every sample, full or skipped, before it is taken: its
// t, the samples already taken in the brick and the colour so far.  The
// render passes NoHook; the differentiable forward stores checkpoints.  An
// active hook keeps `left`, the samples it lets pass before it needs to see
// one again, so runs of skipped samples only stop where it does.
struct NoHook {
  static constexpr bool kActive = false;
  __device__ __forceinline__ void operator()(float, uint32_t, const float4&) {}
};

// integrateBrick (deviceCode.cpp:256-298) over [t0, t1); returns the number
// of samples taken.
template <class Hook, class Loads = DirectLoads>
__device__ __forceinline__ uint32_t march_brick(const DevBrick& b, const float4* __restrict__ tf_s, int n_tf,
                                                const Ray& r, float t0, float t1, float ils, float dt, float et,
                                                float4& color, Hook& hook, Loads& loads) {
  const float4* __restrict__ base = b.base;
  const int sy = b.sy, sz = b.sz, nx = b.n[0], ny = b.n[1], nz = b.n[2];
  const float lox = b.lo[0], loy = b.lo[1], loz = b.lo[2];
  const float nf = (float)n_tf;
  const uint32_t cap = march_cap(t0, t1, dt);
  const uint8_t* __restrict__ empty = b.empty;
  const int mnx = (nx + kMacro - 1) >> kMacroShift, mny = (ny + kMacro - 1) >> kMacroShift;
  // Brick-local ray origin, inverse direction and the rounding margin (voxel
  // units) that makes the macrocell exit bound below conservative: u = o + t d
  // - lo is computed with a few ulps of the largest magnitude involved.
  const float offx = r.o[0] - lox, offy = r.o[1] - loy, offz = r.o[2] - loz;
  const float idx_ = 1.0f / r.d[0], idy = 1.0f / r.d[1], idz = 1.0f / r.d[2];
  const float mag = fmaxf(fmaxf(fabsf(r.o[0]) + fabsf(lox), fabsf(r.o[1]) + fabsf(loy)),
                          fabsf(r.o[2]) + fabsf(loz)) + fabsf(t1);
  const float eps = 2e-6f * mag + 1e-4f;
  uint32_t n = 0;
  float t = first_sample_t(t0, dt, ils);
  const bool exact = exact_steps(t, t1, dt);
  const float inv_dt = 1.0f / dt;
  // Samples before t_cell lie in the last macrocell found non-empty, so they
  // need no lookup.  Only the skip below depends on the lookup (a full sample
  // in an empty macrocell leaves the colour unchanged as well), so the bound
  // only has to be right for speed.
  float t_cell = t0;
  loads.begin_brick();
  if constexpr (Loads::kSteps > 1 && !Hook::kActive && !Loads::kStaged) {
    // The loop below for the render (no hook, direct loads), written out
    // Loads::kSteps steps per trip.
    auto step = [&]() -> bool {
      if (!(t < t1 && color.w < et && n < cap)) return false;
      const float ux = fmaf(t, r.d[0], r.o[0]) - lox;
      const float uy = fmaf(t, r.d[1], r.o[1]) - loy;
      const float uz = fmaf(t, r.d[2], r.o[2]) - loz;
      if (empty && !(t < t_cell)) {
        const int mx = min(max(__float2int_rd(ux), 0), nx - 1) >> kMacroShift;
        const int my = min(max(__float2int_rd(uy), 0), ny - 1) >> kMacroShift;
        const int mz = min(max(__float2int_rd(uz), 0), nz - 1) >> kMacroShift;
        const float bx = (float)(mx << kMacroShift), by = (float)(my << kMacroShift),
                    bz = (float)(mz << kMacroShift);
        const float ex = ((r.d[0] > 0.f ? bx + (float)kMacro - eps : bx + eps) - offx) * idx_;
        const float ey = ((r.d[1] > 0.f ? by + (float)kMacro - eps : by + eps) - offy) * idy;
        const float ez = ((r.d[2] > 0.f ? bz + (float)kMacro - eps : bz + eps) - offz) * idz;
        const float tb = fminf(fminf(fminf(ex, ey), ez), t1);
        if (__ldg(empty + (mz * mny + my) * mnx + mx)) {
          ++n;
          t = t + dt;
          if (exact) {
            run_steps(t, n, tb, cap, dt, inv_dt, 0xffffffffu);
          } else {
            while (t < tb && n < cap) {
              ++n;
              t = t + dt;
            }
          }
          return true;
        }
        t_cell = tb;
      }
      ++n;
      const StencilOut s = stencil(base, sy, sz, nx, ny, nz, ux, uy, uz);
      const float shade = shade_factor(s, r);
      const float4 c = tf_lookup(tf_s, n_tf, nf, s.value);
      composite_step(color, c, shade);
      t = t + dt;
      return true;
    };
    for (bool go = true; go;) {
#pragma unroll
      for (int k = 0; k < Loads::kSteps; ++k) go = go && step();
    }
    return n;
  }
  while (t < t1 && color.w < et && n < cap) {
    const float ux = fmaf(t, r.d[0], r.o[0]) - lox;
    const float uy = fmaf(t, r.d[1], r.o[1]) - loy;
    const float uz = fmaf(t, r.d[2], r.o[2]) - loz;
    if (empty && !(t < t_cell)) {
      const int mx = min(max(__float2int_rd(ux), 0), nx - 1) >> kMacroShift;
      const int my = min(max(__float2int_rd(uy), 0), ny - 1) >> kMacroShift;
      const int mz = min(max(__float2int_rd(uz), 0), nz - 1) >> kMacroShift;
      // tb: the ray's exit from the macrocell's box shrunk by eps; every
      // sample before it lies in this macrocell.
      const float bx = (float)(mx << kMacroShift), by = (float)(my << kMacroShift), bz = (float)(mz << kMacroShift);
      const float ex = ((r.d[0] > 0.f ? bx + (float)kMacro - eps : bx + eps) - offx) * idx_;
      const float ey = ((r.d[1] > 0.f ? by + (float)kMacro - eps : by + eps) - offy) * idy;
      const float ez = ((r.d[2] > 0.f ? bz + (float)kMacro - eps : bz + eps) - offz) * idz;
      const float tb = fminf(fminf(fminf(ex, ey), ez), t1);
      if (__ldg(empty + (mz * mny + my) * mnx + mx)) {
        // Empty macrocell: a sample there has alpha exactly 0 and leaves the
        // colour unchanged, so only t and the sample count advance (the same
        // t += dt sequence as full samples) up to tb; the test resumes there.
        // The first is always taken.  With exact steps the rest of the run is
        // one jump (one more per power of two it crosses, and one per
        // checkpoint the hook needs).
        if constexpr (!Hook::kActive) {
          ++n;
          t = t + dt;
          if (exact) {
            run_steps(t, n, tb, cap, dt, inv_dt, 0xffffffffu);
            continue;
          }
          while (t < tb && n < cap) {
            ++n;
            t = t + dt;
          }
        } else if (exact) {
          hook(t, n, color);
          ++n;
          t = t + dt;
          for (;;) {
            hook.left -= run_steps(t, n, tb, cap, dt, inv_dt, hook.left);
            if (!(t < tb && n < cap)) break;
            hook(t, n, color);  // a checkpoint falls due here (hook.left == 0)
            ++n;
            t = t + dt;
          }
        } else {
          hook(t, n, color);
          ++n;
          t = t + dt;
          while (t < tb && n < cap) {
            uint32_t k = hook.left;
            while (k > 0 && t < tb && n < cap) {
              ++n;
              t = t + dt;
              --k;
            }
            hook.left = k;
            if (k == 0 && t < tb && n < cap) {
              hook(t, n, color);
              ++n;
              t = t + dt;
            }
          }
        }
        continue;
      }
      t_cell = tb;
    }
    hook(t, n, color);
    ++n;
    StencilOut s;
    if constexpr (Loads::kStaged)
      s = loads.sample(base, sy, sz, nx, ny, nz, ux, uy, uz, t, t1, dt, r.o, r.d, lox, loy, loz);
    else
      s = stencil(base, sy, sz, nx, ny, nz, ux, uy, uz);
    const float shade = shade_factor(s, r);
    const float4 c = tf_lookup(tf_s, n_tf, nf, s.value);
    composite_step(color, c, shade);
    t = t + dt;
  }
  return n;
}

template <class Hook>
__device__ __forceinline__ uint32_t march_brick(const DevBrick& b, const float4* __restrict__ tf_s, int n_tf,
                                                const Ray& r, float t0, float t1, float ils, float dt, float et,
                                                float4& color, Hook& hook) {
  DirectLoads direct;
  return march_brick(b, tf_s, n_tf, r, t0, t1, ils, dt, et, color, hook, direct);
}

// ---- Sample-parallel lane groups ------------------------------------------
// G lanes of a warp march one ray together: all hold the serial march's state
// (t, n, colour, t_cell) identically.  One group iteration replaces up to G
// iterations of march_brick:
//  1. at the base sample (t, n) the loop test and the macrocell test run as
//     in the serial loop; an empty macrocell starts the same skip run, taken
//     identically by every lane;
//  2. lane j takes sample j of the group, at the t the serial loop reaches by
//     j more rounded additions of dt, if it lies before t1 and under the
//     iteration cap; past t_cell it looks up its own macrocell and drops the
//     sample if that one is empty (the serial loop would skip it; a full
//     sample of alpha 0 leaves the colour unchanged either way);
//  3. every lane evaluates its sample (stencil, shading, lookup) at once;
//  4. the samples are composited in lane order from shuffled values, in every
//     lane: before sample j the serial loop's head test (t_j < t1, colour
//     alpha < ET, n < cap) decides whether it and the later ones are taken;
//     each taken sample adds 1 to n and dt to t.
// The colour, n and t leave the iteration as the serial loop would leave them
// after the same samples, bit for bit.  A ray's samples take about G times
// fewer dependent steps, at the cost of the shuffles and of the samples
// evaluated past the ray's end.
struct LaneGroup {
  int lane;       // index in the group, 0..G-1
  unsigned mask;  // the group's lanes in the warp
  int base;       // first lane of the group in the warp
};

template <int G>
__device__ __forceinline__ uint32_t march_brick_group(const DevBrick& b, const float4* __restrict__ tf_s, int n_tf,
                                                      const Ray& r, float t0, float t1, float ils, float dt, float et,
                                                      float4& color, const LaneGroup& g) {
  const float4* __restrict__ base = b.base;
  const int sy = b.sy, sz = b.sz, nx = b.n[0], ny = b.n[1], nz = b.n[2];
  const float lox = b.lo[0], loy = b.lo[1], loz = b.lo[2];
  const float nf = (float)n_tf;
  const uint32_t cap = march_cap(t0, t1, dt);
  const uint8_t* __restrict__ empty = b.empty;
  const int mnx = (nx + kMacro - 1) >> kMacroShift, mny = (ny + kMacro - 1) >> kMacroShift;
  const float offx = r.o[0] - lox, offy = r.o[1] - loy, offz = r.o[2] - loz;
  const float idx_ = 1.0f / r.d[0], idy = 1.0f / r.d[1], idz = 1.0f / r.d[2];
  const float mag = fmaxf(fmaxf(fabsf(r.o[0]) + fabsf(lox), fabsf(r.o[1]) + fabsf(loy)),
                          fabsf(r.o[2]) + fabsf(loz)) + fabsf(t1);
  const float eps = 2e-6f * mag + 1e-4f;
  uint32_t n = 0;
  float t = first_sample_t(t0, dt, ils);
  const bool exact = exact_steps(t, t1, dt);
  const float inv_dt = 1.0f / dt;
  float t_cell = t0;
  while (t < t1 && color.w < et && n < cap) {
    if (empty && !(t < t_cell)) {
      // the base sample's macrocell, exactly as march_brick
      const float ux = fmaf(t, r.d[0], r.o[0]) - lox;
      const float uy = fmaf(t, r.d[1], r.o[1]) - loy;
      const float uz = fmaf(t, r.d[2], r.o[2]) - loz;
      const int mx = min(max(__float2int_rd(ux), 0), nx - 1) >> kMacroShift;
      const int my = min(max(__float2int_rd(uy), 0), ny - 1) >> kMacroShift;
      const int mz = min(max(__float2int_rd(uz), 0), nz - 1) >> kMacroShift;
      const float bx = (float)(mx << kMacroShift), by = (float)(my << kMacroShift), bz = (float)(mz << kMacroShift);
      const float ex = ((r.d[0] > 0.f ? bx + (float)kMacro - eps : bx + eps) - offx) * idx_;
      const float ey = ((r.d[1] > 0.f ? by + (float)kMacro - eps : by + eps) - offy) * idy;
      const float ez = ((r.d[2] > 0.f ? bz + (float)kMacro - eps : bz + eps) - offz) * idz;
      const float tb = fminf(fminf(fminf(ex, ey), ez), t1);
      if (__ldg(empty + (mz * mny + my) * mnx + mx)) {
        ++n;
        t = t + dt;
        if (exact) {
          run_steps(t, n, tb, cap, dt, inv_dt, 0xffffffffu);
          continue;
        }
        while (t < tb && n < cap) {
          ++n;
          t = t + dt;
        }
        continue;
      }
      t_cell = tb;
    }
    // this lane's sample: the serial loop's t after g.lane more steps
    float tk = t;
    for (int j = 0; j < g.lane; ++j) tk = tk + dt;
    const bool in_range = tk < t1 && n + (uint32_t)g.lane < cap;
    bool full = in_range;
    float4 c = make_float4(0.f, 0.f, 0.f, 0.f);
    float shade = 0.f;
    if (in_range) {
      const float vx = fmaf(tk, r.d[0], r.o[0]) - lox;
      const float vy = fmaf(tk, r.d[1], r.o[1]) - loy;
      const float vz = fmaf(tk, r.d[2], r.o[2]) - loz;
      if (empty && !(tk < t_cell)) {
        const int mx = min(max(__float2int_rd(vx), 0), nx - 1) >> kMacroShift;
        const int my = min(max(__float2int_rd(vy), 0), ny - 1) >> kMacroShift;
        const int mz = min(max(__float2int_rd(vz), 0), nz - 1) >> kMacroShift;
        full = !__ldg(empty + (mz * mny + my) * mnx + mx);
      }
      if (full) {
        const StencilOut s = stencil(base, sy, sz, nx, ny, nz, vx, vy, vz);
        shade = shade_factor(s, r);
        c = tf_lookup(tf_s, n_tf, nf, s.value);
      }
    }
    const unsigned in_mask = __ballot_sync(g.mask, in_range) >> g.base;
    const unsigned full_mask = __ballot_sync(g.mask, full) >> g.base;
#pragma unroll
    for (int j = 0; j < G; ++j) {
      const float cx = __shfl_sync(g.mask, c.x, j, G), cy = __shfl_sync(g.mask, c.y, j, G);
      const float cz = __shfl_sync(g.mask, c.z, j, G), cw = __shfl_sync(g.mask, c.w, j, G);
      const float sh = __shfl_sync(g.mask, shade, j, G);
      if (!((in_mask >> j) & 1u) || !(color.w < et)) break;
      if ((full_mask >> j) & 1u) composite_step(color, make_float4(cx, cy, cz, cw), sh);
      ++n;
      t = t + dt;
    }
  }
  return n;
}


__device__ __forceinline__ float saturatef_(float x) { return fminf(fmaxf(x, 0.0f), 1.0f); }

// temperature_to_rgb (deviceCode.cpp:300-314).
__device__ __forceinline__ void heat_color(float t, float out[3]) {
  const float K = 4.0f / 6.0f;
  const float h = K - K * t;
  const float v = 0.5f + 0.5f * t;
  const float s = saturatef_(h) * 6.0f;
  out[0] = v * saturatef_(fabsf(s - 3.0f) - 1.0f);
  out[1] = v * saturatef_(2.0f - fabsf(s - 2.0f));
  out[2] = v * saturatef_(2.0f - fabsf(s - 4.0f));
}

__device__ __forceinline__ uint32_t quantize8(float x) {
  const float c = fminf(fmaxf(x, 0.0f), 1.0f);
  return (uint32_t)(c * 255.0f + 0.5f);
}

__device__ __forceinline__ uint32_t pack_rgba(float4 c) {
  return quantize8(c.x) | (quantize8(c.y) << 8) | (quantize8(c.z) << 16) | (quantize8(c.w) << 24);
}

// Loads the transfer function into shared memory with two zero entries on
// each side (border addressing).
__device__ __forceinline__ void load_tf(float4* tf_s, const float4* __restrict__ tf, int n) {
  for (int i = threadIdx.x; i < n + 4; i += blockDim.x) {
    const int k = i - 2;
    tf_s[i] = (k >= 0 && k < n) ? __ldg(tf + k) : make_float4(0.f, 0.f, 0.f, 0.f);
  }
}

// One virtual rank's march for one pixel (deviceCode.cpp:378-399): the
// rank's bricks [j0, j1) of the view schedule front to back, spp draws, early
// termination on the rank's own alpha.  Returns the spp sum of the colours;
// z = nearest brick entry / max depth, ns = samples taken.
template <class Loads = DirectLoads, int G = 1>
__device__ __forceinline__ float4 march_rank(const FrameArgs& a, const DevView& v, const float4* tf_s, const Ray& ray,
                                             const int* __restrict__ rbricks, int j0, int j1, int pixel, float& z,
                                             uint32_t& ns, Loads& loads, const LaneGroup& g = LaneGroup{0, 0u, 0}) {
  uint32_t draw = 0;
  // one pass of the rank's bricks (one sample per pixel of spp)
  auto pass = [&]() -> float4 {
    float4 color = make_float4(0.f, 0.f, 0.f, 0.f);
    float tmin = 0.0f;
    for (int j = j0; j < j1; ++j) {
      const DevBrick b = a.bricks[__ldg(rbricks + j)];
      float t0, t1;
      if (!slab(ray, b.space_lo, b.space_hi, tmin, 1e10f, t0, t1)) continue;
      const float ils = jitter(a.jitter_mode, a.jitter_value, (uint32_t)pixel, (uint32_t)a.accum_id, draw++);
      const float tnear = (t0 > tmin ? t0 : 0.0f) + tmin;
      z = fminf(z, tnear / v.max_depth);
      NoHook none;
      if constexpr (G > 1)
        ns += march_brick_group<G>(b, tf_s, a.n_tf, ray, t0, t1, ils, a.dt, a.et_alpha, color, g);
      else
        ns += march_brick(b, tf_s, a.n_tf, ray, t0, t1, ils, a.dt, a.et_alpha, color, none, loads);
      tmin = t1 + 1e-20f;
      if (!(color.w < a.et_alpha)) break;
    }
    return color;
  };
  // The sum over passes starts from the first pass's colour: 0 + c = c, as a
  // march colour is never -0 (it starts at +0 and every update is an fmaf
  // onto it, and an exact zero sum rounds to +0).  With one pass no sum is
  // then live across the march.
  float4 acc = pass();
  for (int s = 1; s < a.spp; ++s) {
    const float4 color = pass();
    acc.x = acc.x + color.x;
    acc.y = acc.y + color.y;
    acc.z = acc.z + color.z;
    acc.w = acc.w + color.w;
  }
  return acc;
}

// renderFrame's per-rank output stage (deviceCode.cpp:400-416): heat map,
// accumulation buffer, 1/(accumID+1) scale, crosshair, 1/spp.  Writes the
// rank's image and depth into the given [n_ranks][H*W] planes when they are
// not null; returns the rank image.
__device__ __forceinline__ float4 rank_output(const FrameArgs& a, int W, int H, int r, int x, int y, int pixel,
                                              size_t npx, float4 acc, uint32_t ns, float z, float4* img_planes,
                                              float* depth_planes) {
  if (a.heat_map) {
    float hc[3];
    heat_color((float)ns * (a.heat_map_scale / (float)a.spp), hc);
    acc.x = fmaf(0.5f, acc.x, hc[0]);
    acc.y = fmaf(0.5f, acc.y, hc[1]);
    acc.z = fmaf(0.5f, acc.z, hc[2]);
    acc.w = fmaf(0.5f, acc.w, 0.5f);
  }
  if (a.accum) {
    float4* ap = a.accum + ((size_t)r * npx + pixel);
    if (a.accum_id > 0) {
      const float4 old = *ap;
      acc.x = acc.x + old.x;
      acc.y = acc.y + old.y;
      acc.z = acc.z + old.z;
      acc.w = acc.w + old.w;
    }
    if (a.accumulate) *ap = acc;
  }
  const float scale = 1.0f / (float)(a.accum_id + 1);
  acc.x = acc.x * scale;
  acc.y = acc.y * scale;
  acc.z = acc.z * scale;
  acc.w = acc.w * scale;
  if (a.crosshair && (x == W / 2 || y == H / 2)) {
    acc.x = 1.0f - acc.x;
    acc.y = 1.0f - acc.y;
    acc.z = 1.0f - acc.z;
    acc.w = 1.0f - acc.w;
  }
  const float inv_spp = 1.0f / (float)a.spp;
  const float4 img = make_float4(acc.x * inv_spp, acc.y * inv_spp, acc.z * inv_spp, acc.w * inv_spp);
  if (img_planes) img_planes[(size_t)r * npx + pixel] = img;
  if (depth_planes) depth_planes[(size_t)r * npx + pixel] = z;
  return img;
}

// True when renderFrame's output stage leaves a rank image equal to the
// march's colour: one sample per pixel, no accumulation, heat map or
// crosshair (then img = acc * (1 / 1) * (1 / 1) = acc exactly); plain_output
// also wants no rank planes.
__device__ __forceinline__ bool plain_output_stage(const FrameArgs& a) {
  return a.spp == 1 && a.accum_id == 0 && !a.heat_map && !a.crosshair && !(a.accum && a.accumulate);
}
__device__ __forceinline__ bool plain_output(const FrameArgs& a) {
  return plain_output_stage(a) && !a.rank_images && !a.rank_depth;
}

// Front-to-back ordered "over" of rank images (IceT BLEND with
// ORDERED_COMPOSITE, waikikiRenderer.cpp:910-917,1042-1079): in fp32, or on
// images quantised to 8 bits per channel like IceT's RGBA_UBYTE buffers.
// One float4 holds the state of either mode (the ubyte channels as the bits
// of its components; all-zero bits are 0.0f and 0u), so the blend keeps four
// registers live across the march, not eight.
struct OverBlend {
  float4 comp = make_float4(0.f, 0.f, 0.f, 0.f);
  __device__ __forceinline__ void add(int mode, float4 img) {
    if (mode == ALOHA_COMPOSITE_UBYTE) {
      const uint32_t q0 = quantize8(img.x), q1 = quantize8(img.y), q2 = quantize8(img.z), q3 = quantize8(img.w);
      const uint32_t c0 = __float_as_uint(comp.x), c1 = __float_as_uint(comp.y), c2 = __float_as_uint(comp.z),
                     c3 = __float_as_uint(comp.w);
      const uint32_t f = 255u - c3;
      comp.x = __uint_as_float(min(255u, c0 + (q0 * f + 127u) / 255u));
      comp.y = __uint_as_float(min(255u, c1 + (q1 * f + 127u) / 255u));
      comp.z = __uint_as_float(min(255u, c2 + (q2 * f + 127u) / 255u));
      comp.w = __uint_as_float(min(255u, c3 + (q3 * f + 127u) / 255u));
    } else {
      const float oma = 1.0f - comp.w;
      comp.x = fmaf(oma, img.x, comp.x);
      comp.y = fmaf(oma, img.y, comp.y);
      comp.z = fmaf(oma, img.z, comp.z);
      comp.w = fmaf(oma, img.w, comp.w);
    }
  }
  __device__ __forceinline__ uint32_t pack(int mode) const {
    return mode == ALOHA_COMPOSITE_UBYTE ? (__float_as_uint(comp.x) | (__float_as_uint(comp.y) << 8) |
                                            (__float_as_uint(comp.z) << 16) | (__float_as_uint(comp.w) << 24))
                                         : pack_rgba(comp);
  }
};

// Island membership of a pixel (16x16 tiles dealt round-robin).
__device__ __forceinline__ bool pixel_in_island(const FrameArgs& a, int W, int x, int y) {
  if (a.num_islands <= 1) return true;
  const int tiles_x = (W + 15) / 16;
  return (((x >> 4) + tiles_x * (y >> 4)) % a.num_islands) == a.island_id;
}

// One pixel of one view: every virtual rank marches its bricks and runs
// renderFrame's output stage; the rank images are blended front to back.
// Returns the number of samples.
// With G > 1 the G lanes of `g` render the pixel together (a lane group);
// only the group's first lane writes the frame buffer.  The group form has no
// accumulation buffer and no rank planes (the caller ensures it).
template <class Loads = DirectLoads, int G = 1>
__device__ __forceinline__ uint32_t render_pixel(const FrameArgs& a, const DevView& v, const float4* tf_s, int x,
                                                 int y, uint32_t* fb_out, size_t fb_index, Loads& loads,
                                                 const LaneGroup& g = LaneGroup{0, 0u, 0}) {
  const int W = v.width, H = v.height;
  const int pixel = x + W * y;
  const size_t npx = (size_t)W * H;
  const int R = v.n_ranks;
  const int* __restrict__ order = a.sched + v.sched;
  const int* __restrict__ rstart = order + R;
  const int* __restrict__ rbricks = rstart + R + 1;
  const bool in_island = pixel_in_island(a, W, x, y);
  const Ray ray = generate_ray(v, x, y);
  OverBlend blend;
  uint32_t total = 0;
  if (plain_output(a)) {
    // the output stage is the identity (acc * 1 * 1): nothing it needs stays
    // live across the march
    for (int k = 0; k < R; ++k) {
      const int r = __ldg(order + k);
      float z = 1.0f;
      uint32_t ns = 0;
      float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
      if (in_island)
        acc = march_rank<Loads, G>(a, v, tf_s, ray, rbricks, __ldg(rstart + r), __ldg(rstart + r + 1), pixel, z, ns,
                                   loads, g);
      blend.add(a.composite_mode, acc);
      total += ns;
    }
  } else {
    for (int k = 0; k < R; ++k) {
      const int r = __ldg(order + k);
      float z = 1.0f;
      uint32_t ns = 0;
      float4 acc = make_float4(0.f, 0.f, 0.f, 0.f);
      if (in_island)
        acc = march_rank<Loads, G>(a, v, tf_s, ray, rbricks, __ldg(rstart + r), __ldg(rstart + r + 1), pixel, z, ns,
                                   loads, g);
      blend.add(a.composite_mode, rank_output(a, W, H, r, x, y, pixel, npx, acc, ns, z, a.rank_images, a.rank_depth));
      total += ns;
    }
  }
  if (fb_out && (G == 1 || g.lane == 0)) fb_out[fb_index] = blend.pack(a.composite_mode);
  return total;
}

// Work slot k of a view -> chunk (cx, cy) in centre-out square rings; false
// for slots outside the chunk grid.  Ring r >= 1 holds slots
// [(2r-1)^2, (2r+1)^2), walked up the right edge, left along the top, down
// the left edge and right along the bottom.
__device__ __forceinline__ bool ring_chunk(int k, int cxn, int cyn, int& cx, int& cy) {
  int x = 0, y = 0;
  if (k > 0) {
    int r = (int)((sqrtf((float)k) + 1.0f) * 0.5f);
    while ((2 * r + 1) * (2 * r + 1) <= k) ++r;
    while (r > 1 && (2 * r - 1) * (2 * r - 1) > k) --r;
    const int j = k - (2 * r - 1) * (2 * r - 1);
    const int side = j / (2 * r), off = j % (2 * r);
    if (side == 0) {
      x = r;
      y = -r + 1 + off;
    } else if (side == 1) {
      x = r - 1 - off;
      y = r;
    } else if (side == 2) {
      x = -r;
      y = r - 1 - off;
    } else {
      x = -r + 1 + off;
      y = -r;
    }
  }
  cx = x + (cxn - 1) / 2;
  cy = y + (cyn - 1) / 2;
  return cx >= 0 && cx < cxn && cy >= 0 && cy < cyn;
}

// Warp-aggregated add of per-thread sample counts into a 64-bit counter.
__device__ __forceinline__ void count_samples(unsigned long long* counter, uint32_t n) {
  if (!counter) return;
  const unsigned s = __reduce_add_sync(0xffffffffu, n);
  if ((threadIdx.x & 31) == 0 && s) atomicAdd(counter, (unsigned long long)s);
}

}  // namespace aloha
