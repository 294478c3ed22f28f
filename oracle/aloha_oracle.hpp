// aloha_oracle.hpp -- CPU restatement of Aloha's volume hot path.
//
// TEST INFRASTRUCTURE ONLY.  This header is the oracle that the CUDA path is
// checked against; only tests/, __graft_entry__.smoke() and bench.py's CPU
// baseline arm may load it.  The product library never links or calls it.
//
// What it restates (reference file:line, paths inside the Aloha project):
//   generateRay          deviceCode.cpp:94-107
//   slab intersect       deviceCode.cpp:41-57, VolBrickIsect 207-239
//   brick walk           deviceCode.cpp:378-391
//   firstSampleT         deviceCode.cpp:245-254
//   integrateBrick       deviceCode.cpp:256-298
//   output stage         deviceCode.cpp:354-416 (accumulation, crosshair, make_rgba)
//   heat map colours     deviceCode.cpp:300-329
//   volume texture       waikikiRenderer.cpp:715-775 (linear, clamp, normalized coords)
//   transfer function    waikikiRenderer.cpp:964-1008 (linear, border 0, normalized coords)
//   partitionKD          waikikiRenderer.cpp:150-270
//   computeCompositeOrder waikikiRenderer.cpp:281-316
//   ordered blend        waikikiRenderer.cpp:895-917,1030-1079 (IceT BLEND, ORDERED_COMPOSITE)
//   chopSuey splitter    chopSuey.cpp:245-323
//
// Evaluation order.  The reference leaves rounding to the texture unit
// (8-bit fractional filter weights) and to the compiler.  The oracle fixes one
// exact fp32 evaluation order, written out below; every fused multiply-add is
// an explicit std::fma and the file is compiled with -ffp-contract=off, so the
// CUDA kernels (built with -fmad=false and the same explicit fmaf calls) give
// bit-identical results.  The deviations from the reference's literal
// expressions are all exact-math identities:
//   * sampling is done in voxel units u = pos - voxelRange.lower, which equals
//     the texture's texel coordinate tc*N - 1/2 for tc as deviceCode.cpp:271-275
//     computes it; the gradient taps tc +- 0.5/N are u +- 1/2;
//   * the seven trilinear taps share their fractional weights (u - 1/2 and
//     u + 1/2 differ by exactly 1 in fp32), and are evaluated as bilinear
//     interpolation across the tap axis followed by one lerp along it;
//   * N.d is evaluated as (g.d)/|g + 1e-4| instead of (g/|g + 1e-4|).d;
//   * make_rgba rounds to nearest: q = (uint)(clamp(x,0,1)*255 + 0.5).
// Template parameter R = float gives the parity oracle, R = double the FP64
// re-render used to state the fp32 error.
//
// Pinned to the reference: the reference ships no tests, golden images or
// fixtures, and neither its OptiX build nor its ALOHA_CPU build can be
// compiled here (owl, fakeOwl, IceT and cuteeOwl are empty submodules; MPI,
// Qt and OptiX are absent).  Its hot-path sources do compile on their own:
// ref_harness.cpp runs deviceCode.cpp (unchanged), the Partitioner of
// waikikiRenderer.cpp and the chopSuey tool on the CPU against the stand-ins
// in ref_shim/, and tests/test_reference_pin.py compares this restatement
// with them.  Closed forms derived from the reference's arithmetic
// (tests/test_oracle.py) and central differences of the FP64 adjoint check it
// further; tests/golden/ holds regression vectors of this oracle and frames of
// the reference build.
#pragma once

#include <algorithm>
#include <climits>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

namespace aloha_oracle {

// One brick header exactly as a .vol file stores it (chopSuey.cpp:342-345,
// read back at waikikiRenderer.cpp:615-618): box3i cellRange, box3i
// voxelRange, box3f spaceRange, interval<float> valueRange.
struct BrickDesc {
  int32_t cell_lo[3], cell_hi[3];
  int32_t voxel_lo[3], voxel_hi[3];
  float space_lo[3], space_hi[3];
  float value_lo, value_hi;
};
static_assert(sizeof(BrickDesc) == 80, "brick header is 80 bytes");

// LaunchParams::camera (deviceCode.h:84-89).
struct Camera {
  float org[3], dir_00[3], dir_du[3], dir_dv[3];
};

enum { JITTER_NONE = 0, JITTER_CONST = 1, JITTER_HASH = 2 };
enum { COMPOSITE_FP32 = 0, COMPOSITE_UBYTE = 1 };

// Render settings; the fields the reference hard-codes are parameters here
// (dt: waikikiRenderer.cpp:1023; ET .99f: deviceCode.cpp:270,391; crosshair:
// deviceCode.cpp:410-414; spp/accumID: deviceCode.cpp:344,405-408).
struct Params {
  float dt;
  float et_alpha;
  int32_t jitter_mode;
  float jitter_value;
  int32_t crosshair;
  int32_t spp;
  int32_t accum_id;
  int32_t accumulate;
  int32_t heat_map;
  float heat_map_scale;
  int32_t composite_mode;
  int32_t island_id;
  int32_t num_islands;
};

// ---------------------------------------------------------------- scalars

template <class R> inline R lerp(R a, R b, R w) { return std::fma(w, b - a, a); }

// Integer value of an already-floored number; NaN -> 0, saturates far out.
template <class R> inline int to_int(R f) {
  if (!(f == f)) return 0;
  if (f < R(-1073741824.0)) return -1073741824;
  if (f > R(1073741824.0)) return 1073741824;
  return (int)f;
}

template <class R> inline R clamp01(R x) { return std::fmin(std::fmax(x, R(0)), R(1)); }

// make_rgba for one channel (owl's make_rgba is not in the reference tree;
// the value is rounded to nearest here and in the kernels).
template <class R> inline uint32_t quantize8(R x) {
  R c = clamp01(x);
  return (uint32_t)(c * R(255) + R(0.5));
}

template <class R> inline uint32_t pack_rgba(const R c[4]) {
  return quantize8(c[0]) | (quantize8(c[1]) << 8) | (quantize8(c[2]) << 16) | (quantize8(c[3]) << 24);
}

// PCG hash (Jarzynski & Olano, "Hash Functions for GPU Rendering", JCGT 2020).
inline uint32_t pcg_hash(uint32_t v) {
  uint32_t state = v * 747796405u + 2891336453u;
  uint32_t word = ((state >> ((state >> 28u) + 4u)) ^ state) * 277803737u;
  return (word >> 22u) ^ word;
}

// Per-brick jitter offset ils_t0 in [0,1).  The reference draws it from owl's
// LCG<4>(pixelID, accumID) (deviceCode.cpp:12,354,386), which is not in the
// reference tree; the oracle and the kernels use a documented hash of
// (pixel, accumID, draw) instead.
inline float jitter_hash(uint32_t pixel, uint32_t accum_id, uint32_t draw) {
  uint32_t h = pcg_hash(pixel ^ pcg_hash(accum_id ^ pcg_hash(draw)));
  return (float)(h >> 8) * (1.0f / 16777216.0f);
}

inline float jitter_value(const Params& p, uint32_t pixel, uint32_t draw) {
  if (p.jitter_mode == JITTER_CONST) return p.jitter_value;
  if (p.jitter_mode == JITTER_HASH) return jitter_hash(pixel, (uint32_t)p.accum_id, draw);
  return 0.0f;
}

// ---------------------------------------------------------------- geometry

// generateRay (deviceCode.cpp:94-107): dir = normalize(dir_00 + su*du + sv*dv)
// with su = x + .5, sv = y + .5, then every |component| < 1e-5 set to +1e-5.
template <class R> inline void generate_ray(const Camera& c, int x, int y, R org[3], R dir[3]) {
  R su = R((float)x + 0.5f), sv = R((float)y + 0.5f);
  for (int a = 0; a < 3; ++a) {
    org[a] = R(c.org[a]);
    dir[a] = std::fma(sv, R(c.dir_dv[a]), std::fma(su, R(c.dir_du[a]), R(c.dir_00[a])));
  }
  R len2 = std::fma(dir[2], dir[2], std::fma(dir[1], dir[1], dir[0] * dir[0]));
  R inv = R(1) / std::sqrt(len2);
  for (int a = 0; a < 3; ++a) {
    dir[a] = dir[a] * inv;
    if (std::fabs(dir[a]) < R(1e-5f)) dir[a] = R(1e-5f);
  }
}

// Slab test (deviceCode.cpp:41-57).
template <class R>
inline bool slab(const R org[3], const R dir[3], const float lo[3], const float hi[3], R tmin, R tmax,
                 R& t0, R& t1) {
  R nr[3], fr[3];
  for (int a = 0; a < 3; ++a) {
    R l = (R(lo[a]) - org[a]) / dir[a];
    R h = (R(hi[a]) - org[a]) / dir[a];
    nr[a] = std::fmin(l, h);
    fr[a] = std::fmax(l, h);
  }
  t0 = std::fmax(tmin, std::fmax(std::fmax(nr[0], nr[1]), nr[2]));
  t1 = std::fmin(tmax, std::fmin(std::fmin(fr[0], fr[1]), fr[2]));
  return t0 < t1;
}

// firstSampleT (deviceCode.cpp:245-254): first point of the global lattice
// dt*(ils + k) at or after `lower`.
template <class R> inline R first_sample_t(R lower, R dt, R ils) {
  R n = std::floor((lower - dt * ils) / dt);
  R t = dt * (ils + n);
  if (t < lower) t = t + dt;
  return t;
}

// ---------------------------------------------------------------- bricks

struct BrickView {
  const float* voxels;  // x-fastest, n[0]*n[1]*n[2]
  int n[3];             // voxelRange size
  float lo[3];          // voxelRange.lower
  float space_lo[3], space_hi[3];
};

// Texel fetch with cudaAddressModeClamp (waikikiRenderer.cpp:753-755).
template <class R> inline R voxel(const BrickView& b, int x, int y, int z) {
  x = std::min(std::max(x, 0), b.n[0] - 1);
  y = std::min(std::max(y, 0), b.n[1] - 1);
  z = std::min(std::max(z, 0), b.n[2] - 1);
  return R(b.voxels[((size_t)z * b.n[1] + y) * b.n[0] + x]);
}

// The seven taps of integrateBrick (deviceCode.cpp:278-288): the value at u
// and the central differences at u +- 1/2 along each axis.  Texture filtering
// follows CUDA's linear filter on texel coordinate xB = tc*N - 1/2 with
// i = floor(xB), w = xB - i, here with exact fp32 weights.
template <class R> struct Stencil {
  R value;
  R grad[3];
};

template <class R> inline Stencil<R> stencil(const BrickView& b, const R u[3]) {
  R fm[3], f[3], fc[3], g[3];
  int i[3], c[3];
  bool hi[3];
  for (int a = 0; a < 3; ++a) {
    R m = u[a] - R(0.5);
    fm[a] = std::floor(m);
    f[a] = m - fm[a];
    fc[a] = std::floor(u[a]);
    g[a] = u[a] - fc[a];
    i[a] = to_int(fm[a]);
    c[a] = to_int(fc[a]);
    hi[a] = (fc[a] != fm[a]);  // floor(u) == floor(u - 1/2) + 1
  }
  auto V = [&](int x, int y, int z) { return voxel<R>(b, x, y, z); };
  // x taps: columns x = i+k, bilinear in (y: weight g.y, then z: weight g.z)
  R X[3], Y[3], Z[3];
  for (int k = 0; k < 3; ++k) {
    int x = i[0] + k;
    X[k] = lerp(lerp(V(x, c[1], c[2]), V(x, c[1] + 1, c[2]), g[1]),
                lerp(V(x, c[1], c[2] + 1), V(x, c[1] + 1, c[2] + 1), g[1]), g[2]);
  }
  // y taps: rows y = i+k, bilinear in (x: weight g.x, then z: weight g.z)
  for (int k = 0; k < 3; ++k) {
    int y = i[1] + k;
    Y[k] = lerp(lerp(V(c[0], y, c[2]), V(c[0] + 1, y, c[2]), g[0]),
                lerp(V(c[0], y, c[2] + 1), V(c[0] + 1, y, c[2] + 1), g[0]), g[2]);
  }
  // z taps: slices z = i+k, bilinear in (x: weight g.x, then y: weight g.y)
  for (int k = 0; k < 3; ++k) {
    int z = i[2] + k;
    Z[k] = lerp(lerp(V(c[0], c[1], z), V(c[0] + 1, c[1], z), g[0]),
                lerp(V(c[0], c[1] + 1, z), V(c[0] + 1, c[1] + 1, z), g[0]), g[1]);
  }
  Stencil<R> s;
  s.value = hi[0] ? lerp(X[1], X[2], g[0]) : lerp(X[0], X[1], g[0]);
  s.grad[0] = lerp(X[1], X[2], f[0]) - lerp(X[0], X[1], f[0]);
  s.grad[1] = lerp(Y[1], Y[2], f[1]) - lerp(Y[0], Y[1], f[1]);
  s.grad[2] = lerp(Z[1], Z[2], f[2]) - lerp(Z[0], Z[1], f[2]);
  return s;
}

// tex1D on the transfer function (waikikiRenderer.cpp:990-1008): linear,
// normalized coordinates, border colour 0.  v is used raw as the coordinate
// (deviceCode.cpp:289).
template <class R> inline void tf_lookup(const float* tf, int n, R v, R out[4]) {
  R xb = v * R(n) - R(0.5);
  R fl = std::floor(xb);
  R w = xb - fl;
  int i = to_int(fl);
  for (int ch = 0; ch < 4; ++ch) {
    R e0 = (i >= 0 && i < n) ? R(tf[(size_t)i * 4 + ch]) : R(0);
    R e1 = (i + 1 >= 0 && i + 1 < n) ? R(tf[(size_t)(i + 1) * 4 + ch]) : R(0);
    out[ch] = lerp(e0, e1, w);
  }
}

// Gradient shading factor .1 + .9*|N.d|, N = g/|g + 1e-4| (deviceCode.cpp:285,294).
template <class R> inline R shade_factor(const R g[3], const R dir[3]) {
  R e0 = g[0] + R(1e-4f), e1 = g[1] + R(1e-4f), e2 = g[2] + R(1e-4f);
  R len = std::sqrt(std::fma(e2, e2, std::fma(e1, e1, e0 * e0)));
  R gd = std::fma(g[2], dir[2], std::fma(g[1], dir[1], g[0] * dir[0]));
  return std::fma(R(0.9f), std::fabs(gd / len), R(0.1f));
}

// integrateBrick (deviceCode.cpp:256-298) over [t0, t1).  Returns the number
// of loop-body executions (samples).
template <class R>
inline uint64_t march(const BrickView& b, const float* tf, int n_tf, const R org[3], const R dir[3], R t0, R t1,
                      R ils, R dt, R et, R color[4]) {
  // Iteration cap (not in the reference): twice the lattice points plus 16;
  // it only binds when t + dt rounds back to t for huge ray parameters.
  const float span = (float)(t1 - t0) / (float)dt;
  const uint64_t cap = span < 1e8f ? (uint64_t)(uint32_t)(span * 2.0f) + 16u : 200000016u;
  uint64_t n = 0;
  for (R t = first_sample_t(t0, dt, ils); t < t1 && color[3] < et && n < cap; t = t + dt) {
    ++n;
    R u[3];
    for (int a = 0; a < 3; ++a) u[a] = std::fma(t, dir[a], org[a]) - R(b.lo[a]);
    Stencil<R> s = stencil(b, u);
    R shade = shade_factor(s.grad, dir);
    R c[4];
    tf_lookup(tf, n_tf, s.value, c);
    R oma = R(1) - color[3];
    R s1 = oma * c[3];
    color[0] = std::fma(s1 * c[0], shade, color[0]);
    color[1] = std::fma(s1 * c[1], shade, color[1]);
    color[2] = std::fma(s1 * c[2], shade, color[2]);
    color[3] = std::fma(oma, c[3], color[3]);
  }
  return n;
}

// temperature_to_rgb (deviceCode.cpp:300-314).
template <class R> inline R saturate(R x) { return std::fmin(std::fmax(x, R(0)), R(1)); }
template <class R> inline void heat_color(R t, R out[3]) {
  R K = R(4.0f / 6.0f);
  R h = K - K * t;
  R v = R(0.5f) + R(0.5f) * t;
  R s = saturate(h) * R(6);
  out[0] = v * saturate(std::fabs(s - R(3)) - R(1));
  out[1] = v * saturate(R(2) - std::fabs(s - R(2)));
  out[2] = v * saturate(R(2) - std::fabs(s - R(4)));
}

// ---------------------------------------------------------------- frame

struct Schedule {
  int n_ranks;
  const int* rank_order;   // [n_ranks] front to back (IceT composite order)
  const int* rank_start;   // [n_ranks+1] CSR offsets, indexed by rank id
  const int* rank_bricks;  // bricks of each rank in front-to-back order
};

template <class R> struct Outputs {
  uint32_t* fb;          // [H*W] RGBA8
  R* final_rgba;         // [H*W*4] composite before quantization (fp32 mode)
  R* rank_images;        // [n_ranks*H*W*4] by rank id, after the output stage
  float* rank_depth;     // [n_ranks*H*W]
  R* accum;              // [n_ranks*H*W*4] progressive accumulation, in/out
  uint32_t* pixel_samples;  // [H*W] samples per pixel over all ranks
  uint64_t* samples;     // total samples over the rows rendered
};

// The IceT ordered BLEND of one rank image under the composite so far
// (waikikiRenderer.cpp:1042-1077): premultiplied "over" in fp32 (one fused
// multiply-add per channel), or IceT's RGBA8 form (quantise the rank image,
// blend in 8 bits with rounding).
template <class R>
inline void blend_over(int mode, const R img[4], R comp[4], uint32_t comp8[4]) {
  if (mode == COMPOSITE_UBYTE) {
    uint32_t q[4] = {quantize8(img[0]), quantize8(img[1]), quantize8(img[2]), quantize8(img[3])};
    uint32_t f = 255u - comp8[3];
    for (int ch = 0; ch < 4; ++ch) comp8[ch] = std::min(255u, comp8[ch] + (q[ch] * f + 127u) / 255u);
  } else {
    R oma = R(1) - comp[3];
    for (int ch = 0; ch < 4; ++ch) comp[ch] = std::fma(oma, img[ch], comp[ch]);
  }
}

// The same for an RGBA8 rank image (the blend of IceT's RGBA_UBYTE images).
inline void blend_over_rgba8(uint32_t q, uint32_t comp8[4]) {
  const uint32_t f = 255u - comp8[3];
  for (int ch = 0; ch < 4; ++ch) comp8[ch] = std::min(255u, comp8[ch] + (((q >> (8 * ch)) & 255u) * f + 127u) / 255u);
}

// One pixel: every virtual rank marches its own bricks (with its own early
// termination, as each MPI rank does in the reference), runs renderFrame's
// output stage, and the rank images are blended front to back.
template <class R>
inline uint64_t render_pixel(const BrickView* bricks, const float* tf, int n_tf, const Schedule& sch,
                             const Camera& cam, int W, int H, int x, int y, const Params& p, float max_depth,
                             const Outputs<R>& out) {
  const int pixel = x + W * y;
  const size_t npx = (size_t)W * H;
  const R dt = R(p.dt), et = R(p.et_alpha);
  const int spp = p.spp;
  bool in_island = true;
  if (p.num_islands > 1) {
    int tiles_x = (W + 15) / 16;
    int block = (x / 16) + tiles_x * (y / 16);
    in_island = (block % p.num_islands) == p.island_id;
  }
  R org[3], dir[3];
  generate_ray(cam, x, y, org, dir);
  R comp[4] = {0, 0, 0, 0};
  uint32_t comp8[4] = {0, 0, 0, 0};
  uint64_t total = 0;
  for (int k = 0; k < sch.n_ranks; ++k) {
    const int r = sch.rank_order[k];
    R acc[4] = {0, 0, 0, 0};
    R z = R(1);
    uint64_t ns = 0;
    if (in_island) {
      uint32_t draw = 0;
      for (int s = 0; s < spp; ++s) {
        R color[4] = {0, 0, 0, 0};
        R tmin = R(0);
        for (int j = sch.rank_start[r]; j < sch.rank_start[r + 1]; ++j) {
          const BrickView& b = bricks[sch.rank_bricks[j]];
          R t0, t1;
          if (!slab(org, dir, b.space_lo, b.space_hi, tmin, R(1e10f), t0, t1)) continue;
          R ils = R(jitter_value(p, (uint32_t)pixel, draw++));
          R tnear = (t0 > tmin ? t0 : R(0)) + tmin;
          z = std::fmin(z, tnear / R(max_depth));
          ns += march(b, tf, n_tf, org, dir, t0, t1, ils, dt, et, color);
          tmin = t1 + R(1e-20f);
          if (!(color[3] < et)) break;
        }
        for (int ch = 0; ch < 4; ++ch) acc[ch] = acc[ch] + color[ch];
      }
    }
    if (p.heat_map) {
      R hc[3];
      heat_color(R((float)ns) * (R(p.heat_map_scale) / R((float)spp)), hc);
      for (int ch = 0; ch < 3; ++ch) acc[ch] = std::fma(R(0.5f), acc[ch], hc[ch]);
      acc[3] = std::fma(R(0.5f), acc[3], R(0.5f));
    }
    R* accum_px = out.accum ? out.accum + ((size_t)r * npx + pixel) * 4 : nullptr;
    if (p.accum_id > 0 && accum_px)
      for (int ch = 0; ch < 4; ++ch) acc[ch] = acc[ch] + accum_px[ch];
    if (p.accumulate && accum_px)
      for (int ch = 0; ch < 4; ++ch) accum_px[ch] = acc[ch];
    const R scale = R(1) / R((float)(p.accum_id + 1));
    for (int ch = 0; ch < 4; ++ch) acc[ch] = acc[ch] * scale;
    if (p.crosshair && (x == W / 2 || y == H / 2))
      for (int ch = 0; ch < 4; ++ch) acc[ch] = R(1) - acc[ch];
    const R inv_spp = R(1) / R((float)spp);
    R img[4];
    for (int ch = 0; ch < 4; ++ch) img[ch] = acc[ch] * inv_spp;
    if (out.rank_images)
      for (int ch = 0; ch < 4; ++ch) out.rank_images[((size_t)r * npx + pixel) * 4 + ch] = img[ch];
    if (out.rank_depth) out.rank_depth[(size_t)r * npx + pixel] = (float)z;
    blend_over(p.composite_mode, img, comp, comp8);
    total += ns;
  }
  if (out.final_rgba)
    for (int ch = 0; ch < 4; ++ch) out.final_rgba[(size_t)pixel * 4 + ch] = comp[ch];
  if (out.fb) {
    if (p.composite_mode == COMPOSITE_UBYTE)
      out.fb[pixel] = comp8[0] | (comp8[1] << 8) | (comp8[2] << 16) | (comp8[3] << 24);
    else
      out.fb[pixel] = pack_rgba(comp);
  }
  if (out.pixel_samples) out.pixel_samples[pixel] = (uint32_t)total;
  return total;
}

// ---------------------------------------------------------------- adjoint
//
// Reverse-mode derivative of one pixel's colour C (front-to-back composite of
// integrateBrick samples, single virtual rank, spp 1) with respect to the
// transfer-function table and the voxel densities.  Written as the textbook
// recursion over stored per-sample states, independent of the GPU's
// segment-parallel formulation:
//   rgb' = rgb + (1-a) alpha s c,  a' = a + (1-a) alpha
//   dL/dalpha = (1-a)(s g.c + gA'),  dL/dc = g (1-a) alpha s,
//   dL/ds = (1-a) alpha g.c,  gA = gA' (1-alpha) - alpha s g.c
// with g = dL/drgb (constant along the ray) and gA' the adjoint of alpha after
// the sample.  Early termination is treated as fixed (no derivative).

struct Grid {
  int lo[3];
  int dims[3];
};

template <class R>
inline void scatter_voxel(const BrickView& b, int x, int y, int z, R w, R* grid, const Grid& gr) {
  x = std::min(std::max(x, 0), b.n[0] - 1);
  y = std::min(std::max(y, 0), b.n[1] - 1);
  z = std::min(std::max(z, 0), b.n[2] - 1);
  const int gx = (int)b.lo[0] + x - gr.lo[0], gy = (int)b.lo[1] + y - gr.lo[1], gz = (int)b.lo[2] + z - gr.lo[2];
  if (gx < 0 || gy < 0 || gz < 0 || gx >= gr.dims[0] || gy >= gr.dims[1] || gz >= gr.dims[2]) return;
  R* dst = grid + ((size_t)gz * gr.dims[1] + gy) * gr.dims[0] + gx;
#ifdef _OPENMP
#pragma omp atomic
#endif
  *dst += w;
}

// Scatters w * (trilinear weights at texel coordinate (xb, yb, zb)).
template <class R>
inline void scatter_trilinear(const BrickView& b, R xb, R yb, R zb, R w, R* grid, const Grid& gr) {
  if (w == R(0)) return;
  const R fx = std::floor(xb), fy = std::floor(yb), fz = std::floor(zb);
  const R ax = xb - fx, ay = yb - fy, az = zb - fz;
  const int ix = to_int(fx), iy = to_int(fy), iz = to_int(fz);
  for (int k = 0; k < 2; ++k)
    for (int j = 0; j < 2; ++j)
      for (int i = 0; i < 2; ++i) {
        const R wt = (i ? ax : R(1) - ax) * (j ? ay : R(1) - ay) * (k ? az : R(1) - az);
        scatter_voxel(b, ix + i, iy + j, iz + k, w * wt, grid, gr);
      }
}

// d(value)/d(voxels) * dv and d(gradient)/d(voxels) . dg for the seven taps.
template <class R>
inline void stencil_backward(const BrickView& b, const R u[3], R dv, const R dg[3], R* grid, const Grid& gr) {
  scatter_trilinear(b, u[0], u[1], u[2], dv, grid, gr);
  const R h = R(0.5);
  scatter_trilinear(b, u[0] + h, u[1], u[2], dg[0], grid, gr);
  scatter_trilinear(b, u[0] - h, u[1], u[2], -dg[0], grid, gr);
  scatter_trilinear(b, u[0], u[1] + h, u[2], dg[1], grid, gr);
  scatter_trilinear(b, u[0], u[1] - h, u[2], -dg[1], grid, gr);
  scatter_trilinear(b, u[0], u[1], u[2] + h, dg[2], grid, gr);
  scatter_trilinear(b, u[0], u[1], u[2] - h, -dg[2], grid, gr);
}

// The lookup and its backward on a given segment i (entries i, i+1) and the
// shading with a given sign of N.d: the branch the float32 forward took at a
// sample, evaluated in R (w may then leave [0, 1] by a rounding, the
// continuous extension of that branch).
template <class R> inline void tf_lookup_at(const float* tf, int n, R v, int i, R out[4]) {
  const R w = v * R(n) - R(0.5) - R(i);
  for (int ch = 0; ch < 4; ++ch) {
    R e0 = (i >= 0 && i < n) ? R(tf[(size_t)i * 4 + ch]) : R(0);
    R e1 = (i + 1 >= 0 && i + 1 < n) ? R(tf[(size_t)(i + 1) * 4 + ch]) : R(0);
    out[ch] = lerp(e0, e1, w);
  }
}

template <class R> inline R tf_backward_at(const float* tf, int n, R v, int i, const R dch[4], R* dtf) {
  const R w = v * R(n) - R(0.5) - R(i);
  R dv = 0;
  for (int ch = 0; ch < 4; ++ch) {
    R e0 = (i >= 0 && i < n) ? R(tf[(size_t)i * 4 + ch]) : R(0);
    R e1 = (i + 1 >= 0 && i + 1 < n) ? R(tf[(size_t)(i + 1) * 4 + ch]) : R(0);
    if (i >= 0 && i < n) {
#ifdef _OPENMP
#pragma omp atomic
#endif
      dtf[(size_t)i * 4 + ch] += (R(1) - w) * dch[ch];
    }
    if (i + 1 >= 0 && i + 1 < n) {
#ifdef _OPENMP
#pragma omp atomic
#endif
      dtf[(size_t)(i + 1) * 4 + ch] += w * dch[ch];
    }
    dv += dch[ch] * (e1 - e0) * R(n);
  }
  return dv;
}

template <class R> inline R shade_factor_signed(const R g[3], const R dir[3], int sgn) {
  R e0 = g[0] + R(1e-4f), e1 = g[1] + R(1e-4f), e2 = g[2] + R(1e-4f);
  R len = std::sqrt(std::fma(e2, e2, std::fma(e1, e1, e0 * e0)));
  R gd = std::fma(g[2], dir[2], std::fma(g[1], dir[1], g[0] * dir[0]));
  return std::fma(R(0.9f), R(sgn) * (gd / len), R(0.1f));
}

template <class R> inline void shade_backward_signed(const R g[3], const R dir[3], R ds, int sgn, R dg[3]) {
  R e[3] = {g[0] + R(1e-4f), g[1] + R(1e-4f), g[2] + R(1e-4f)};
  R len = std::sqrt(e[0] * e[0] + e[1] * e[1] + e[2] * e[2]);
  R gd = g[0] * dir[0] + g[1] * dir[1] + g[2] * dir[2];
  R k = ds * R(0.9f) * R(sgn);
  for (int a = 0; a < 3; ++a) dg[a] = k * (dir[a] / len - gd * e[a] / (len * len * len));
}

struct SampleRec {
  int brick;
  double t;
  double a;  // alpha before the sample
  int seg;   // the float32 forward's transfer-function segment
  int sgn;   // and its sign of N.d (shading)
};

// Adjoint of one pixel; returns the number of samples.
template <class R>
inline uint64_t adjoint_pixel(const BrickView* bricks, const float* tf, int n_tf, const Schedule& sch,
                              const Camera& cam, int W, int x, int y, const Params& p, const R dl[4], R* dtf,
                              R* dgrid, const Grid& gr) {
  const int pixel = x + W * y;
  // The sample set is the float32 forward's, the rendered image's: which
  // samples are taken, at which t, and where the ray terminates (the walk of
  // render_pixel for one rank); so are the branches of each sample's
  // piecewise pieces, the transfer-function segment and the sign of N.d in
  // the shading.  An R = double forward would decide some of these
  // differently (a sample at a brick exit where the step is not exact in
  // float, the sample that crosses the termination threshold, a value within
  // a rounding of a transfer-function knot, N.d within a rounding of 0), and
  // then differentiate another function than the image's.
  std::vector<SampleRec> recs;
  {
    const float dt = p.dt, et = p.et_alpha;
    float org[3], dir[3];
    generate_ray(cam, x, y, org, dir);
    float color[4] = {0.f, 0.f, 0.f, 0.f};
    float tmin = 0.f;
    uint32_t draw = 0;
    const int r = sch.rank_order[0];
    for (int j = sch.rank_start[r]; j < sch.rank_start[r + 1]; ++j) {
      const int bi = sch.rank_bricks[j];
      const BrickView& b = bricks[bi];
      float t0, t1;
      if (!slab(org, dir, b.space_lo, b.space_hi, tmin, 1e10f, t0, t1)) continue;
      const float ils = jitter_value(p, (uint32_t)pixel, draw++);
      const float span = (t1 - t0) / dt;
      const uint64_t cap = span < 1e8f ? (uint64_t)(uint32_t)(span * 2.0f) + 16u : 200000016u;
      uint64_t n = 0;
      for (float t = first_sample_t(t0, dt, ils); t < t1 && color[3] < et && n < cap; t = t + dt) {
        ++n;
        float u[3];
        for (int a = 0; a < 3; ++a) u[a] = std::fma(t, dir[a], org[a]) - b.lo[a];
        Stencil<float> s = stencil(b, u);
        const float shade = shade_factor(s.grad, dir);
        float c[4];
        tf_lookup(tf, n_tf, s.value, c);
        const int seg = to_int(std::floor(s.value * (float)n_tf - 0.5f));
        const float gd = std::fma(s.grad[2], dir[2], std::fma(s.grad[1], dir[1], s.grad[0] * dir[0]));
        recs.push_back(SampleRec{bi, (double)t, 0.0, seg, gd > 0.f ? 1 : (gd < 0.f ? -1 : 0)});
        const float oma = 1.0f - color[3];
        const float s1 = oma * c[3];
        color[0] = std::fma(s1 * c[0], shade, color[0]);
        color[1] = std::fma(s1 * c[1], shade, color[1]);
        color[2] = std::fma(s1 * c[2], shade, color[2]);
        color[3] = std::fma(oma, c[3], color[3]);
      }
      tmin = t1 + 1e-20f;
      if (!(color[3] < et)) break;
    }
  }
  // the alpha before each sample, composited in R along that set
  R org[3], dir[3];
  generate_ray(cam, x, y, org, dir);
  {
    R alpha = R(0);
    for (SampleRec& rec : recs) {
      const BrickView& b = bricks[rec.brick];
      const R t = R(rec.t);
      R u[3];
      for (int ax = 0; ax < 3; ++ax) u[ax] = std::fma(t, dir[ax], org[ax]) - R(b.lo[ax]);
      Stencil<R> s = stencil(b, u);
      R c[4];
      tf_lookup_at(tf, n_tf, s.value, rec.seg, c);
      rec.a = (double)alpha;
      alpha = std::fma(R(1) - alpha, c[3], alpha);
    }
  }
  R gA = dl[3];
  for (size_t k = recs.size(); k-- > 0;) {
    const BrickView& b = bricks[recs[k].brick];
    const R t = R(recs[k].t), a = R(recs[k].a);
    R u[3];
    for (int ax = 0; ax < 3; ++ax) u[ax] = std::fma(t, dir[ax], org[ax]) - R(b.lo[ax]);
    Stencil<R> s = stencil(b, u);
    R shade = shade_factor_signed(s.grad, dir, recs[k].sgn);
    R c[4];
    tf_lookup_at(tf, n_tf, s.value, recs[k].seg, c);
    const R oma = R(1) - a;
    const R gc = dl[0] * c[0] + dl[1] * c[1] + dl[2] * c[2];
    R dch[4];
    for (int ch = 0; ch < 3; ++ch) dch[ch] = dl[ch] * oma * c[3] * shade;
    dch[3] = oma * (shade * gc + gA);
    const R ds = oma * c[3] * gc;
    gA = gA * (R(1) - c[3]) - c[3] * shade * gc;
    const R dv = tf_backward_at(tf, n_tf, s.value, recs[k].seg, dch, dtf);
    R dg[3];
    shade_backward_signed(s.grad, dir, ds, recs[k].sgn, dg);
    stencil_backward(b, u, dv, dg, dgrid, gr);
  }
  return recs.size();
}

// ---------------------------------------------------------------- layout

// chopSuey VolumeSplitter (chopSuey.cpp:245-323): repeatedly split the domain
// with the largest space volume at the middle of its longest cell axis; voxel
// ranges carry a one-sided upper ghost layer, min(cell.hi + 1, dims).
// Returns false when the requested count cannot be reached (the reference
// recursion would not terminate).
inline bool chopsuey_split(const int dims[3], unsigned n_desired, std::vector<BrickDesc>& out) {
  BrickDesc root{};
  for (int a = 0; a < 3; ++a) {
    root.cell_lo[a] = 0;
    root.cell_hi[a] = dims[a];
    root.voxel_lo[a] = 0;
    root.voxel_hi[a] = dims[a] + 1;
    root.space_lo[a] = 0.f;
    root.space_hi[a] = (float)dims[a];
  }
  std::vector<BrickDesc> cl{root};
  size_t guard = 0;
  do {
    if (++guard > (size_t)1 << 24) return false;
    unsigned pick = 0;
    float max_vol = 0.f;
    for (unsigned k = 0; k < cl.size(); ++k) {
      float sx = cl[k].space_hi[0] - cl[k].space_lo[0];
      float sy = cl[k].space_hi[1] - cl[k].space_lo[1];
      float sz = cl[k].space_hi[2] - cl[k].space_lo[2];
      float vol = sx * sy * sz;
      if (vol > max_vol) {
        pick = k;
        max_vol = vol;
      }
    }
    BrickDesc d = cl[pick];
    cl.erase(cl.begin() + pick);
    int size[3] = {d.cell_hi[0] - d.cell_lo[0], d.cell_hi[1] - d.cell_lo[1], d.cell_hi[2] - d.cell_lo[2]};
    int axis = 0;
    if (size[1] > size[0] && size[1] >= size[2])
      axis = 1;
    else if (size[2] > size[0] && size[2] >= size[1])
      axis = 2;
    int plane = (int)((float)d.cell_lo[axis] + (float)size[axis] * 0.5f);
    BrickDesc L = d, Rb = d;
    L.cell_hi[axis] = plane;
    Rb.cell_lo[axis] = plane;
    for (BrickDesc* h : {&L, &Rb}) {
      for (int a = 0; a < 3; ++a) {
        h->voxel_lo[a] = h->cell_lo[a];
        h->voxel_hi[a] = std::min(h->cell_hi[a] + 1, dims[a]);
        h->space_lo[a] = (float)h->cell_lo[a];
        h->space_hi[a] = (float)h->cell_hi[a];
      }
      h->value_lo = 0.f;
      h->value_hi = 0.f;
    }
    auto cells = [](const BrickDesc& h) {
      return (long long)(h.cell_hi[0] - h.cell_lo[0]) * (h.cell_hi[1] - h.cell_lo[1]) * (h.cell_hi[2] - h.cell_lo[2]);
    };
    if (cells(L) > 0) cl.push_back(L);
    if (cells(Rb) > 0) cl.push_back(Rb);
  } while (cl.size() < n_desired);
  out = cl;
  return true;
}

// ---------------------------------------------------------------- ordering

struct KDNode {
  int axis;
  float plane;
  int child1, child2;  // ~rank for leaves, INT_MAX when unset
};

// Partitioner::partitionKD (waikikiRenderer.cpp:150-270): assign clusters to
// ranks by middle splits of the cluster bounds, centroid side test.
inline bool partition_kd(const float* boxes, int n, int n_ranks, std::vector<int>& cluster_rank,
                         std::vector<KDNode>& kd) {
  struct Group {
    float lo[3], hi[3];
    std::vector<int> ids;
    int node;
  };
  auto empty_box = [](Group& g) {
    for (int a = 0; a < 3; ++a) {
      g.lo[a] = 1e30f;
      g.hi[a] = -1e30f;
    }
  };
  auto extend = [&](Group& g, int id) {
    for (int a = 0; a < 3; ++a) {
      g.lo[a] = std::min(g.lo[a], boxes[id * 6 + a]);
      g.hi[a] = std::max(g.hi[a], boxes[id * 6 + 3 + a]);
    }
  };
  const size_t per_rank = (size_t)(n / n_ranks);
  Group all;
  empty_box(all);
  for (int k = 0; k < n; ++k) {
    extend(all, k);
    all.ids.push_back(k);
  }
  all.node = 0;
  std::vector<Group> open{all}, assigned;
  kd.clear();
  kd.push_back(KDNode{0, 0.f, INT_MAX, INT_MAX});
  size_t steps = 0;  // a split that makes no progress would repeat forever
  while (!open.empty()) {
    if (++steps > 64 * (size_t)n + 64) return false;
    unsigned pick = 0;
    size_t max_ids = 0;
    for (unsigned k = 0; k < open.size(); ++k)
      if (open[k].ids.size() > max_ids) {
        pick = k;
        max_ids = open[k].ids.size();
      }
    Group cs = open[pick];
    open.erase(open.begin() + pick);
    if (cs.ids.size() <= per_rank || assigned.size() == (size_t)n_ranks - 1) {
      int rank = (int)assigned.size();
      kd[cs.node].child1 = ~rank;
      kd[cs.node].child2 = ~rank;
      assigned.push_back(cs);
      if (assigned.size() == (size_t)n_ranks) {
        Group& last = assigned.back();
        while (!open.empty()) {
          for (int id : open[0].ids) last.ids.push_back(id);
          open.erase(open.begin());
        }
        break;
      }
      continue;
    }
    float size[3] = {cs.hi[0] - cs.lo[0], cs.hi[1] - cs.lo[1], cs.hi[2] - cs.lo[2]};
    int axis = 0;
    if (size[1] > size[0] && size[1] >= size[2])
      axis = 1;
    else if (size[2] > size[0] && size[2] >= size[1])
      axis = 2;
    float plane = cs.lo[axis] + size[axis] * 0.5f;
    Group L, Rg;
    empty_box(L);
    empty_box(Rg);
    for (int id : cs.ids) {
      float centroid = (boxes[id * 6 + axis] + boxes[id * 6 + 3 + axis]) / 2.f;
      if (centroid < plane) {
        extend(L, id);
        L.ids.push_back(id);
      } else {
        extend(Rg, id);
        Rg.ids.push_back(id);
      }
    }
    kd[cs.node].axis = axis;
    kd[cs.node].plane = plane;
    L.node = (int)kd.size();
    kd[cs.node].child1 = L.node;
    kd.push_back(KDNode{0, 0.f, INT_MAX, INT_MAX});
    open.push_back(L);
    Rg.node = (int)kd.size();
    kd[cs.node].child2 = Rg.node;
    kd.push_back(KDNode{0, 0.f, INT_MAX, INT_MAX});
    open.push_back(Rg);
  }
  cluster_rank.assign(n, -1);
  for (size_t r = 0; r < assigned.size(); ++r)
    for (int id : assigned[r].ids) cluster_rank[id] = (int)r;
  return true;
}

// Partitioner::computeCompositeOrder (waikikiRenderer.cpp:281-316): front-to-
// back walk of the KD tree from the camera position.
inline void composite_order_kd(const std::vector<KDNode>& kd, const float ref[3], std::vector<int>& order) {
  order.clear();
  if (kd.empty()) return;
  std::vector<int> stack{0};
  int addr = 0;
  while (!stack.empty()) {
    KDNode node = kd[addr];
    if (node.child1 < 0 && node.child2 < 0) {
      order.push_back(~node.child1);
      addr = stack.back();
      stack.pop_back();
    } else if (node.child1 == INT_MAX) {
      addr = stack.back();
      stack.pop_back();
    } else if (ref[node.axis] < node.plane) {
      addr = node.child1;
      stack.push_back(node.child2);
    } else {
      addr = node.child2;
      stack.push_back(node.child1);
    }
  }
}

// Front-to-back order of items (each a union of boxes) from actual faces: a
// separating-plane tree is built by taking, for axes 0..2 and candidate
// planes in ascending order, the first axis-aligned plane with every item on
// one side; the camera's side of each plane is visited first.  Items that no
// plane separates fall back to ascending squared distance of their bounds'
// centre from the camera.  (Replaces the reference's midplane KD test, which
// can mis-order bricks whose faces are not at the midplane.)
inline void visibility_order(const float* boxes, const int* item_of_box, int n_boxes, int n_items,
                             const float cam[3], std::vector<int>& order) {
  std::vector<float> ilo(n_items * 3, 1e30f), ihi(n_items * 3, -1e30f);
  std::vector<int> has(n_items, 0);
  for (int b = 0; b < n_boxes; ++b) {
    int it = item_of_box[b];
    has[it] = 1;
    for (int a = 0; a < 3; ++a) {
      ilo[it * 3 + a] = std::min(ilo[it * 3 + a], boxes[b * 6 + a]);
      ihi[it * 3 + a] = std::max(ihi[it * 3 + a], boxes[b * 6 + 3 + a]);
    }
  }
  order.clear();
  std::vector<int> all(n_items);
  for (int k = 0; k < n_items; ++k) all[k] = k;
  // recursive lambda via explicit stack of work lists
  struct Work {
    std::vector<int> items;
  };
  std::vector<Work> stack;
  stack.push_back(Work{all});
  while (!stack.empty()) {
    Work w = stack.back();
    stack.pop_back();
    if (w.items.size() <= 1) {
      for (int it : w.items) order.push_back(it);
      continue;
    }
    bool split = false;
    for (int a = 0; a < 3 && !split; ++a) {
      std::vector<float> cand;
      for (int it : w.items)
        if (has[it]) {
          cand.push_back(ilo[it * 3 + a]);
          cand.push_back(ihi[it * 3 + a]);
        }
      std::sort(cand.begin(), cand.end());
      cand.erase(std::unique(cand.begin(), cand.end()), cand.end());
      for (float p : cand) {
        std::vector<int> lo_side, hi_side;
        bool ok = true;
        for (int it : w.items) {
          if (!has[it] || ihi[it * 3 + a] <= p)
            lo_side.push_back(it);
          else if (ilo[it * 3 + a] >= p)
            hi_side.push_back(it);
          else {
            ok = false;
            break;
          }
        }
        if (!ok || lo_side.empty() || hi_side.empty()) continue;
        // stack: push the far side first so the near side pops first
        if (cam[a] < p) {
          stack.push_back(Work{hi_side});
          stack.push_back(Work{lo_side});
        } else {
          stack.push_back(Work{lo_side});
          stack.push_back(Work{hi_side});
        }
        split = true;
        break;
      }
    }
    if (!split) {
      std::vector<std::pair<float, int>> d;
      for (int it : w.items) {
        float s = 0.f;
        for (int a = 0; a < 3; ++a) {
          float c = has[it] ? (ilo[it * 3 + a] + ihi[it * 3 + a]) * 0.5f : cam[a];
          s += (c - cam[a]) * (c - cam[a]);
        }
        d.push_back({s, it});
      }
      std::stable_sort(d.begin(), d.end(),
                       [](const std::pair<float, int>& l, const std::pair<float, int>& r) { return l.first < r.first; });
      for (auto& e : d) order.push_back(e.second);
    }
  }
}

// maxDepth as handleCameraEvent computes it (waikikiRenderer.cpp:858-859).
inline float max_depth(const float bounds_lo[3], const float bounds_hi[3], const float org[3]) {
  float c[3], s1 = 0.f, s2 = 0.f;
  for (int a = 0; a < 3; ++a) c[a] = (bounds_lo[a] + bounds_hi[a]) / 2.f;
  for (int a = 0; a < 3; ++a) {
    float q = c[a] + bounds_hi[a];
    s1 = s1 + q * q;
    float o = org[a] + c[a];
    s2 = s2 + o * o;
  }
  return std::sqrt(s2) + std::sqrt(s1);
}

}  // namespace aloha_oracle
