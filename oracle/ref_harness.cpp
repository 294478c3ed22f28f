// ref_harness.cpp -- runs the reference's own volume code on the CPU.
//
// TEST INFRASTRUCTURE ONLY: it pins the oracle restatement (aloha_oracle.hpp)
// to the reference.  Built by `make ref` from the reference sources where
// they lie (nothing of them is copied into this repository):
//   * deviceCode.cpp, compiled unchanged against ref_shim/ (the stand-ins of
//     OWL, OptiX and the CUDA runtime), gives renderFrame (340-421) with
//     generateRay (94-107), VolBrickIsect (207-239), firstSampleT (245-254)
//     and integrateBrick (256-298);
//   * the Partitioner of waikikiRenderer.cpp (126-338: partitionKD and
//     computeCompositeOrder), extracted by line range at build time into
//     _ref/partitioner.inc, because the rest of that file needs MPI, IceT,
//     OWL and Qt.
// This file plays the role of the OptiX runtime and of fakeOwl: it sets up
// LaunchParams and one rank's brick buffer the way Renderer does
// (waikikiRenderer.cpp:686-797, 1015-1028), launches the raygen once per
// pixel, emulates closest-hit traversal of the rank's bricks, and evaluates
// the texture fetches.
//
// Emulation choices (the reference leaves them to OptiX / the texture unit):
//   * traversal tests the rank's bricks in the order given (front to back);
//     a report is accepted when tmin <= t < the closest hit so far, and
//     optixGetRayTmax() returns that closest hit, as OptiX specifies for
//     intersection programs.  Equal hit distances keep the brick tested first
//     (OptiX leaves their order unspecified);
//   * tex3D / tex1D use exact fp32 filter weights (the texture unit uses
//     8-bit fractions) and lerp(a, b, w) = a + w*(b - a) along x, then y,
//     then z;
//   * the sample count of a pixel is the number of transfer-function fetches
//     (integrateBrick makes exactly one per loop iteration, line 289).
#include <cassert>
#include <climits>
#include <cmath>
#include <cstring>
#include <iostream>
#include <numeric>
#include <vector>

#include <omp.h>

#include "deviceCode.h"
#include "aloha_oracle.hpp"

namespace maui {

extern "C" {
LaunchParams optixLaunchParams;
}

void optix_raygen_renderFrame();
void optix_isect_VolBrickIsect();

// waikikiRenderer.cpp:120-123 (outside the extracted range)
inline int div_up(int a, int b) { return (a + b - 1) / b; }

#include "partitioner.inc"

}  // namespace maui

using owl::common::vec2i;
using owl::common::vec3f;

namespace {

constexpr OptixTraversableHandle kWorld = 1, kVolBricks = 2;

struct Volume3 {
  const float* data;
  int n[3];
};
struct Table1 {
  const float* rgba;
  int n;
};

// Scene of the current launch (set before the parallel pixel loop, read-only in it).
std::vector<Volume3> g_volumes;  // texture handle k >= 1 -> g_volumes[k - 1]
Table1 g_tf;                     // texture handle kTF
constexpr cudaTextureObject_t kTF = 1u << 20;
std::vector<int> g_test_order;   // local brick ids in traversal test order
maui::BrickGeom g_geom;
int g_width = 0, g_height = 0;
int g_jitter_mode = 0;
float g_jitter_value = 0.f;

struct Thread {
  int x = 0, y = 0;
  void* prd = nullptr;
  owl::Ray ray;
  float closest = 0.f;
  unsigned prim = 0;
  uint32_t samples = 0;
};
thread_local Thread t_state;

inline float lerp(float a, float b, float w) { return a + w * (b - a); }

}  // namespace

// ------------------------------------------------------ shim callbacks
float aloha_ref_tex3D(cudaTextureObject_t tex, float x, float y, float z) {
  const Volume3& v = g_volumes[tex - 1];
  const float c[3] = {x, y, z};
  int i[3];
  float w[3];
  for (int a = 0; a < 3; ++a) {
    // texel coordinate; beyond [-1, n] every tap clamps to an edge voxel
    const float xb = std::fmin(std::fmax(c[a] * (float)v.n[a] - 0.5f, -1.f), (float)v.n[a]);
    const float f = std::floor(xb);
    i[a] = (int)f;
    w[a] = xb - f;
  }
  auto at = [&](int dx, int dy, int dz) {
    const int xx = std::min(std::max(i[0] + dx, 0), v.n[0] - 1);
    const int yy = std::min(std::max(i[1] + dy, 0), v.n[1] - 1);
    const int zz = std::min(std::max(i[2] + dz, 0), v.n[2] - 1);
    return v.data[((size_t)zz * v.n[1] + yy) * v.n[0] + xx];
  };
  float yz[2][2];
  for (int dz = 0; dz < 2; ++dz)
    for (int dy = 0; dy < 2; ++dy) yz[dz][dy] = lerp(at(0, dy, dz), at(1, dy, dz), w[0]);
  const float z0 = lerp(yz[0][0], yz[0][1], w[1]);
  const float z1 = lerp(yz[1][0], yz[1][1], w[1]);
  return lerp(z0, z1, w[2]);
}

float4 aloha_ref_tex1D(cudaTextureObject_t tex, float x) {
  (void)tex;
  ++t_state.samples;
  const int n = g_tf.n;
  const float xb = std::fmin(std::fmax(x * (float)n - 0.5f, -2.f), (float)n + 1.f);
  const float f = std::floor(xb);
  const int i = (int)f;
  const float w = xb - f;
  float e[2][4];
  for (int k = 0; k < 2; ++k)
    for (int ch = 0; ch < 4; ++ch) e[k][ch] = (i + k >= 0 && i + k < n) ? g_tf.rgba[(i + k) * 4 + ch] : 0.f;
  return float4{lerp(e[0][0], e[1][0], w), lerp(e[0][1], e[1][1], w), lerp(e[0][2], e[1][2], w),
                lerp(e[0][3], e[1][3], w)};
}

long long aloha_ref_clock() { return 0; }

float owl::common::aloha_ref_jitter(unsigned pixel, unsigned accum_id, unsigned draw) {
  if (g_jitter_mode == 1) return g_jitter_value;
  if (g_jitter_mode == 2) return aloha_oracle::jitter_hash(pixel, accum_id, draw);
  return 0.f;
}

unsigned optixGetPrimitiveIndex() { return t_state.prim; }
float3 optixGetObjectRayOrigin() {
  const vec3f& o = t_state.ray.origin;
  return float3{o.x, o.y, o.z};
}
float3 optixGetObjectRayDirection() {
  const vec3f& d = t_state.ray.direction;
  return float3{d.x, d.y, d.z};
}
float optixGetRayTmin() { return t_state.ray.tmin; }
float optixGetRayTmax() { return t_state.closest; }
bool optixReportIntersection(float t, unsigned) {
  if (!(t >= t_state.ray.tmin && t < t_state.closest)) return false;
  t_state.closest = t;
  return true;
}
uint3 optixGetLaunchDimensions() { return uint3{(unsigned)g_width, (unsigned)g_height, 1u}; }

vec2i owl::getLaunchIndex() { return vec2i(t_state.x, t_state.y); }
vec2i owl::getLaunchDims() { return vec2i(g_width, g_height); }
void* owl::aloha_ref_prd() { return t_state.prd; }
const void* owl::aloha_ref_program_data() { return &g_geom; }

void owl::aloha_ref_trace(OptixTraversableHandle group, const Ray& ray, void* prd) {
  if (group != kVolBricks) return;  // the triangle world is empty in volume mode
  Thread& s = t_state;
  void* const saved_prd = s.prd;
  const Ray saved_ray = s.ray;
  s.prd = prd;
  s.ray = ray;
  s.closest = ray.tmax;
  for (int id : g_test_order) {
    s.prim = (unsigned)id;
    maui::optix_isect_VolBrickIsect();
  }
  s.prd = saved_prd;
  s.ray = saved_ray;
}

// ------------------------------------------------------------- C API
extern "C" {

// Rows [y0, y1) of one rank's frame through the reference raygen (pixel ids,
// and with them the jitter draws, are those of the whole width x height
// frame; only those rows of the outputs are written).  bricks: the rank's
// bricks as .vol headers (80 bytes each, in the rank's load order); voxels:
// their voxel ranges, x fastest; test_order: local brick indices front to
// back; tf: n_tf RGBA entries; cam: org, dir_00, dir_du, dir_dv.  accum: W*H
// float4 (read when accum_id > 0, always written, as renderFrame does).
// Outputs: fb (RGBA8), depth, per-pixel sample counts.
int ref_render_rank_rows(const aloha_oracle::BrickDesc* bricks, const float* const* voxels, int n_bricks,
                         const int* test_order, int n_test, const float* tf, int n_tf, const float* cam, int width,
                         int height, float dt, float max_depth, int spp, int accum_id, int jitter_mode,
                         float jitter_value, float* accum, uint32_t* fb, float* depth, uint32_t* samples, int y0,
                         int y1, int threads) {
  if (n_bricks < 0 || width < 1 || height < 1 || n_tf < 1 || spp < 1) return -1;
  if (y0 < 0 || y1 > height || y0 >= y1) return -1;
  std::vector<maui::VolBrick> vb(n_bricks);
  g_volumes.resize(n_bricks);
  for (int b = 0; b < n_bricks; ++b) {
    const aloha_oracle::BrickDesc& d = bricks[b];
    maui::VolBrick& v = vb[b];
    v.cellRange = owl::box3i{owl::vec3i(d.cell_lo[0], d.cell_lo[1], d.cell_lo[2]),
                             owl::vec3i(d.cell_hi[0], d.cell_hi[1], d.cell_hi[2])};
    v.voxelRange = owl::box3i{owl::vec3i(d.voxel_lo[0], d.voxel_lo[1], d.voxel_lo[2]),
                              owl::vec3i(d.voxel_hi[0], d.voxel_hi[1], d.voxel_hi[2])};
    v.spaceRange = owl::box3f{vec3f(d.space_lo[0], d.space_lo[1], d.space_lo[2]),
                              vec3f(d.space_hi[0], d.space_hi[1], d.space_hi[2])};
    v.valueRange = range1f(d.value_lo, d.value_hi);
    v.texture = (cudaTextureObject_t)(b + 1);
    g_volumes[b] = Volume3{voxels[b], {d.voxel_hi[0] - d.voxel_lo[0], d.voxel_hi[1] - d.voxel_lo[1],
                                       d.voxel_hi[2] - d.voxel_lo[2]}};
  }
  for (int k = 0; k < n_test; ++k)
    if (test_order[k] < 0 || test_order[k] >= n_bricks) return -2;
  g_test_order.assign(test_order, test_order + n_test);
  g_tf = Table1{tf, n_tf};
  g_geom.brickBuffer = vb.data();
  g_width = width;
  g_height = height;
  g_jitter_mode = jitter_mode;
  g_jitter_value = jitter_value;

  maui::LaunchParams& lp = maui::optixLaunchParams;
  std::memset(static_cast<void*>(&lp), 0, sizeof lp);
  lp.fbPointer = fb;
  lp.fbDepth = depth;
  lp.accumBuffer = reinterpret_cast<float4*>(accum);
  lp.accumID = accum_id;
  lp.islandID = 0;
  lp.numIslands = 1;
  lp.world = kWorld;
  lp.volBricks = kVolBricks;
  lp.brickBuffer = vb.data();
  lp.maxDepth = max_depth;
  lp.transferFunc.texture = kTF;
  lp.camera.org = vec3f(cam[0], cam[1], cam[2]);
  lp.camera.dir_00 = vec3f(cam[3], cam[4], cam[5]);
  lp.camera.dir_du = vec3f(cam[6], cam[7], cam[8]);
  lp.camera.dir_dv = vec3f(cam[9], cam[10], cam[11]);
  lp.render.dt = dt;
  lp.render.heatMapEnabled = 0;
  lp.render.heatMapScale = 0.f;
  lp.render.spp = spp;

#pragma omp parallel for schedule(dynamic, 1) num_threads(threads > 0 ? threads : omp_get_max_threads())
  for (int y = y0; y < y1; ++y) {
    for (int x = 0; x < width; ++x) {
      t_state.x = x;
      t_state.y = y;
      t_state.samples = 0;
      maui::optix_raygen_renderFrame();
      samples[(size_t)y * width + x] = t_state.samples;
    }
  }
  return 0;
}

// The whole frame.
int ref_render_rank(const aloha_oracle::BrickDesc* bricks, const float* const* voxels, int n_bricks,
                    const int* test_order, int n_test, const float* tf, int n_tf, const float* cam, int width,
                    int height, float dt, float max_depth, int spp, int accum_id, int jitter_mode,
                    float jitter_value, float* accum, uint32_t* fb, float* depth, uint32_t* samples, int threads) {
  return ref_render_rank_rows(bricks, voxels, n_bricks, test_order, n_test, tf, n_tf, cam, width, height, dt,
                              max_depth, spp, accum_id, jitter_mode, jitter_value, accum, fb, depth, samples, 0,
                              height, threads);
}

// partitionKD over n boxes (space ranges, lo xyz hi xyz) for n_ranks ranks,
// then computeCompositeOrder for each reference point: brick_rank[n],
// orders[n_points][n_ranks] (the order's length is returned; -1 on error).
int ref_partition(const float* boxes, int n, int n_ranks, const float* points, int n_points, int* brick_rank,
                  int* orders) {
  if (n < 1 || n_ranks < 1) return -1;
  std::vector<maui::Cluster> clusters(n);
  for (int i = 0; i < n; ++i) {
    const float* b = boxes + 6 * i;
    clusters[i].id = i;
    clusters[i].rank = -1;
    clusters[i].domain = owl::box3f{vec3f(b[0], b[1], b[2]), vec3f(b[3], b[4], b[5])};
  }
  maui::Partitioner p(clusters, n_ranks);
  p.partitionKD();
  for (int i = 0; i < n; ++i) brick_rank[i] = -1;
  for (int r = 0; r < n_ranks && r < (int)p.perRank.size(); ++r)
    for (int id : p.perRank[r]) brick_rank[id] = r;
  int len = 0;
  for (int k = 0; k < n_points; ++k) {
    p.computeCompositeOrder(vec3f(points[3 * k], points[3 * k + 1], points[3 * k + 2]));
    len = (int)p.compositeOrder.size();
    if (len > n_ranks) return -1;
    for (int j = 0; j < len; ++j) orders[k * n_ranks + j] = p.compositeOrder[j];
  }
  return len;
}

}  // extern "C"
