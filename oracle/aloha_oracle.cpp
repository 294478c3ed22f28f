// aloha_oracle.cpp -- C ABI of the CPU oracle (ctypes-friendly).
//
// TEST INFRASTRUCTURE ONLY: loaded by tests/, __graft_entry__.smoke() and
// bench.py's CPU-baseline arm, never by the product library.  Built with
// -ffp-contract=off (see aloha_oracle.hpp for the evaluation order).
#include "aloha_oracle.hpp"

#include <atomic>
#include <vector>
#ifdef _OPENMP
#include <omp.h>
#endif

using namespace aloha_oracle;

namespace {

struct Scene {
  const BrickDesc* descs;
  const float* const* voxels;
  int n_bricks;
  const float* tf;
  int n_tf;
};

template <class R>
int render_rows(const Scene* sc, const Schedule* sch, const Camera* cam, int W, int H, const Params* p,
                float max_depth, const Outputs<R>* out, int row_begin, int row_end, int n_threads) {
  if (!sc || !sch || !cam || !p || !out || W <= 0 || H <= 0 || p->spp <= 0) return -1;
  std::vector<BrickView> views(sc->n_bricks);
  for (int b = 0; b < sc->n_bricks; ++b) {
    const BrickDesc& d = sc->descs[b];
    BrickView& v = views[b];
    v.voxels = sc->voxels[b];
    for (int a = 0; a < 3; ++a) {
      v.n[a] = d.voxel_hi[a] - d.voxel_lo[a];
      v.lo[a] = (float)d.voxel_lo[a];
      v.space_lo[a] = d.space_lo[a];
      v.space_hi[a] = d.space_hi[a];
      if (v.n[a] <= 0) return -2;
    }
  }
  if (row_begin < 0) row_begin = 0;
  if (row_end > H || row_end < 0) row_end = H;
  uint64_t total = 0;
#ifdef _OPENMP
  if (n_threads <= 0) n_threads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(n_threads) reduction(+ : total)
#endif
  for (int y = row_begin; y < row_end; ++y) {
    for (int x = 0; x < W; ++x)
      total += render_pixel<R>(views.data(), sc->tf, sc->n_tf, *sch, *cam, W, H, x, y, *p, max_depth, *out);
  }
  if (out->samples) *out->samples = total;
  return 0;
}

// Adjoint of the single-rank render: accumulates dL/dtf [n_tf*4] and dL/d
// density on the grid [dims z][y][x] starting at grid_lo, for dL/dRGBA per
// pixel.  Returns 0, or -1 on bad arguments.
template <class R>
int adjoint_rows(const Scene* sc, const Schedule* sch, const Camera* cam, int W, int H, const Params* p,
                 const R* dl, R* dtf, R* dgrid, const int* grid_lo, const int* grid_dims, int row_begin, int row_end,
                 int n_threads, uint64_t* samples) {
  if (!sc || !sch || !cam || !p || !dl || !dtf || !dgrid || W <= 0 || H <= 0 || sch->n_ranks != 1) return -1;
  std::vector<BrickView> views(sc->n_bricks);
  for (int b = 0; b < sc->n_bricks; ++b) {
    const BrickDesc& d = sc->descs[b];
    BrickView& v = views[b];
    v.voxels = sc->voxels[b];
    for (int a = 0; a < 3; ++a) {
      v.n[a] = d.voxel_hi[a] - d.voxel_lo[a];
      v.lo[a] = (float)d.voxel_lo[a];
      v.space_lo[a] = d.space_lo[a];
      v.space_hi[a] = d.space_hi[a];
    }
  }
  Grid gr;
  for (int a = 0; a < 3; ++a) {
    gr.lo[a] = grid_lo[a];
    gr.dims[a] = grid_dims[a];
  }
  if (row_begin < 0) row_begin = 0;
  if (row_end > H || row_end < 0) row_end = H;
  uint64_t total = 0;
#ifdef _OPENMP
  if (n_threads <= 0) n_threads = omp_get_max_threads();
#pragma omp parallel for schedule(dynamic, 1) num_threads(n_threads) reduction(+ : total)
#endif
  for (int y = row_begin; y < row_end; ++y)
    for (int x = 0; x < W; ++x)
      total += adjoint_pixel<R>(views.data(), sc->tf, sc->n_tf, *sch, *cam, W, x, y, *p, dl + ((size_t)y * W + x) * 4,
                                dtf, dgrid, gr);
  if (samples) *samples = total;
  return 0;
}

}  // namespace

extern "C" {

int ora_abi_version() { return 1; }

int ora_max_threads() {
#ifdef _OPENMP
  return omp_get_max_threads();
#else
  return 1;
#endif
}

int ora_render_f32(const Scene* sc, const Schedule* sch, const Camera* cam, int W, int H, const Params* p,
                   float max_depth, const Outputs<float>* out, int row_begin, int row_end, int n_threads) {
  return render_rows<float>(sc, sch, cam, W, H, p, max_depth, out, row_begin, row_end, n_threads);
}

int ora_render_f64(const Scene* sc, const Schedule* sch, const Camera* cam, int W, int H, const Params* p,
                   float max_depth, const Outputs<double>* out, int row_begin, int row_end, int n_threads) {
  return render_rows<double>(sc, sch, cam, W, H, p, max_depth, out, row_begin, row_end, n_threads);
}

int ora_adjoint_f64(const Scene* sc, const Schedule* sch, const Camera* cam, int W, int H, const Params* p,
                    const double* dl, double* dtf, double* dgrid, const int* grid_lo, const int* grid_dims,
                    int row_begin, int row_end, int n_threads, uint64_t* samples) {
  return adjoint_rows<double>(sc, sch, cam, W, H, p, dl, dtf, dgrid, grid_lo, grid_dims, row_begin, row_end,
                              n_threads, samples);
}

// chopSuey split: returns the number of bricks written, or -1.
int ora_chopsuey_split(const int* dims, int n_desired, BrickDesc* out, int max_out) {
  std::vector<BrickDesc> v;
  if (!chopsuey_split(dims, (unsigned)std::max(n_desired, 1), v)) return -1;
  if ((int)v.size() > max_out) return -1;
  for (size_t k = 0; k < v.size(); ++k) out[k] = v[k];
  return (int)v.size();
}

// partitionKD: boxes [n*6] (lo xyz, hi xyz); writes cluster_rank[n] and the
// kd nodes (axis, plane, child1, child2) as 4 int32 each (plane bit-cast).
int ora_partition_kd(const float* boxes, int n, int n_ranks, int* cluster_rank, int* kd_out, int max_nodes) {
  if (n <= 0 || n_ranks <= 0 || n_ranks > n) return -1;
  std::vector<int> cr;
  std::vector<KDNode> kd;
  if (!partition_kd(boxes, n, n_ranks, cr, kd)) return -1;
  if ((int)kd.size() > max_nodes) return -1;
  for (int k = 0; k < n; ++k) cluster_rank[k] = cr[k];
  for (size_t k = 0; k < kd.size(); ++k) {
    kd_out[k * 4 + 0] = kd[k].axis;
    std::memcpy(&kd_out[k * 4 + 1], &kd[k].plane, 4);
    kd_out[k * 4 + 2] = kd[k].child1;
    kd_out[k * 4 + 3] = kd[k].child2;
  }
  return (int)kd.size();
}

int ora_composite_order_kd(const int* kd_in, int n_nodes, const float* ref, int* order, int max_order) {
  std::vector<KDNode> kd(n_nodes);
  for (int k = 0; k < n_nodes; ++k) {
    kd[k].axis = kd_in[k * 4 + 0];
    std::memcpy(&kd[k].plane, &kd_in[k * 4 + 1], 4);
    kd[k].child1 = kd_in[k * 4 + 2];
    kd[k].child2 = kd_in[k * 4 + 3];
  }
  std::vector<int> o;
  composite_order_kd(kd, ref, o);
  if ((int)o.size() > max_order) return -1;
  for (size_t k = 0; k < o.size(); ++k) order[k] = o[k];
  return (int)o.size();
}

int ora_visibility_order(const float* boxes, const int* item_of_box, int n_boxes, int n_items, const float* cam,
                         int* order) {
  std::vector<int> o;
  visibility_order(boxes, item_of_box, n_boxes, n_items, cam, o);
  for (size_t k = 0; k < o.size(); ++k) order[k] = o[k];
  return (int)o.size();
}

float ora_max_depth(const float* lo, const float* hi, const float* org) { return max_depth(lo, hi, org); }

float ora_jitter_hash(uint32_t pixel, uint32_t accum_id, uint32_t draw) { return jitter_hash(pixel, accum_id, draw); }

// Single-sample probes used by the closed-form unit tests.
float ora_first_sample_t(float lower, float dt, float ils) { return first_sample_t<float>(lower, dt, ils); }

void ora_tf_lookup(const float* tf, int n, float v, float* out) { tf_lookup<float>(tf, n, v, out); }

// The ordered composite of n float rank images ([n][npx][4]) front to back
// in `order`, fp32 or RGBA8 blend, into RGBA8 pixels.
void ora_composite_over(const float* images, const int* order, int n, int npx, int mode, uint32_t* fb) {
  for (int px = 0; px < npx; ++px) {
    float comp[4] = {0.f, 0.f, 0.f, 0.f};
    uint32_t comp8[4] = {0u, 0u, 0u, 0u};
    for (int k = 0; k < n; ++k) blend_over(mode, images + ((size_t)order[k] * npx + px) * 4, comp, comp8);
    fb[px] = mode == COMPOSITE_UBYTE ? (comp8[0] | (comp8[1] << 8) | (comp8[2] << 16) | (comp8[3] << 24))
                                     : pack_rgba(comp);
  }
}

// The same for RGBA8 rank images ([n][npx] packed RGBA8).
void ora_composite_over_rgba8(const uint32_t* images, const int* order, int n, int npx, uint32_t* fb) {
  for (int px = 0; px < npx; ++px) {
    uint32_t comp8[4] = {0u, 0u, 0u, 0u};
    for (int k = 0; k < n; ++k) blend_over_rgba8(images[(size_t)order[k] * npx + px], comp8);
    fb[px] = comp8[0] | (comp8[1] << 8) | (comp8[2] << 16) | (comp8[3] << 24);
  }
}

void ora_stencil(const float* voxels, const int* n, const float* u, float* out4) {
  BrickView b{};
  b.voxels = voxels;
  for (int a = 0; a < 3; ++a) {
    b.n[a] = n[a];
    b.lo[a] = 0.f;
  }
  Stencil<float> s = stencil<float>(b, u);
  out4[0] = s.value;
  out4[1] = s.grad[0];
  out4[2] = s.grad[1];
  out4[3] = s.grad[2];
}

}  // extern "C"
