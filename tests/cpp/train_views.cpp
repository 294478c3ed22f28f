// train_views.cpp -- the differentiable form through the C ABI from C++:
// bricks from a .vol file, one aloha_forward_views launch over several views
// into host images, then one aloha_backward_views call with host dL/dRGBA
// buffers into a host transfer-function gradient and a host density grid.
//
// usage: train_views file.vol tf.f32 n_tf k W H n_views cams.f32 dl.f32 img.f32 dtf.f32 dden.f32 nx ny nz
//   cams.f32: n_views x 12 floats (org, dir_00, dir_du, dir_dv); dl.f32: n_views x H x W x 4 floats.
//   Writes the images (n_views x H x W x 4), dL/dtf (n_tf x 4) and dL/ddensity (nz x ny x nx).
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "aloha_renderer.hpp"

namespace {

bool read_floats(const char* path, std::vector<float>& v) {
  std::FILE* f = std::fopen(path, "rb");
  if (!f) return false;
  const size_t got = std::fread(v.data(), sizeof(float), v.size(), f);
  std::fclose(f);
  return got == v.size();
}

bool write_floats(const char* path, const std::vector<float>& v) {
  std::FILE* f = std::fopen(path, "wb");
  if (!f) return false;
  const size_t put = std::fwrite(v.data(), sizeof(float), v.size(), f);
  std::fclose(f);
  return put == v.size();
}

void check(int rc, aloha_ctx* ctx) {
  if (rc != ALOHA_OK) throw aloha::Error(rc, ctx ? aloha_last_error(ctx) : aloha_status_string(rc));
}

}  // namespace

int main(int argc, char** argv) {
  if (argc != 16) {
    std::fprintf(stderr, "usage: %s file.vol tf.f32 n_tf k W H n_views cams.f32 dl.f32 img.f32 dtf.f32 dden.f32 "
                         "nx ny nz\n", argv[0]);
    return 2;
  }
  const int n_tf = std::atoi(argv[3]), k = std::atoi(argv[4]), W = std::atoi(argv[5]), H = std::atoi(argv[6]);
  const int n_views = std::atoi(argv[7]);
  const int dims[3] = {std::atoi(argv[13]), std::atoi(argv[14]), std::atoi(argv[15])};
  const size_t npx = (size_t)W * H, grid = (size_t)dims[0] * dims[1] * dims[2];
  std::vector<float> tf((size_t)n_tf * 4), cams((size_t)n_views * 12), dl((size_t)n_views * npx * 4);
  if (!read_floats(argv[2], tf) || !read_floats(argv[8], cams) || !read_floats(argv[9], dl)) return 3;
  aloha_ctx* ctx = nullptr;
  try {
    std::vector<aloha_brick_desc> descs;
    std::vector<std::vector<float>> voxels;
    aloha::read_vol(argv[1], descs, voxels);
    check(aloha_create(0, &ctx), nullptr);
    std::vector<const float*> vptr;
    for (const auto& v : voxels) vptr.push_back(v.data());
    check(aloha_set_bricks(ctx, descs.data(), vptr.data(), (int)descs.size()), ctx);
    check(aloha_set_transfer_function(ctx, tf.data(), n_tf), ctx);
    check(aloha_set_ranks(ctx, 1), ctx);
    std::vector<int> views(n_views);
    for (int v = 0; v < n_views; ++v) {
      const float* c = &cams[(size_t)v * 12];
      views[v] = v;
      check(aloha_set_camera(ctx, v, c, c + 3, c + 6, c + 9), ctx);
      check(aloha_resize(ctx, v, W, H), ctx);
    }
    std::vector<float> img((size_t)n_views * npx * 4);
    std::vector<float*> outs;
    std::vector<const float*> grads;
    for (int v = 0; v < n_views; ++v) {
      outs.push_back(&img[(size_t)v * npx * 4]);
      grads.push_back(&dl[(size_t)v * npx * 4]);
    }
    check(aloha_forward_views(ctx, n_views, views.data(), outs.data(), k, nullptr), ctx);
    std::vector<float> dtf((size_t)n_tf * 4, 0.f), dden(grid, 0.f);
    const int lo[3] = {0, 0, 0};
    check(aloha_backward_views(ctx, n_views, views.data(), grads.data(), dtf.data(), dden.data(), lo, dims, nullptr),
          ctx);
    aloha_destroy(ctx);
    ctx = nullptr;
    if (!write_floats(argv[10], img) || !write_floats(argv[11], dtf) || !write_floats(argv[12], dden)) return 4;
  } catch (const aloha::Error& e) {
    std::fprintf(stderr, "aloha error %d: %s\n", e.code, e.what());
    if (ctx) aloha_destroy(ctx);
    return 5;
  }
  return 0;
}
