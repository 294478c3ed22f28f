// aloha_renderer.hpp -- header-only C++ drop-in for the reference's renderer
// host API, on top of the C ABI in aloha.h.
//
// Mirrors maui::mpi::DistributedRenderer (DistributedRenderer.h:29-71) and
// maui::Renderer (waikikiRenderer.h:28-118) for the volume path:
// setCamera / resize / screenShot / setColorMap queue events, processEvents()
// replays them through the virtual handle*Event methods, and render(fb)
// processes the events and renders one frame into fb (host or device memory,
// width*height RGBA8).  One process drives one GPU; the MPI ranks of the
// reference become virtual ranks (bricks) inside the library, so there is no
// event broadcast and no IceT.  Errors throw aloha::Error carrying the
// library's status code.
#pragma once

#include <cstdint>
#include <cstdio>
#include <fstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "aloha.h"

namespace aloha {

struct vec2i {
  int x, y;
};
struct vec3f {
  float x, y, z;
};
struct vec4f {
  float x, y, z, w;
};

class Error : public std::runtime_error {
 public:
  Error(int code, const std::string& msg) : std::runtime_error(msg), code(code) {}
  int code;
};

// Reads a .vol file (chopSuey.cpp:325-349 layout, read like
// waikikiRenderer.cpp:597-665): all bricks' headers and voxels.
inline void read_vol(const std::string& path, std::vector<aloha_brick_desc>& descs,
                     std::vector<std::vector<float>>& voxels) {
  std::ifstream f(path, std::ios::binary);
  if (!f) throw Error(ALOHA_ERR_INVALID_ARGUMENT, "cannot open " + path);
  uint64_t n = 0;
  int32_t cell[6], voxel[6];
  float space[6];
  f.read((char*)&n, 8);
  f.read((char*)cell, sizeof cell);
  f.read((char*)voxel, sizeof voxel);
  f.read((char*)space, sizeof space);
  if (!f || n == 0 || n > 65536) throw Error(ALOHA_ERR_INVALID_ARGUMENT, "bad .vol header in " + path);
  descs.resize(n);
  voxels.resize(n);
  for (uint64_t i = 0; i < n; ++i) {
    aloha_brick_desc& d = descs[i];
    f.read((char*)&d, sizeof d);
    const long long nx = d.voxel_hi[0] - d.voxel_lo[0], ny = d.voxel_hi[1] - d.voxel_lo[1],
                    nz = d.voxel_hi[2] - d.voxel_lo[2];
    if (!f || nx <= 0 || ny <= 0 || nz <= 0) throw Error(ALOHA_ERR_INVALID_ARGUMENT, "bad brick header in " + path);
    voxels[i].resize((size_t)(nx * ny * nz));
    f.read((char*)voxels[i].data(), (std::streamsize)(voxels[i].size() * sizeof(float)));
    if (!f) throw Error(ALOHA_ERR_INVALID_ARGUMENT, "truncated brick data in " + path);
  }
}

// mpi::DistributedRenderer without MPI: events are queued and replayed in order.
class DistributedRenderer {
 public:
  virtual ~DistributedRenderer() = default;

  void setCamera(const vec3f& org, const vec3f& dir_00, const vec3f& dir_du, const vec3f& dir_dv) {
    Event e;
    e.type = Event::Camera;
    e.cam[0] = org;
    e.cam[1] = dir_00;
    e.cam[2] = dir_du;
    e.cam[3] = dir_dv;
    events_.push_back(e);
  }
  void resize(const vec2i& newSize) {
    Event e;
    e.type = Event::Resize;
    e.size = newSize;
    events_.push_back(e);
  }
  void screenShot(const std::string& baseName) {
    Event e;
    e.type = Event::ScreenShot;
    e.name = baseName;
    events_.push_back(e);
  }
  void setColorMap(const std::vector<vec4f>& newCM) {
    Event e;
    e.type = Event::ColorMap;
    e.cmap = newCM;
    events_.push_back(e);
  }

  virtual void handleCameraEvent(const vec3f& org, const vec3f& dir_00, const vec3f& dir_du, const vec3f& dir_dv) = 0;
  virtual void handleResizeEvent(const vec2i& newSize) = 0;
  virtual void handleScreenShotEvent(const std::string&) {}
  virtual void handleColorMapEvent(const std::vector<vec4f>&) {}

  void processEvents() {
    std::vector<Event> ev;
    ev.swap(events_);
    for (const Event& e : ev) {
      switch (e.type) {
        case Event::Camera: handleCameraEvent(e.cam[0], e.cam[1], e.cam[2], e.cam[3]); break;
        case Event::Resize: handleResizeEvent(e.size); break;
        case Event::ScreenShot: handleScreenShotEvent(e.name); break;
        case Event::ColorMap: handleColorMapEvent(e.cmap); break;
      }
    }
  }

 private:
  struct Event {
    enum Type { Camera, Resize, ScreenShot, ColorMap } type;
    vec3f cam[4];
    vec2i size{0, 0};
    std::string name;
    std::vector<vec4f> cmap;
  };
  std::vector<Event> events_;
};

// maui::Renderer for volumes on one GPU: the bricks of a .vol file become
// virtual ranks (partitionKD over `numRanks`, 0 = one rank per brick).
class Renderer : public DistributedRenderer {
 public:
  explicit Renderer(const std::string& volFile, int numRanks = 0, int device = 0) {
    check(aloha_create(device, &ctx_), nullptr);
    std::vector<aloha_brick_desc> descs;
    std::vector<std::vector<float>> vox;
    read_vol(volFile, descs, vox);
    std::vector<const float*> ptrs;
    for (auto& v : vox) ptrs.push_back(v.data());
    check(aloha_set_bricks(ctx_, descs.data(), ptrs.data(), (int)descs.size()), ctx_);
    if (numRanks > 0) check(aloha_set_ranks(ctx_, numRanks), ctx_);
    check(aloha_default_render_params(&params_), ctx_);
    check(aloha_set_render_params(ctx_, &params_), ctx_);
  }
  ~Renderer() override {
    if (ctx_) aloha_destroy(ctx_);
  }
  Renderer(const Renderer&) = delete;
  Renderer& operator=(const Renderer&) = delete;

  // Renderer::render (waikikiRenderer.cpp:1015-1080): events, then one frame.
  void render(uint32_t* fbPointer, void* stream = nullptr) {
    fb_ = fbPointer;
    processEvents();
    check(aloha_render(ctx_, 0, fbPointer, stream), ctx_);
    if (!pendingShot_.empty()) {
      writeScreenShot(pendingShot_);
      pendingShot_.clear();
    }
  }

  void handleCameraEvent(const vec3f& org, const vec3f& dir_00, const vec3f& dir_du, const vec3f& dir_dv) override {
    check(aloha_set_camera(ctx_, 0, &org.x, &dir_00.x, &dir_du.x, &dir_dv.x), ctx_);
    params_.accum_id = 0;  // accumID = 0 (waikikiRenderer.cpp:870)
    check(aloha_set_render_params(ctx_, &params_), ctx_);
  }
  void handleResizeEvent(const vec2i& newSize) override {
    check(aloha_resize(ctx_, 0, newSize.x, newSize.y), ctx_);
    size_ = newSize;
  }
  void handleColorMapEvent(const std::vector<vec4f>& newCM) override {
    check(aloha_set_transfer_function(ctx_, &newCM[0].x, (int)newCM.size()), ctx_);
  }
  // Written after the next frame: rows flipped, alpha forced to 255
  // (waikikiRenderer.cpp:922-943), as binary PPM (no image library).
  void handleScreenShotEvent(const std::string& baseName) override { pendingShot_ = baseName; }

  aloha_render_params& params() { return params_; }
  void applyParams() { check(aloha_set_render_params(ctx_, &params_), ctx_); }
  aloha_ctx* context() { return ctx_; }

 private:
  static void check(int rc, aloha_ctx* c) {
    if (rc != ALOHA_OK)
      throw Error(rc, std::string(aloha_status_string(rc)) + (c ? std::string(": ") + aloha_last_error(c) : ""));
  }
  void writeScreenShot(const std::string& base) {
    std::vector<uint32_t> px((size_t)size_.x * size_.y);
    // render() may have written device memory: let the library copy a fresh host frame
    check(aloha_render(ctx_, 0, px.data(), nullptr), ctx_);
    std::FILE* f = std::fopen((base + ".ppm").c_str(), "wb");
    if (!f) return;
    std::fprintf(f, "P6\n%d %d\n255\n", size_.x, size_.y);
    for (int y = size_.y - 1; y >= 0; --y)
      for (int x = 0; x < size_.x; ++x) {
        const uint32_t p = px[(size_t)y * size_.x + x];
        const unsigned char rgb[3] = {(unsigned char)(p & 255), (unsigned char)((p >> 8) & 255),
                                      (unsigned char)((p >> 16) & 255)};
        std::fwrite(rgb, 1, 3, f);
      }
    std::fclose(f);
  }

  aloha_ctx* ctx_ = nullptr;
  aloha_render_params params_{};
  uint32_t* fb_ = nullptr;
  vec2i size_{0, 0};
  std::string pendingShot_;
};

}  // namespace aloha
