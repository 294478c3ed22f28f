// render_vol.cpp -- drives the C++ drop-in renderer (include/aloha_renderer.hpp)
// the way the reference's viewer drives maui::Renderer: colour map, resize and
// camera events, then render(fb) into host memory.
//
// usage: render_vol file.vol tf.f32 n_tf out.u32 W H n_ranks org(3) dir_00(3) dir_du(3) dir_dv(3)
#include <cstdio>
#include <cstdlib>
#include <vector>

#include "aloha_renderer.hpp"

int main(int argc, char** argv) {
  if (argc != 20) {
    std::fprintf(stderr, "usage: %s file.vol tf.f32 n_tf out.u32 W H n_ranks org dir_00 dir_du dir_dv\n", argv[0]);
    return 2;
  }
  const int n_tf = std::atoi(argv[3]);
  const int W = std::atoi(argv[5]), H = std::atoi(argv[6]), ranks = std::atoi(argv[7]);
  std::vector<aloha::vec4f> cm(n_tf);
  std::FILE* f = std::fopen(argv[2], "rb");
  if (!f || std::fread(cm.data(), sizeof(aloha::vec4f), n_tf, f) != (size_t)n_tf) return 3;
  std::fclose(f);
  float c[12];
  for (int i = 0; i < 12; ++i) c[i] = (float)std::atof(argv[8 + i]);
  try {
    aloha::Renderer r(argv[1], ranks);
    r.setColorMap(cm);
    r.resize({W, H});
    r.setCamera({c[0], c[1], c[2]}, {c[3], c[4], c[5]}, {c[6], c[7], c[8]}, {c[9], c[10], c[11]});
    std::vector<uint32_t> fb((size_t)W * H);
    r.render(fb.data());
    std::FILE* o = std::fopen(argv[4], "wb");
    if (!o) return 4;
    std::fwrite(fb.data(), 4, fb.size(), o);
    std::fclose(o);
  } catch (const aloha::Error& e) {
    std::fprintf(stderr, "aloha error %d: %s\n", e.code, e.what());
    return 5;
  }
  return 0;
}
