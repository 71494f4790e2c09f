// Test infrastructure: the reference library itself (src/renderer, compiled unmodified by
// oracle/Makefile `user-ref`) running the shader classes of tests/cpp/user_shaders.h on the
// scenes of tests/cpp/user_scene.h.  Writes the shader's framebuffer of every case --
// RGBA8 colour, FP32 depth, per-pixel drawPixel count -- to <outdir>/<case>_ref.bin, the
// fixtures tests/golden/make_user_golden.py hashes for the GPU test of the same shaders.
#include <cstdio>
#include <cstring>
#include <limits>
#include <string>
#include <vector>

#include "Renderer.h"  // the reference's umbrella header (src/renderer/Renderer.h)
#include "../tests/cpp/user_scene.h"
#include "../tests/cpp/user_shaders.h"

int main(int argc, char** argv) {
  if (argc < 2) {
    fprintf(stderr, "usage: %s <outdir>\n", argv[0]);
    return 1;
  }
  const std::string out = argv[1];
  const int w = 320, h = 240;
  std::vector<uint32_t> color((size_t)w * h), count((size_t)w * h);
  std::vector<float> depth((size_t)w * h);
  g_target.color = color.data();
  g_target.depth = depth.data();
  g_target.count = count.data();
  g_target.width = w;
  g_target.height = h;
  for (int k = 0; k < user_case_count(); ++k) {
    UserScene sc = user_scene(k);
    memcpy(g_mvp, sc.mvp, sizeof(g_mvp));
    std::fill(color.begin(), color.end(), 0u);
    std::fill(count.begin(), count.end(), 0u);
    std::fill(depth.begin(), depth.end(), std::numeric_limits<float>::infinity());
    swr::Rasterizer r;
    r.setRasterMode((swr::RasterMode)sc.raster);
    r.setScissorRect(sc.scissor[0], sc.scissor[1], sc.scissor[2], sc.scissor[3]);
    if (k == 3)
      r.setPixelShader<LastWriterPS>();
    else
      r.setPixelShader<StripePS>();
    if (sc.direct) {
      r.drawTriangleList((const swr::RasterizerVertex*)sc.rv.data(), sc.indices.data(), sc.indices.size());
    } else {
      swr::VertexProcessor v(&r);
      v.setViewport(sc.viewport[0], sc.viewport[1], sc.viewport[2], sc.viewport[3]);
      v.setDepthRange(sc.depth_range[0], sc.depth_range[1]);
      v.setCullMode((swr::CullMode)sc.cull);
      v.setVertexShader<FogVS>();
      v.setVertexAttribPointer(0, 16, sc.pos.data());
      v.setVertexAttribPointer(1, 12, sc.attr.data());
      v.drawElements((swr::DrawMode)sc.draw_mode, sc.indices.size(), sc.indices.data());
    }
    FILE* f = fopen((out + "/" + std::to_string(k) + "_ref.bin").c_str(), "wb");
    if (!f) return 2;
    fwrite(color.data(), 4, color.size(), f);
    fwrite(depth.data(), 4, depth.size(), f);
    fwrite(count.data(), 4, count.size(), f);
    fclose(f);
  }
  printf("ok\n");
  return 0;
}
