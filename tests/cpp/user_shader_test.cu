// Shaders the library does not ship, drawn on the GPU through the header-only C++ API
// (include/swr/Renderer.h: Rasterizer / VertexProcessor with setPixelShader<PS>() and
// setVertexShader<VS>()) and through the C ABI (swr_set_vertex_program /
// swr_set_pixel_program).  For every case of tests/cpp/user_scene.h and both paths it
// writes the shader's framebuffer -- RGBA8 colour, FP32 depth, per-pixel drawPixel count,
// width x height each -- to <outdir>/<case>_<path>.bin; the test compares them with the
// reference library running the same shader classes (tests/golden/user_shader.json).
//
//   nvcc -gencode arch=compute_103a,code=sm_103a -std=c++17 -fmad=false -Iinclude -Itests/cpp \
//        tests/cpp/user_shader_test.cu -Lsoftwarerenderer_gb300/_build -lswr_gb300 -o user_shader_test
//   ./user_shader_test <outdir>
#include <swr/Renderer.h>

#include <cstdio>
#include <limits>
#include <string>
#include <vector>

#include "user_scene.h"
#include "user_shaders.h"

namespace {

void cuda_ok(cudaError_t e, const char* what) {
  if (e != cudaSuccess) {
    fprintf(stderr, "%s: %s\n", what, cudaGetErrorString(e));
    exit(2);
  }
}

void abi_ok(int rc, const char* what) {
  if (rc != SWR_OK) {
    fprintf(stderr, "%s: %s\n", what, swr_status_string(rc));
    exit(3);
  }
}

struct DeviceTarget {
  int w, h;
  uint32_t* color;
  float* depth;
  uint32_t* count;
  DeviceTarget(int w_, int h_) : w(w_), h(h_) {
    cuda_ok(cudaMalloc(&color, (size_t)w * h * 4), "cudaMalloc");
    cuda_ok(cudaMalloc(&depth, (size_t)w * h * 4), "cudaMalloc");
    cuda_ok(cudaMalloc(&count, (size_t)w * h * 4), "cudaMalloc");
    UserTarget t = {color, depth, count, w, h};
    cuda_ok(cudaMemcpyToSymbol(g_target, &t, sizeof(t)), "g_target");
  }
  void clear() {
    std::vector<float> inf((size_t)w * h, std::numeric_limits<float>::infinity());
    cuda_ok(cudaMemset(color, 0, (size_t)w * h * 4), "clear");
    cuda_ok(cudaMemset(count, 0, (size_t)w * h * 4), "clear");
    cuda_ok(cudaMemcpy(depth, inf.data(), (size_t)w * h * 4, cudaMemcpyHostToDevice), "clear");
  }
  void save(const std::string& path) const {
    std::vector<uint32_t> buf((size_t)w * h * 3);
    const size_t n = (size_t)w * h;
    cuda_ok(cudaMemcpy(buf.data(), color, n * 4, cudaMemcpyDeviceToHost), "read");
    cuda_ok(cudaMemcpy(buf.data() + n, depth, n * 4, cudaMemcpyDeviceToHost), "read");
    cuda_ok(cudaMemcpy(buf.data() + 2 * n, count, n * 4, cudaMemcpyDeviceToHost), "read");
    FILE* f = fopen(path.c_str(), "wb");
    if (!f || fwrite(buf.data(), 4, buf.size(), f) != buf.size()) {
      fprintf(stderr, "cannot write %s\n", path.c_str());
      exit(4);
    }
    fclose(f);
  }
};

template <class T>
T* to_device(const std::vector<T>& v) {
  T* p = nullptr;
  cuda_ok(cudaMalloc(&p, v.size() * sizeof(T)), "cudaMalloc");
  cuda_ok(cudaMemcpy(p, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice), "upload");
  return p;
}

// Case 3 draws with the order-only shader, every other case with the depth-tested one.
bool last_writer(int k) { return k == 3; }

// The reference's API: Rasterizer + VertexProcessor.  Even cases pass host arrays (copied at
// each draw), odd cases device arrays.
void draw_template(int k, const UserScene& sc, swr::Rasterizer& r) {
  r.setRasterMode((swr::RasterMode)sc.raster);
  r.setScissorRect(sc.scissor[0], sc.scissor[1], sc.scissor[2], sc.scissor[3]);
  if (last_writer(k))
    r.setPixelShader<LastWriterPS>();
  else
    r.setPixelShader<StripePS>();
  const bool host = (k % 2) == 0;
  std::vector<int> idx = sc.indices;
  int* di = host ? idx.data() : to_device(sc.indices);
  if (sc.direct) {
    const swr::RasterizerVertex* rv = (const swr::RasterizerVertex*)sc.rv.data();
    if (!host) rv = (const swr::RasterizerVertex*)to_device(sc.rv);
    r.drawTriangleList(rv, di, idx.size());
    if (!host) cudaFree((void*)rv);
  } else {
    swr::VertexProcessor v(&r);
    v.setViewport(sc.viewport[0], sc.viewport[1], sc.viewport[2], sc.viewport[3]);
    v.setDepthRange(sc.depth_range[0], sc.depth_range[1]);
    v.setCullMode((swr::CullMode)sc.cull);
    v.setVertexShader<FogVS>();
    const float* p0 = host ? sc.pos.data() : to_device(sc.pos);
    const uint32_t* p1 = host ? sc.attr.data() : to_device(sc.attr);
    v.setVertexAttribPointer(0, 16, p0);
    v.setVertexAttribPointer(1, 12, p1);
    v.drawElements((swr::DrawMode)sc.draw_mode, idx.size(), di);
    if (!host) {
      cudaFree((void*)p0);
      cudaFree((void*)p1);
    }
  }
  if (!host) cudaFree(di);
}

// The C ABI with the same shader classes (device arrays).
void draw_capi(int k, const UserScene& sc) {
  swr_context* c = nullptr;
  abi_ok(swr_create(&c), "swr_create");
  abi_ok(swr_set_vertex_program(c, swr::vertex_program<FogVS>()), "swr_set_vertex_program");
  abi_ok(swr_set_pixel_program(c, last_writer(k) ? swr::pixel_program<LastWriterPS>() : swr::pixel_program<StripePS>()),
         "swr_set_pixel_program");
  abi_ok(swr_set_raster_mode(c, sc.raster), "raster mode");
  abi_ok(swr_set_scissor_rect(c, sc.scissor[0], sc.scissor[1], sc.scissor[2], sc.scissor[3]), "scissor");
  abi_ok(swr_set_viewport(c, sc.viewport[0], sc.viewport[1], sc.viewport[2], sc.viewport[3]), "viewport");
  abi_ok(swr_set_depth_range(c, sc.depth_range[0], sc.depth_range[1]), "depth range");
  abi_ok(swr_set_cull_mode(c, sc.cull), "cull mode");
  SwrUniforms u;
  memset(&u, 0, sizeof(u));
  u.width = sc.width;  // the pipeline's target extent; the shader owns its buffers
  u.height = sc.height;
  u.color = (void*)&u;  // a target key only
  abi_ok(swr_set_uniforms(c, &u), "uniforms");
  int* di = to_device(sc.indices);
  float* p0 = to_device(sc.pos);
  uint32_t* p1 = to_device(sc.attr);
  float* rv = sc.direct ? to_device(sc.rv) : nullptr;
  abi_ok(swr_set_vertex_attrib_pointer(c, 0, 16, p0, sc.pos.size() * 4), "attrib 0");
  abi_ok(swr_set_vertex_attrib_pointer(c, 1, 12, p1, sc.attr.size() * 4), "attrib 1");
  for (int attempt = 0;; ++attempt) {
    if (sc.direct)
      abi_ok(swr_draw_list(c, sc.draw_mode, rv, sc.rv.size() / 36, di, sc.indices.size(), nullptr), "swr_draw_list");
    else
      abi_ok(swr_draw_elements(c, sc.draw_mode, sc.indices.size(), (const uint32_t*)di, nullptr),
             "swr_draw_elements");
    swr_stats st;
    const int rc = swr_finish(c, nullptr, &st);
    if (rc == SWR_EOVERFLOW && attempt < 3) continue;
    abi_ok(rc, "swr_finish");
    break;
  }
  cudaFree(di);
  cudaFree(p0);
  cudaFree(p1);
  if (rv) cudaFree(rv);
  abi_ok(swr_destroy(c), "swr_destroy");
}

}  // namespace

int main(int argc, char** argv) {
  if (argc < 2) {
    fprintf(stderr, "usage: %s <outdir>\n", argv[0]);
    return 1;
  }
  const std::string out = argv[1];
  DeviceTarget t(320, 240);
  swr::Rasterizer r;
  for (int k = 0; k < user_case_count(); ++k) {
    const UserScene sc = user_scene(k);
    cuda_ok(cudaMemcpyToSymbol(g_mvp, sc.mvp, sizeof(sc.mvp)), "g_mvp");
    t.clear();
    try {
      draw_template(k, sc, r);
    } catch (const swr::Error& e) {
      fprintf(stderr, "case %d: %s\n", k, e.what());
      return 5;
    }
    t.save(out + "/" + std::to_string(k) + "_template.bin");
    t.clear();
    draw_capi(k, sc);
    t.save(out + "/" + std::to_string(k) + "_capi.bin");
    printf("case %d: %llu fragments\n", k, (unsigned long long)r.lastStats().fragments);
  }
  cuda_ok(cudaDeviceSynchronize(), "sync");
  printf("ok\n");
  return 0;
}
