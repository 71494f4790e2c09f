// Shader classes written once against the reference's public API (VertexShaderBase /
// PixelShaderBase, src/renderer/VertexShaderBase.h:33-51, PixelShaderBase.h:40-137) and
// shipped by neither library: nvcc compiles them against include/swr/Renderer.h (the GPU
// pipeline), g++ against the reference's own headers (the oracle harness,
// oracle/user_shader_ref.cpp).  The includer provides namespace swr first.
//
// Their "statics" are device globals on the GPU and plain globals on the host:
//   g_mvp      model-view-projection matrix, row-major
//   g_target   the shader's own framebuffer: RGBA8 colour, FP32 depth, drawPixel count
#pragma once
#include <stdint.h>

#ifdef __CUDACC__
#define USER_SHADER __device__
#define USER_GLOBAL __device__
#else
#define USER_SHADER
#define USER_GLOBAL
#endif

struct UserTarget {
  uint32_t* color;
  float* depth;
  uint32_t* count;
  int width, height;
};

USER_GLOBAL float g_mvp[16];
USER_GLOBAL UserTarget g_target;

// [0, 1], NaN -> 0 (so no NaN reaches a float-to-int conversion, undefined in C++).
USER_SHADER inline float user_clamp01(float v) { return v >= 0.0f ? (v > 1.0f ? 1.0f : v) : 0.0f; }

USER_SHADER inline uint32_t user_u8(float v) { return (uint32_t)(int)(user_clamp01(v) * 255.0f + 0.5f); }

// Two attribute streams: stream 0 = {x, y, z, h} floats (16 B), stream 1 = {rgba8, u, v}
// (12 B).  AVar = {r, g, b, h} (affine), PVar = {u, v, w / 8} (perspective-correct).
class FogVS : public swr::VertexShaderBase<FogVS> {
 public:
  static const int AttribCount = 2;
  static const int AVarCount = 4;
  static const int PVarCount = 3;

  USER_SHADER static void processVertex(swr::VertexShaderInput in, swr::VertexShaderOutput* out) {
    const float* p = static_cast<const float*>(in[0]);
    const uint32_t* c = static_cast<const uint32_t*>(in[1]);
    const float* t = static_cast<const float*>(in[1]);
    const float x = p[0], y = p[1], z = p[2];
    float clip[4];
    for (int r = 0; r < 4; ++r) {
      float acc = g_mvp[4 * r] * x;
      acc = acc + g_mvp[4 * r + 1] * y;
      acc = acc + g_mvp[4 * r + 2] * z;
      clip[r] = acc + g_mvp[4 * r + 3];
    }
    out->x = clip[0];
    out->y = clip[1];
    out->z = clip[2];
    out->w = clip[3];
    const uint32_t rgba = c[0];
    out->avar[0] = (float)(rgba & 0xffu) / 255.0f;
    out->avar[1] = (float)((rgba >> 8) & 0xffu) / 255.0f;
    out->avar[2] = (float)((rgba >> 16) & 0xffu) / 255.0f;
    out->avar[3] = p[3];
    out->pvar[0] = t[1];
    out->pvar[1] = t[2];
    out->pvar[2] = clip[3] / 8.0f;
  }
};

// Depth-tested into the shader's own buffers; colour = vertex colour x a stripe pattern of
// the perspective-correct uv, darkened by a fog term and, on triangles, tinted by the uv
// footprint from PixelData::computePerspectiveDerivatives.  Counts every call per pixel.
class StripePS : public swr::PixelShaderBase<StripePS> {
 public:
  static const bool InterpolateZ = true;
  static const bool InterpolateW = true;
  static const int AVarCount = 4;
  static const int PVarCount = 3;

  USER_SHADER static void drawPixel(const swr::PixelData& p) {
    const UserTarget t = g_target;
    if (p.x < 0 || p.y < 0 || p.x >= t.width || p.y >= t.height) return;
    const int i = p.y * t.width + p.x;
    t.count[i] += 1u;
    if (!(p.z < t.depth[i])) return;
    t.depth[i] = p.z;
    const int su = (int)(user_clamp01(p.pvar[0]) * 8.0f);
    const int sv = (int)(user_clamp01(p.pvar[1]) * 8.0f);
    const float stripe = ((su + sv) & 1) ? 1.0f : 0.6f;
    const float fog = user_clamp01(1.0f - p.pvar[2] * 0.5f + p.avar[3] * 0.1f);
    float tint = 0.0f;
    if (p.equations) {
      float dudx, dudy, dvdx, dvdy;
      p.computePerspectiveDerivatives(*p.equations, 0, dudx, dudy);
      p.computePerspectiveDerivatives(*p.equations, 1, dvdx, dvdy);
      const float rho = (dudx * dudx + dvdx * dvdx) + (dudy * dudy + dvdy * dvdy);
      tint = user_clamp01(rho * 2000.0f);
    }
    const float r = p.avar[0] * stripe * fog;
    const float g = p.avar[1] * stripe * fog;
    const float b = user_clamp01(p.avar[2] * stripe * fog + tint);
    t.color[i] = user_u8(r) | (user_u8(g) << 8) | (user_u8(b) << 16) | 0xff000000u;
  }
};

// Writes every fragment's interpolants as colour (no depth test): the last primitive in
// the reference's order wins each pixel.  AVar = {r, g, b}.
class LastWriterPS : public swr::PixelShaderBase<LastWriterPS> {
 public:
  static const bool InterpolateZ = false;
  static const bool InterpolateW = false;
  static const int AVarCount = 3;
  static const int PVarCount = 0;

  USER_SHADER static void drawPixel(const swr::PixelData& p) {
    const UserTarget t = g_target;
    if (p.x < 0 || p.y < 0 || p.x >= t.width || p.y >= t.height) return;
    const int i = p.y * t.width + p.x;
    t.count[i] += 1u;
    t.color[i] = user_u8(p.avar[0]) | (user_u8(p.avar[1]) << 8) | (user_u8(p.avar[2]) << 16) | 0xff000000u;
  }
};
