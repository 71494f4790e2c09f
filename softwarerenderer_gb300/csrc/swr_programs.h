// Built-in shader programs: vertex shaders (VertexShaderBase, VertexShaderBase.h:33-51)
// and pixel shaders (PixelShaderBase, PixelShaderBase.h:40-137) written once as
// host+device functors.  The same source is compiled into the CUDA kernels, into the
// CPU oracle port and into the harness that drives the reference library, so all
// three run the identical per-vertex and per-fragment arithmetic (IEEE binary32, no
// FMA, correctly rounded divide and square root only).
//
// Vertex shader contract (mirrors VertexShaderBase): static AttribCount, AVarCount,
// PVarCount, the bytes read from each attribute element (Bytes0, Bytes1) and
// processVertex(in, out, uniforms) where in[i] points at element
// `index` of attribute stream i (VertexProcessor::attribPointer,
// VertexProcessor.cpp:134-139) and out exposes x, y, z, w, avar[], pvar[].
//
// Pixel shader contract: static AVarCount, PVarCount, InterpolateZ, InterpolateW
// (PixelShaderBase.h:44-53), a per-pixel State that the reference keeps in the
// shader's own static buffers (with `frags` and `writes` counters), and
// load / drawPixel / store / earlyReject / shade / apply.  earlyReject(z, s) returns true
// when drawPixel with depth z would do nothing but count the fragment (a failing depth
// test); it then counts it itself, so the rasterizer may skip building the other
// interpolants.  Every built-in drawPixel is apply(s, z, shade(p, u), prim) with shade a
// pure function of the fragment and the uniforms (evaluated only when it is used), so the
// rasterizer may compute shade() for a fragment early and apply() it in primitive order.  drawPixel is the
// reference's drawPixel(const PixelData&) (PixelShaderBase.h:116); load/store move
// the pixel's framebuffer values between memory and State.  Calling
// load + drawPixel + store per fragment is exactly the reference's side effect; the
// GPU tile walker calls load once per pixel, drawPixel per fragment in primitive
// order, and store once, which is the same sequence of memory states as seen from
// outside the draw.
#pragma once
#include "swr_math.h"

// Uniform block shared by every built-in program.  The reference keeps these
// values in shader statics (e.g. Box.cpp:150-199); here they travel with the draw.
// Pointers are device pointers for the GPU path and host pointers for the oracle.
struct SwrUniforms {
  float mvp[16];          // row-major: clip = mvp * (x, y, z, 1)
  float light[4];         // unit light direction xyz, ambient term w
  const void* tex;        // texels: RGBA8 packed in uint32, or RGBA32F as 4 floats
  int32_t tex_w, tex_h;
  void* color;            // RGBA8 (uint32 per pixel) or RGBA32F (4 floats per pixel)
  float* depth;           // FP32 depth buffer (unused by shaders without depth test)
  uint32_t* frag_count;   // optional: per-pixel count of drawPixel calls
  int32_t* winner;        // optional: per-pixel primitive id of the last colour write
  int32_t width, height;  // render target size in pixels; row pitch == width
  int32_t checker;        // checker squares per unit of uv for procedural albedo
  int32_t _pad;
};

// Vertex attribute pointers as handed to VS::processVertex (VertexConfig.h:34-40).
struct SwrVertexInput {
  const void* p[8];
};

// ---------------------------------------------------------------------------
// small shared helpers
SWR_HD void swr_xform4(const float* m, float x, float y, float z, float* o) {
  // ((m0*x + m1*y) + m2*z) + m3 per row, left to right.
  for (int r = 0; r < 4; ++r)
    o[r] = swr_add(swr_add(swr_add(swr_mul(m[4 * r + 0], x), swr_mul(m[4 * r + 1], y)),
                           swr_mul(m[4 * r + 2], z)),
                   m[4 * r + 3]);
}

SWR_HD float swr_clamp01(float v) { return swr_minf(swr_maxf(v, 0.0f), 1.0f); }

SWR_HD uint32_t swr_to_u8(float v) {
  return (uint32_t)swr_trunc_int(swr_add(swr_mul(swr_clamp01(v), 255.0f), 0.5f));
}

SWR_HD uint32_t swr_pack_rgba8(float r, float g, float b, float a) {
  return swr_to_u8(r) | (swr_to_u8(g) << 8) | (swr_to_u8(b) << 16) | (swr_to_u8(a) << 24);
}

SWR_HD float swr_u8_channel(uint32_t c, int sh) { return (float)((c >> sh) & 0xffu); }

// ---------------------------------------------------------------------------
// Vertex shaders

// Textured mesh: stream 0 = {x, y, z, u, v} (20 B).  PVar = uv.
struct VsPosUV {
  enum { AttribCount = 1, AVarCount = 0, PVarCount = 2, Bytes0 = 20, Bytes1 = 0 };
  template <class Out>
  SWR_HD static void processVertex(const SwrVertexInput& in, Out* out, const SwrUniforms& u) {
    const float* d = (const float*)in.p[0];
    float c[4];
    swr_xform4(u.mvp, d[0], d[1], d[2], c);
    out->x = c[0]; out->y = c[1]; out->z = c[2]; out->w = c[3];
    out->pvar[0] = d[3];
    out->pvar[1] = d[4];
  }
};

// Lit mesh: stream 0 = {x, y, z, nx, ny, nz} (24 B), stream 1 = {u, v} (8 B).
// AVar = normal, PVar = uv.
struct VsPosNrmUV {
  enum { AttribCount = 2, AVarCount = 3, PVarCount = 2, Bytes0 = 24, Bytes1 = 8 };
  template <class Out>
  SWR_HD static void processVertex(const SwrVertexInput& in, Out* out, const SwrUniforms& u) {
    const float* d = (const float*)in.p[0];
    const float* t = (const float*)in.p[1];
    float c[4];
    swr_xform4(u.mvp, d[0], d[1], d[2], c);
    out->x = c[0]; out->y = c[1]; out->z = c[2]; out->w = c[3];
    out->avar[0] = d[3]; out->avar[1] = d[4]; out->avar[2] = d[5];
    out->pvar[0] = t[0]; out->pvar[1] = t[1];
  }
};

// Vertex colour, perspective-correct: stream 0 = {x, y, z, r, g, b} (24 B).  PVar = rgb.
struct VsPosRGB {
  enum { AttribCount = 1, AVarCount = 0, PVarCount = 3, Bytes0 = 24, Bytes1 = 0 };
  template <class Out>
  SWR_HD static void processVertex(const SwrVertexInput& in, Out* out, const SwrUniforms& u) {
    const float* d = (const float*)in.p[0];
    float c[4];
    swr_xform4(u.mvp, d[0], d[1], d[2], c);
    out->x = c[0]; out->y = c[1]; out->z = c[2]; out->w = c[3];
    out->pvar[0] = d[3]; out->pvar[1] = d[4]; out->pvar[2] = d[5];
  }
};

// Vertex colour, affine: stream 0 = {x, y, z, r, g, b} (24 B).  AVar = rgb.  With an
// identity mvp this is the vertex shader of Benchmark.cpp:32-49 / VertexProcessorTest.
struct VsPosRGBAffine {
  enum { AttribCount = 1, AVarCount = 3, PVarCount = 0, Bytes0 = 24, Bytes1 = 0 };
  template <class Out>
  SWR_HD static void processVertex(const SwrVertexInput& in, Out* out, const SwrUniforms& u) {
    const float* d = (const float*)in.p[0];
    float c[4];
    swr_xform4(u.mvp, d[0], d[1], d[2], c);
    out->x = c[0]; out->y = c[1]; out->z = c[2]; out->w = c[3];
    out->avar[0] = d[3]; out->avar[1] = d[4]; out->avar[2] = d[5];
  }
};

// Differentiable-rendering mesh: stream 0 = {x, y, z, r, g, b, u, v} (32 B).
// PVar = {r, g, b, u, v}.
struct VsPosRGBUV {
  enum { AttribCount = 1, AVarCount = 0, PVarCount = 5, Bytes0 = 32, Bytes1 = 0 };
  template <class Out>
  SWR_HD static void processVertex(const SwrVertexInput& in, Out* out, const SwrUniforms& u) {
    const float* d = (const float*)in.p[0];
    float c[4];
    swr_xform4(u.mvp, d[0], d[1], d[2], c);
    out->x = c[0]; out->y = c[1]; out->z = c[2]; out->w = c[3];
    for (int i = 0; i < 5; ++i) out->pvar[i] = d[3 + i];
  }
};

// ---------------------------------------------------------------------------
// Pixel shaders.  State is the pixel's framebuffer view while fragments are applied.

struct SwrStateRGBA8 {
  float depth;
  uint32_t color;
  uint32_t frags;   // drawPixel calls applied to this State
  uint32_t writes;  // colour writes (depth-test passes)
  int32_t winner;
};

struct SwrStateRGBA32F {
  float depth;
  float color[4];
  uint32_t frags;
  uint32_t writes;
  int32_t winner;
};

// Early depth rejection shared by the depth-tested shaders: their drawPixel does only
// `s.frags++` when !(z < s.depth).
template <class State>
SWR_HD bool swr_depth_reject(float z, State& s) {
  if (z < s.depth) return false;
  s.frags++;
  return true;
}

// Colour write of the RGBA8 depth-tested shaders, and their drawPixel in apply() form.
SWR_HD void swr_write(SwrStateRGBA8& s, float z, uint32_t c, int prim) {
  s.depth = z;
  s.color = c;
  s.winner = prim;
  s.writes++;
}

SWR_HD void swr_apply_depth(SwrStateRGBA8& s, float z, uint32_t c, int prim) {
  s.frags++;
  if (z < s.depth) swr_write(s, z, c, prim);
}

template <bool kDepth>
SWR_HD void swr_load_rgba8(SwrStateRGBA8& s, int x, int y, const SwrUniforms& u) {
  const size_t i = (size_t)y * (size_t)u.width + (size_t)x;
  s.depth = kDepth ? u.depth[i] : 0.0f;
  s.color = 0u;
  s.frags = 0u;
  s.writes = 0u;
  s.winner = -1;
}

SWR_HD void swr_store_rgba8(const SwrStateRGBA8& s, int x, int y, const SwrUniforms& u,
                            bool depth) {
  const size_t i = (size_t)y * (size_t)u.width + (size_t)x;
  if (s.writes) {
    ((uint32_t*)u.color)[i] = s.color;
    if (depth) u.depth[i] = s.depth;
    if (u.winner) u.winner[i] = s.winner;
  }
  if (u.frag_count && s.frags) u.frag_count[i] += s.frags;
}

// Nearest-texel RGBA8 fetch with clamp addressing.
SWR_HD uint32_t swr_tex_nearest(const SwrUniforms& u, float tu, float tv) {
  int tx = swr_trunc_int(swr_mul(swr_clamp01(tu), (float)u.tex_w));
  int ty = swr_trunc_int(swr_mul(swr_clamp01(tv), (float)u.tex_h));
  tx = swr_mini(tx, u.tex_w - 1);
  ty = swr_mini(ty, u.tex_h - 1);
  return ((const uint32_t*)u.tex)[(size_t)ty * (size_t)u.tex_w + (size_t)tx];
}

// Textured, depth-tested (config: textured cube).  PVar = uv.
struct PsTexNearest {
  enum { AVarCount = 0, PVarCount = 2, InterpolateZ = 1, InterpolateW = 1, HasDepth = 1 };
  typedef SwrStateRGBA8 State;
  SWR_HD static void load(State& s, int x, int y, const SwrUniforms& u) { swr_load_rgba8<true>(s, x, y, u); }
  SWR_HD static void store(const State& s, int x, int y, const SwrUniforms& u) { swr_store_rgba8(s, x, y, u, true); }
  SWR_HD static bool earlyReject(float z, State& s) { return swr_depth_reject(z, s); }
  typedef uint32_t Color;
  template <class PD>
  SWR_HD static Color shade(const PD& p, const SwrUniforms& u) {
    return swr_tex_nearest(u, p.pvar[0], p.pvar[1]) | 0xff000000u;
  }
  SWR_HD static void apply(State& s, float z, Color c, int prim) { swr_apply_depth(s, z, c, prim); }
  template <class PD>
  SWR_HD static void drawPixel(const PD& p, int prim, State& s, const SwrUniforms& u) {
    s.frags++;
    if (p.z < s.depth) swr_write(s, p.z, shade(p, u), prim);
  }
};

// Lambert-lit procedural checker, depth-tested (config: dense icosphere).
// AVar = normal, PVar = uv.
struct PsLambert {
  enum { AVarCount = 3, PVarCount = 2, InterpolateZ = 1, InterpolateW = 1, HasDepth = 1 };
  typedef SwrStateRGBA8 State;
  SWR_HD static void load(State& s, int x, int y, const SwrUniforms& u) { swr_load_rgba8<true>(s, x, y, u); }
  SWR_HD static void store(const State& s, int x, int y, const SwrUniforms& u) { swr_store_rgba8(s, x, y, u, true); }
  SWR_HD static bool earlyReject(float z, State& s) { return swr_depth_reject(z, s); }
  SWR_HD static float intensity(float n0, float n1, float n2, const SwrUniforms& u) {
    const float len2 = swr_add(swr_add(swr_mul(n0, n0), swr_mul(n1, n1)), swr_mul(n2, n2));
    float d = 0.0f;
    if (len2 > 0.0f) {
      const float dot = swr_add(swr_add(swr_mul(n0, u.light[0]), swr_mul(n1, u.light[1])),
                                swr_mul(n2, u.light[2]));
      d = swr_maxf(swr_div(dot, swr_sqrt(len2)), 0.0f);
    }
    return swr_add(u.light[3], swr_mul(swr_sub(1.0f, u.light[3]), d));
  }
  SWR_HD static float checker(float tu, float tv, const SwrUniforms& u) {
    const int cu = swr_trunc_int(swr_mul(swr_clamp01(tu), (float)u.checker));
    const int cv = swr_trunc_int(swr_mul(swr_clamp01(tv), (float)u.checker));
    return ((cu + cv) & 1) ? 1.0f : 0.55f;
  }
  typedef uint32_t Color;
  template <class PD>
  SWR_HD static Color shade(const PD& p, const SwrUniforms& u) {
    const float li = intensity(p.avar[0], p.avar[1], p.avar[2], u);
    const float al = checker(p.pvar[0], p.pvar[1], u);
    const float c = swr_mul(al, li);
    return swr_pack_rgba8(c, swr_mul(c, 0.9f), swr_mul(c, 0.75f), 1.0f);
  }
  SWR_HD static void apply(State& s, float z, Color c, int prim) { swr_apply_depth(s, z, c, prim); }
  template <class PD>
  SWR_HD static void drawPixel(const PD& p, int prim, State& s, const SwrUniforms& u) {
    s.frags++;
    if (p.z < s.depth) swr_write(s, p.z, shade(p, u), prim);
  }
};

// Lambert-lit and textured (nearest RGBA8), depth-tested (config: batched meshes).
struct PsLambertTex {
  enum { AVarCount = 3, PVarCount = 2, InterpolateZ = 1, InterpolateW = 1, HasDepth = 1 };
  typedef SwrStateRGBA8 State;
  SWR_HD static void load(State& s, int x, int y, const SwrUniforms& u) { swr_load_rgba8<true>(s, x, y, u); }
  SWR_HD static void store(const State& s, int x, int y, const SwrUniforms& u) { swr_store_rgba8(s, x, y, u, true); }
  SWR_HD static bool earlyReject(float z, State& s) { return swr_depth_reject(z, s); }
  typedef uint32_t Color;
  template <class PD>
  SWR_HD static Color shade(const PD& p, const SwrUniforms& u) {
    const float li = PsLambert::intensity(p.avar[0], p.avar[1], p.avar[2], u);
    const uint32_t t = swr_tex_nearest(u, p.pvar[0], p.pvar[1]);
    const float sc = swr_div(li, 255.0f);
    return swr_pack_rgba8(swr_mul(swr_u8_channel(t, 0), sc), swr_mul(swr_u8_channel(t, 8), sc),
                          swr_mul(swr_u8_channel(t, 16), sc), 1.0f);
  }
  SWR_HD static void apply(State& s, float z, Color c, int prim) { swr_apply_depth(s, z, c, prim); }
  template <class PD>
  SWR_HD static void drawPixel(const PD& p, int prim, State& s, const SwrUniforms& u) {
    s.frags++;
    if (p.z < s.depth) swr_write(s, p.z, shade(p, u), prim);
  }
};

// Perspective-correct vertex colour, depth-tested (config: triangle soup).  PVar = rgb.
struct PsVColor {
  enum { AVarCount = 0, PVarCount = 3, InterpolateZ = 1, InterpolateW = 1, HasDepth = 1 };
  typedef SwrStateRGBA8 State;
  SWR_HD static void load(State& s, int x, int y, const SwrUniforms& u) { swr_load_rgba8<true>(s, x, y, u); }
  SWR_HD static void store(const State& s, int x, int y, const SwrUniforms& u) { swr_store_rgba8(s, x, y, u, true); }
  SWR_HD static bool earlyReject(float z, State& s) { return swr_depth_reject(z, s); }
  typedef uint32_t Color;
  template <class PD>
  SWR_HD static Color shade(const PD& p, const SwrUniforms&) {
    return swr_pack_rgba8(p.pvar[0], p.pvar[1], p.pvar[2], 1.0f);
  }
  SWR_HD static void apply(State& s, float z, Color c, int prim) { swr_apply_depth(s, z, c, prim); }
  template <class PD>
  SWR_HD static void drawPixel(const PD& p, int prim, State& s, const SwrUniforms& u) {
    s.frags++;
    if (p.z < s.depth) swr_write(s, p.z, shade(p, u), prim);
  }
};

// Affine vertex colour without depth test: every fragment overwrites the pixel, so the
// final image is decided purely by primitive order (the pixel shaders of
// Benchmark.cpp:14-26 and VertexProcessorTest / RasterizerTest).  AVar = rgb.
struct PsVColorAffine {
  enum { AVarCount = 3, PVarCount = 0, InterpolateZ = 0, InterpolateW = 0, HasDepth = 0 };
  typedef SwrStateRGBA8 State;
  SWR_HD static void load(State& s, int x, int y, const SwrUniforms& u) { swr_load_rgba8<false>(s, x, y, u); }
  SWR_HD static void store(const State& s, int x, int y, const SwrUniforms& u) { swr_store_rgba8(s, x, y, u, false); }
  SWR_HD static bool earlyReject(float, State&) { return false; }
  typedef uint32_t Color;
  template <class PD>
  SWR_HD static Color shade(const PD& p, const SwrUniforms&) {
    return swr_pack_rgba8(p.avar[0], p.avar[1], p.avar[2], 1.0f);
  }
  SWR_HD static void apply(State& s, float, Color c, int prim) {
    s.frags++;
    s.color = c;
    s.winner = prim;
    s.writes++;
  }
  template <class PD>
  SWR_HD static void drawPixel(const PD& p, int prim, State& s, const SwrUniforms& u) {
    apply(s, 0.0f, shade(p, u), prim);
  }
};

// Bilinear RGBA32F fetch with the addressing of the reference's example texture
// sampler (Texture.h:146-181: px = u*(w-1), x0 = floor, x1 = min(w-1, x0+1)), in float.
SWR_HD void swr_tex_bilinear_f32(const SwrUniforms& u, float tu, float tv, float* out) {
  const float px = swr_mul(swr_clamp01(tu), (float)(u.tex_w - 1));
  const float py = swr_mul(swr_clamp01(tv), (float)(u.tex_h - 1));
  const int x0 = swr_trunc_int(px);  // px >= 0: truncation == floor
  const int y0 = swr_trunc_int(py);
  const int x1 = swr_mini(u.tex_w - 1, x0 + 1);
  const int y1 = swr_mini(u.tex_h - 1, y0 + 1);
  const float fx = swr_sub(px, (float)x0);
  const float fy = swr_sub(py, (float)y0);
  const float* t = (const float*)u.tex;
  const size_t w = (size_t)u.tex_w;
  const float* c00 = t + 4 * ((size_t)y0 * w + (size_t)x0);
  const float* c10 = t + 4 * ((size_t)y0 * w + (size_t)x1);
  const float* c01 = t + 4 * ((size_t)y1 * w + (size_t)x0);
  const float* c11 = t + 4 * ((size_t)y1 * w + (size_t)x1);
  const float gx = swr_sub(1.0f, fx), gy = swr_sub(1.0f, fy);
  for (int c = 0; c < 4; ++c) {
    const float top = swr_add(swr_mul(c00[c], gx), swr_mul(c10[c], fx));
    const float bot = swr_add(swr_mul(c01[c], gx), swr_mul(c11[c], fx));
    out[c] = swr_add(swr_mul(top, gy), swr_mul(bot, fy));
  }
}

// Differentiable-rendering shader: colour = vertex rgb * bilinear(texture, uv), RGBA32F
// target, depth-tested.  PVar = {r, g, b, u, v}.
struct PsDiff {
  enum { AVarCount = 0, PVarCount = 5, InterpolateZ = 1, InterpolateW = 1, HasDepth = 1 };
  typedef SwrStateRGBA32F State;
  SWR_HD static void load(State& s, int x, int y, const SwrUniforms& u) {
    const size_t i = (size_t)y * (size_t)u.width + (size_t)x;
    s.depth = u.depth[i];
    s.color[0] = s.color[1] = s.color[2] = s.color[3] = 0.0f;
    s.frags = 0u;
    s.writes = 0u;
    s.winner = -1;
  }
  SWR_HD static bool earlyReject(float z, State& s) { return swr_depth_reject(z, s); }
  SWR_HD static void store(const State& s, int x, int y, const SwrUniforms& u) {
    const size_t i = (size_t)y * (size_t)u.width + (size_t)x;
    if (s.writes) {
      float* c = (float*)u.color + 4 * i;
      c[0] = s.color[0]; c[1] = s.color[1]; c[2] = s.color[2]; c[3] = s.color[3];
      u.depth[i] = s.depth;
      if (u.winner) u.winner[i] = s.winner;
    }
    if (u.frag_count && s.frags) u.frag_count[i] += s.frags;
  }
  struct Color {
    float c[4];
  };
  template <class PD>
  SWR_HD static Color shade(const PD& p, const SwrUniforms& u) {
    float t[4];
    swr_tex_bilinear_f32(u, p.pvar[3], p.pvar[4], t);
    Color o;
    o.c[0] = swr_mul(p.pvar[0], t[0]);
    o.c[1] = swr_mul(p.pvar[1], t[1]);
    o.c[2] = swr_mul(p.pvar[2], t[2]);
    o.c[3] = t[3];
    return o;
  }
  SWR_HD static void write(State& s, float z, const Color& c, int prim) {
    s.depth = z;
    s.color[0] = c.c[0]; s.color[1] = c.c[1]; s.color[2] = c.c[2]; s.color[3] = c.c[3];
    s.winner = prim;
    s.writes++;
  }
  SWR_HD static void apply(State& s, float z, const Color& c, int prim) {
    s.frags++;
    if (z < s.depth) write(s, z, c, prim);
  }
  template <class PD>
  SWR_HD static void drawPixel(const PD& p, int prim, State& s, const SwrUniforms& u) {
    s.frags++;
    if (p.z < s.depth) write(s, p.z, shade(p, u), prim);
  }
};

// Program registry ids (stable C-ABI values).
enum SwrVsId { SWR_VS_POS_UV = 1, SWR_VS_POS_NRM_UV = 2, SWR_VS_POS_RGB = 3,
               SWR_VS_POS_RGB_AFFINE = 4, SWR_VS_POS_RGB_UV = 5 };
enum SwrPsId { SWR_PS_TEX_NEAREST = 1, SWR_PS_LAMBERT = 2, SWR_PS_VCOLOR = 3,
               SWR_PS_VCOLOR_AFFINE = 4, SWR_PS_LAMBERT_TEX = 5, SWR_PS_DIFF = 6 };
