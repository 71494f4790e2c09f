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
  int32_t max_aniso;      // mip-mapped sampler: anisotropic sample limit (0 = 8, the default)
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
  enum { AVarCount = 0, PVarCount = 2, InterpolateZ = 1, InterpolateW = 1, HasDepth = 1, DepthMin = 1 };
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
  // 128-primitive chunks: on the dense 1080p mesh 2 % faster than 64 (fewer chunk passes in
  // the silhouette tiles that set the raster's length); 64 suits the other workloads
  enum { AVarCount = 3, PVarCount = 2, InterpolateZ = 1, InterpolateW = 1, HasDepth = 1, RasterOccupancy = 5,
         DepthCull = 0, RasterChunk = 128, DepthMin = 1, RasterSlices = 1 };
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
  enum { AVarCount = 3, PVarCount = 2, InterpolateZ = 1, InterpolateW = 1, HasDepth = 1, RasterOccupancy = 6,
         DepthCull = 0, DepthMin = 1 };
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
  enum { AVarCount = 0, PVarCount = 3, InterpolateZ = 1, InterpolateW = 1, HasDepth = 1, DepthMin = 1 };
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
  enum { AVarCount = 3, PVarCount = 0, InterpolateZ = 0, InterpolateW = 0, HasDepth = 0, Overwrite = 1 };
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
  enum { AVarCount = 0, PVarCount = 5, InterpolateZ = 1, InterpolateW = 1, HasDepth = 1, RasterOccupancy = 5,
         DepthCull = 0 };
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

// ---------------------------------------------------------------------------
// Mip-mapped texture sampling: a restatement of the reference's example texture
// (src/examples/Texture.h) for a mip chain held in device memory.  Texels are packed
// 0x00RRGGBB (the SDL surface format of Texture.h:225-231: R in bits 16-23); the chain is
// level 0 (tex_w x tex_h) followed by every smaller level down to 1 x 1, each
// max(1, w / 2) x max(1, h / 2) of the one before (Texture.h:246-290).

// Number of levels of the chain of a w x h texture.
SWR_HD int swr_mip_levels(int w, int h) {
  int n = 1;
  while (w > 1 || h > 1) {
    w = swr_maxi(1, w / 2);
    h = swr_maxi(1, h / 2);
    ++n;
  }
  return n;
}

struct SwrMip {
  const uint32_t* p;
  int w, h;
};

SWR_HD SwrMip swr_mip_level(const SwrUniforms& u, int level) {
  SwrMip m;
  m.p = (const uint32_t*)u.tex;
  m.w = u.tex_w;
  m.h = u.tex_h;
  for (int l = 0; l < level; ++l) {
    m.p += (size_t)m.w * (size_t)m.h;
    m.w = swr_maxi(1, m.w / 2);
    m.h = swr_maxi(1, m.h / 2);
  }
  return m;
}

SWR_HD uint32_t swr_rgb_channel(uint32_t c, int sh) { return (c >> sh) & 0xffu; }

// Texture::lerpColors (Texture.h:191-196).  The reference converts the possibly negative
// float (c2 - c1) * t straight to Uint8, which C++ leaves undefined; this takes the
// x86-64 result (truncate toward zero, keep the low 8 bits), i.e. c1 + trunc(d * t)
// wrapped to 8 bits -- the intended linear interpolation.
SWR_HD uint32_t swr_rgb_lerp(uint32_t c1, uint32_t c2, float t) {
  uint32_t out = 0;
  for (int sh = 16; sh >= 0; sh -= 8) {
    const int a = (int)swr_rgb_channel(c1, sh), b = (int)swr_rgb_channel(c2, sh);
    const int d = swr_trunc_int(swr_mul((float)(b - a), t));
    out |= ((uint32_t)(a + d) & 0xffu) << sh;
  }
  return out;
}

// Texture::bilinearLerpColors (Texture.h:198-218): per channel
// ((c00*(1-fx))*(1-fy) + (c10*fx)*(1-fy)) + (c01*(1-fx))*fy + (c11*fx)*fy, truncated.
SWR_HD uint32_t swr_rgb_bilerp(uint32_t c00, uint32_t c10, uint32_t c01, uint32_t c11, float fx, float fy) {
  const float gx = swr_sub(1.0f, fx), gy = swr_sub(1.0f, fy);
  uint32_t out = 0;
  for (int sh = 16; sh >= 0; sh -= 8) {
    float v = swr_mul(swr_mul((float)swr_rgb_channel(c00, sh), gx), gy);
    v = swr_add(v, swr_mul(swr_mul((float)swr_rgb_channel(c10, sh), fx), gy));
    v = swr_add(v, swr_mul(swr_mul((float)swr_rgb_channel(c01, sh), gx), fy));
    v = swr_add(v, swr_mul(swr_mul((float)swr_rgb_channel(c11, sh), fx), fy));
    out |= ((uint32_t)swr_trunc_int(v) & 0xffu) << sh;
  }
  return out;
}

// Texture::sampleBilinear (Texture.h:146-181) on one level; u, v in [0, 1].
SWR_HD uint32_t swr_sample_bilinear(const SwrMip& m, float u, float v) {
  const float px = swr_mul(u, (float)(m.w - 1));
  const float py = swr_mul(v, (float)(m.h - 1));
  const int x0 = swr_maxi(0, swr_trunc_int(swr_floorf(px)));
  const int y0 = swr_maxi(0, swr_trunc_int(swr_floorf(py)));
  const int x1 = swr_mini(m.w - 1, x0 + 1);
  const int y1 = swr_mini(m.h - 1, y0 + 1);
  const float fx = swr_sub(px, (float)x0);
  const float fy = swr_sub(py, (float)y0);
  const size_t w = (size_t)m.w;
  return swr_rgb_bilerp(m.p[(size_t)y0 * w + x0], m.p[(size_t)y0 * w + x1], m.p[(size_t)y1 * w + x0],
                        m.p[(size_t)y1 * w + x1], fx, fy);
}

SWR_HD float swr_clampf(float v, float lo, float hi) { return v < lo ? lo : (hi < v ? hi : v); }  // std::clamp

// Texture::sampleTrilinear (Texture.h:122-144).  A NaN footprint (the reference then
// converts NaN to int, which is undefined) samples level 0.
SWR_HD uint32_t swr_sample_trilinear(const SwrUniforms& t, float u, float v, float rho) {
  const int levels = swr_mip_levels(t.tex_w, t.tex_h);
  float lod = swr_log2(swr_maxf(rho, 1e-6f));
  if (swr_isnan(lod)) lod = 0.0f;
  lod = swr_clampf(lod, 0.0f, (float)(levels - 1));
  const int base = swr_trunc_int(swr_floorf(lod));
  const int next = swr_mini(base + 1, levels - 1);
  const float frac = swr_clampf(swr_sub(lod, (float)base), 0.0f, 1.0f);
  const uint32_t cb = swr_sample_bilinear(swr_mip_level(t, base), u, v);
  if (base == next) return cb;
  return swr_rgb_lerp(cb, swr_sample_bilinear(swr_mip_level(t, next), u, v), frac);
}

// u mod 1 into [0, 1) as Texture::sample wraps it (Texture.h:42-45); NaN (undefined
// downstream in the reference) wraps to 0.
SWR_HD float swr_wrap01(float u) {
  u = swr_fmodf(u, 1.0f);
  if (u < 0.0f) u = swr_add(u, 1.0f);
  return swr_isnan(u) ? 0.0f : u;
}

// Texture::sample (Texture.h:35-119): anisotropic filtering along the major axis of the
// pixel footprint, up to max_aniso trilinear taps.  Derivatives come from
// PixelData::computePerspectiveDerivatives.
SWR_HD uint32_t swr_tex_sample(const SwrUniforms& t, float u, float v, float dudx, float dvdx, float dudy,
                               float dvdy) {
  u = swr_wrap01(u);
  v = swr_wrap01(v);
  const float fw = (float)t.tex_w, fh = (float)t.tex_h;
  const float dudx_s = swr_mul(dudx, fw), dvdx_s = swr_mul(dvdx, fh);
  const float dudy_s = swr_mul(dudy, fw), dvdy_s = swr_mul(dvdy, fh);
  float dx_len = swr_sqrt(swr_add(swr_mul(dudx_s, dudx_s), swr_mul(dvdx_s, dvdx_s)));
  float dy_len = swr_sqrt(swr_add(swr_mul(dudy_s, dudy_s), swr_mul(dvdy_s, dvdy_s)));
  dx_len = swr_maxf(dx_len, 1e-6f);
  dy_len = swr_maxf(dy_len, 1e-6f);
  const float major = swr_maxf(dx_len, dy_len);
  const float minor = swr_minf(dx_len, dy_len);
  const int aniso = t.max_aniso > 0 ? swr_mini(t.max_aniso, 16) : 8;  // Texture.h:13-17
  const float ratio = swr_minf(swr_div(major, minor), (float)aniso);
  const int n = swr_isnan(ratio) ? 1 : swr_maxi(1, swr_trunc_int(swr_ceilf(ratio)));
  if (n <= 1) return swr_sample_trilinear(t, u, v, major);
  float mdu, mdv;
  if (dx_len > dy_len) {
    mdu = swr_div(dudx, dx_len);
    mdv = swr_div(dvdx, dx_len);
  } else {
    mdu = swr_div(dudy, dy_len);
    mdv = swr_div(dvdy, dy_len);
  }
  float r = 0.0f, g = 0.0f, b = 0.0f;
  const float step = swr_div(1.0f, (float)n);
  for (int i = 0; i < n; ++i) {
    const float k = swr_sub(swr_mul(swr_add((float)i, 0.5f), step), 0.5f);
    const float su = swr_wrap01(swr_add(u, swr_mul(swr_mul(mdu, major), k)));
    const float sv = swr_wrap01(swr_add(v, swr_mul(swr_mul(mdv, major), k)));
    const uint32_t c = swr_sample_trilinear(t, su, sv, minor);
    r = swr_add(r, (float)swr_rgb_channel(c, 16));
    g = swr_add(g, (float)swr_rgb_channel(c, 8));
    b = swr_add(b, (float)swr_rgb_channel(c, 0));
  }
  const float fn = (float)n;
  r = swr_minf(255.0f, swr_div(r, fn));
  g = swr_minf(255.0f, swr_div(g, fn));
  b = swr_minf(255.0f, swr_div(b, fn));
  return ((uint32_t)swr_trunc_int(r) << 16) | ((uint32_t)swr_trunc_int(g) << 8) | (uint32_t)swr_trunc_int(b);
}

// Mip-mapped textured shader of the reference's Box example (Box.cpp:40-66): no depth
// test, every fragment overwrites the pixel with the anisotropic sample at (u, v), its
// footprint from the perspective-correct derivatives of u and v.  PVar = uv.
struct PsTexMip {
  enum { AVarCount = 0, PVarCount = 2, InterpolateZ = 0, InterpolateW = 1, HasDepth = 0, NeedsEquations = 1,
         Overwrite = 1 };
  typedef SwrStateRGBA8 State;
  SWR_HD static void load(State& s, int x, int y, const SwrUniforms& u) { swr_load_rgba8<false>(s, x, y, u); }
  SWR_HD static void store(const State& s, int x, int y, const SwrUniforms& u) { swr_store_rgba8(s, x, y, u, false); }
  SWR_HD static bool earlyReject(float, State&) { return false; }
  typedef uint32_t Color;
  template <class PD>
  SWR_HD static Color shade(const PD& p, const SwrUniforms& u) {
    float dudx, dudy, dvdx, dvdy;
    swr_persp_deriv(p, 0, dudx, dudy);
    swr_persp_deriv(p, 1, dvdx, dvdy);
    return swr_tex_sample(u, p.pvar[0], p.pvar[1], dudx, dvdx, dudy, dvdy);
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

// Writes the perspective-correct derivatives of pvar 0 and 1 (PixelData.h:128-145) as
// RGBA32F (du/dx, du/dy, dv/dx, dv/dy), depth-tested: the derivative path itself.
struct PsPerspDeriv {
  enum { AVarCount = 0, PVarCount = 2, InterpolateZ = 1, InterpolateW = 1, HasDepth = 1, NeedsEquations = 1 };
  typedef SwrStateRGBA32F State;
  SWR_HD static void load(State& s, int x, int y, const SwrUniforms& u) { PsDiff::load(s, x, y, u); }
  SWR_HD static bool earlyReject(float z, State& s) { return swr_depth_reject(z, s); }
  SWR_HD static void store(const State& s, int x, int y, const SwrUniforms& u) { PsDiff::store(s, x, y, u); }
  typedef PsDiff::Color Color;
  template <class PD>
  SWR_HD static Color shade(const PD& p, const SwrUniforms&) {
    Color o;
    swr_persp_deriv(p, 0, o.c[0], o.c[1]);
    swr_persp_deriv(p, 1, o.c[2], o.c[3]);
    return o;
  }
  SWR_HD static void apply(State& s, float z, const Color& c, int prim) { PsDiff::apply(s, z, c, prim); }
  template <class PD>
  SWR_HD static void drawPixel(const PD& p, int prim, State& s, const SwrUniforms& u) {
    s.frags++;
    if (p.z < s.depth) PsDiff::write(s, p.z, shade(p, u), prim);
  }
};

// PixelData::computePerspectiveDerivatives (PixelData.h:128-145) from the triangle's
// parameter equations (a, b, c per equation, evaluated ((a x) + (b y)) + c at the pixel
// centre): d(var/invw) by the quotient rule, in the reference's operation order.
SWR_HD void swr_persp_deriv_eq(const float* pv, const float* iw, int x, int y, float& ddx, float& ddy) {
  const float fx = swr_add((float)x, 0.5f), fy = swr_add((float)y, 0.5f);
  const float var = swr_eval(pv[0], pv[1], pv[2], fx, fy);
  const float inv = swr_eval(iw[0], iw[1], iw[2], fx, fy);
  const float den = swr_mul(inv, inv);
  ddx = swr_div(swr_sub(swr_mul(inv, pv[0]), swr_mul(var, iw[0])), den);
  ddy = swr_div(swr_sub(swr_mul(inv, pv[1]), swr_mul(var, iw[1])), den);
}

// Program registry ids (stable C-ABI values).
enum SwrVsId { SWR_VS_POS_UV = 1, SWR_VS_POS_NRM_UV = 2, SWR_VS_POS_RGB = 3,
               SWR_VS_POS_RGB_AFFINE = 4, SWR_VS_POS_RGB_UV = 5 };
enum SwrPsId { SWR_PS_TEX_NEAREST = 1, SWR_PS_LAMBERT = 2, SWR_PS_VCOLOR = 3,
               SWR_PS_VCOLOR_AFFINE = 4, SWR_PS_LAMBERT_TEX = 5, SWR_PS_DIFF = 6,
               SWR_PS_TEX_MIP = 7, SWR_PS_PERSP_DERIV = 8 };

// Pixel shaders whose apply() is frags++, writes++ and an unconditional overwrite of the
// colour and winner: a pixel's final State after n fragments depends only on the last
// fragment's shade() and on n, so a rasterizer may shade only that fragment.
template <class PS, class = void>
struct SwrOverwrite {
  enum { value = 0 };
};
template <class PS>
struct SwrOverwrite<PS, decltype((void)PS::Overwrite)> {
  enum { value = PS::Overwrite };
};

// Depth-tested shaders (HasDepth, InterpolateZ, earlyReject = swr_depth_reject): a fragment
// with !(z < State::depth) only counts, and a write only lowers State::depth.  A rasterizer
// may therefore count, without interpolating, every fragment of a primitive whose z is
// provably not below the largest depth held by the pixels it covers.  A shader may opt out
// with DepthCull = 0.  The Lambert and differentiable shaders do: their tile rasters run at
// 5-6 CTAs per SM in 40-48 registers, where the cull's code made the Lambert rasters 3-5 %
// slower on their single-mesh workloads (which have nothing to cull) and the differentiable
// one spill.
template <class PS, class = void>
struct SwrDepthCull {
  enum { value = PS::HasDepth && PS::InterpolateZ && !SwrOverwrite<PS>::value };
};
template <class PS>
struct SwrDepthCull<PS, decltype((void)PS::DepthCull)> {
  enum { value = PS::DepthCull && PS::HasDepth && PS::InterpolateZ && !SwrOverwrite<PS>::value };
};

// Overwrite shaders' State after two consecutive runs of fragments: the later run's last
// writer (colour, winner) if it wrote at all, and the summed counters.  Lets a rasterizer
// split one pixel's fragments into ordered slices and merge their states.
SWR_HD void swr_overwrite_merge(SwrStateRGBA8& acc, const SwrStateRGBA8& later) {
  if (later.writes) {
    acc.color = later.color;
    acc.winner = later.winner;
  }
  acc.frags += later.frags;
  acc.writes += later.writes;
}

// Depth-tested RGBA8 shaders whose drawPixel is exactly `s.frags++; if (z < s.depth)
// swr_write(s, z, shade(p, u), prim)` with a shade() that reads nothing but the fragment
// (DepthMin = 1 in the shader).  In primitive order such a pixel ends with the depth
// min(d0, z_1 .. z_n) and the colour and winner of the FIRST fragment reaching it (a later
// equal z fails the strict test), so a pixel's fragments may be cut into ordered runs, each
// run from the draw's starting State, and the runs' States merged in order: a later run
// takes over only with a strictly smaller depth.  The merged colour, depth, winner and
// fragment count equal the sequential ones; `writes` becomes the sum of the runs' depth-test
// passes, each against the depth its run started from (at least the sequential count).
template <class PS, class = void>
struct SwrDepthMin {
  enum { value = 0 };
};
template <class PS>
struct SwrDepthMin<PS, decltype((void)PS::DepthMin)> {
  enum { value = PS::DepthMin && PS::HasDepth && PS::InterpolateZ && !SwrOverwrite<PS>::value };
};

// Heavy-tile slicing default of a depth-min shader (RasterSlices in the shader): tiles of
// more than RasterSlices raster chunks of bin entries are rasterized in runs; 0: whole tiles.
// Measured per workload: it pays where a few heavy tiles set the raster's length (a dense
// mesh's silhouette), and costs where heavy tiles are many (each run starts from the draw's
// starting depths, so fewer fragments fail early).
template <class PS, class = void>
struct SwrRasterSlices {
  enum { value = 0 };
};
template <class PS>
struct SwrRasterSlices<PS, decltype((void)PS::RasterSlices)> {
  enum { value = SwrDepthMin<PS>::value ? PS::RasterSlices : 0 };
};

// Depth-min shaders' State after two consecutive runs that both started from the same
// State (SwrDepthMin).  A run that wrote holds a depth below the starting one, so the
// merged State has writes != 0 exactly when some run's write survives.
SWR_HD void swr_depth_merge(SwrStateRGBA8& acc, const SwrStateRGBA8& later) {
  if (later.writes && later.depth < acc.depth) {
    acc.depth = later.depth;
    acc.color = later.color;
    acc.winner = later.winner;
  }
  acc.frags += later.frags;
  acc.writes += later.writes;
}

// Resident tile-raster CTAs per SM the register allocation of a shader's k_raster must
// allow (RasterOccupancy in the shader; measured per workload, default 4).
template <class PS, class = void>
struct SwrRasterOccupancy {
  enum { value = 4 };
};
template <class PS>
struct SwrRasterOccupancy<PS, decltype((void)PS::RasterOccupancy)> {
  enum { value = PS::RasterOccupancy };
};

// Pixel shaders whose drawPixel has side effects beyond its State (user shaders that write
// their own buffers, include/swr/Renderer.h): the rasterizer must call drawPixel once per
// fragment in primitive order and may not evaluate anything of the shader ahead of it.
template <class PS, class = void>
struct SwrNoCompact {
  enum { value = 0 };
};
template <class PS>
struct SwrNoCompact<PS, decltype((void)PS::NoCompact)> {
  enum { value = PS::NoCompact };
};

// Binned primitives the tile rasterizer stages per chunk for a shader (RasterChunk in the
// shader: 32, 64, 96 or 128; measured per workload, default SWR_CHUNK).
#ifndef SWR_CHUNK
#define SWR_CHUNK 64
#endif
template <class PS, class = void>
struct SwrRasterChunk {
  enum { value = SWR_CHUNK };
};
template <class PS>
struct SwrRasterChunk<PS, decltype((void)PS::RasterChunk)> {
  enum { value = PS::RasterChunk };
};

// Pixel shaders whose shade() reads the triangle's equations (PixelData::equations) --
// set only for triangles; the reference dereferences a null pointer for points and lines.
template <class PS, class = void>
struct SwrNeedsEquations {
  enum { value = 0 };
};
template <class PS>
struct SwrNeedsEquations<PS, decltype((void)PS::NeedsEquations)> {
  enum { value = PS::NeedsEquations };
};
