// Seeded scenes for the user-shader tests, generated identically by the GPU test program
// (tests/cpp/user_shader_test.cu) and the oracle harness (oracle/user_shader_ref.cpp):
// integers from a 64-bit LCG, floats only from exact conversions and single IEEE
// operations, the camera matrix computed in double and rounded once.
#pragma once
#include <stdint.h>
#include <vector>

struct UserScene {
  int width = 320, height = 240;
  int draw_mode = 2;   // DrawMode: 0 point, 1 line, 2 triangle
  int cull = 2;        // CullMode: 0 None, 1 CCW, 2 CW
  int raster = 0;      // RasterMode: 0 Span, 1 Block, 2 Adaptive
  int viewport[4] = {0, 0, 320, 240};
  int scissor[4] = {0, 0, 320, 240};
  float depth_range[2] = {0.0f, 1.0f};
  float mvp[16];
  std::vector<float> pos;      // 4 floats per vertex: x, y, z, h
  std::vector<uint32_t> attr;  // 3 words per vertex: rgba8, u (float bits), v (float bits)
  std::vector<int> indices;
  bool direct = false;         // Rasterizer::drawTriangleList of screen-space vertices
  std::vector<float> rv;       // direct: 36 floats per RasterizerVertex
};

struct UserLcg {
  uint64_t s;
  explicit UserLcg(uint64_t seed) : s(seed * 6364136223846793005ull + 1442695040888963407ull) {}
  uint32_t next() {
    s = s * 6364136223846793005ull + 1442695040888963407ull;
    return (uint32_t)(s >> 32);
  }
  float unit() { return (float)(next() >> 8) * (1.0f / 16777216.0f); }  // exact, [0, 1)
};

inline uint32_t user_float_bits(float f) {
  union {
    float f;
    uint32_t u;
  } c;
  c.f = f;
  return c.u;
}

// Perspective (60 degree vertical field of view, cot 30 deg = sqrt 3) times a translation
// by -dist along z, rounded to float once.
inline void user_camera(float* m, double aspect, double n, double f, double dist, double ox) {
  const double cot = 1.7320508075688772;  // sqrt(3) to double precision
  double p[16] = {cot / aspect, 0, 0, 0, 0, cot, 0, 0, 0, 0, (f + n) / (n - f), 2 * f * n / (n - f), 0, 0, -1, 0};
  double t[16] = {1, 0, 0, ox, 0, 1, 0, 0, 0, 0, 1, -dist, 0, 0, 0, 1};
  for (int r = 0; r < 4; ++r)
    for (int c = 0; c < 4; ++c) {
      double a = 0;
      for (int k = 0; k < 4; ++k) a += p[4 * r + k] * t[4 * k + c];
      m[4 * r + c] = (float)a;
    }
}

// Case k of the test: triangles in every raster and cull mode (some crossing the near
// plane), lines, points, and a direct screen-space triangle list.
inline int user_case_count() { return 8; }

inline UserScene user_scene(int k) {
  UserScene sc;
  UserLcg g(1000 + (uint64_t)k);
  const int nv = 1200;
  sc.pos.resize(4 * nv);
  sc.attr.resize(3 * nv);
  for (int i = 0; i < nv; ++i) {
    sc.pos[4 * i + 0] = g.unit() * 4.0f - 2.0f;
    sc.pos[4 * i + 1] = g.unit() * 3.0f - 1.5f;
    sc.pos[4 * i + 2] = g.unit() * 5.0f - 2.5f;
    sc.pos[4 * i + 3] = g.unit();
    sc.attr[3 * i + 0] = g.next() | 0xff000000u;
    sc.attr[3 * i + 1] = user_float_bits(g.unit());
    sc.attr[3 * i + 2] = user_float_bits(g.unit());
  }
  user_camera(sc.mvp, 320.0 / 240.0, 0.5, 20.0, 3.0 + 0.25 * k, 0.1 * k);
  static const int modes[8][3] = {  // draw mode, cull, raster
      {2, 2, 0}, {2, 0, 1}, {2, 1, 2}, {2, 0, 0}, {2, 2, 1}, {1, 0, 0}, {0, 0, 0}, {2, 0, 2}};
  sc.draw_mode = modes[k][0];
  sc.cull = modes[k][1];
  sc.raster = modes[k][2];
  if (k == 4) {  // offset viewport, narrower depth range, scissor inside the target
    sc.viewport[0] = 16; sc.viewport[1] = 8; sc.viewport[2] = 288; sc.viewport[3] = 224;
    sc.scissor[0] = 24; sc.scissor[1] = 16; sc.scissor[2] = 272; sc.scissor[3] = 200;
    sc.depth_range[0] = 0.25f; sc.depth_range[1] = 0.75f;
  }
  const int per = sc.draw_mode == 2 ? 3 : (sc.draw_mode == 1 ? 2 : 1);
  const int nprims = sc.draw_mode == 2 ? 2500 : 900;  // 3 batches of 1024 triangles
  for (int p = 0; p < nprims; ++p) {
    const int a = (int)(g.next() % (uint32_t)nv);
    for (int j = 0; j < per; ++j) {
      // neighbouring vertices (small triangles) or anywhere (large ones)
      const int v = (g.next() & 3) ? (a + (int)(g.next() % 24u)) % nv : (int)(g.next() % (uint32_t)nv);
      sc.indices.push_back(j == 0 ? a : v);
    }
  }
  if (k == 7) {  // direct Rasterizer path: screen-space vertices, some primitives skipped (-1)
    sc.direct = true;
    sc.rv.assign(36 * nv, 0.0f);
    for (int i = 0; i < nv; ++i) {
      float* r = &sc.rv[36 * i];
      r[0] = g.unit() * 340.0f - 10.0f;
      r[1] = g.unit() * 260.0f - 10.0f;
      r[2] = g.unit();
      r[3] = 1.0f;
      for (int a = 0; a < 32; ++a) r[4 + a] = g.unit();
    }
    for (size_t p = 0; p + 3 <= sc.indices.size(); p += 3)
      if (g.next() % 16u == 0u) sc.indices[p] = -1;
  }
  return sc;
}
