// Test infrastructure: CPU restatement of the reference's hot path
// (VertexProcessor + Rasterizer of trenki2/SoftwareRenderer, src/renderer/).  It is the
// oracle the CUDA kernels are checked against on machines where the reference sources
// are absent, and the CPU baseline timed beside them.  It is pinned to the reference
// itself by tests/golden (fixtures generated by running the compiled reference through
// oracle/ref_harness.cpp).  Nothing in the product links or calls this file.
//
// Every floating-point expression keeps the reference's operation order; build with
// -ffp-contract=off (no FMA) so each operation rounds exactly once.
// OpenMP pragmas sit where the reference has them (Rasterizer.h:257, :369, :396).
#include <omp.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <vector>
#include <utility>
#include "../oracle_abi.h"

namespace port {

enum { kMaxVars = 16, kBlock = 8, kBatchPrims = 1024 };

// RasterizerVertex / VertexShaderOutput (IRasterizer.h:42-53, VertexConfig.h:37).
struct Vtx {
  float x, y, z, w;
  float avar[kMaxVars];
  float pvar[kMaxVars];
};

// EdgeEquation (EdgeEquation.h:31-84).
struct Edge {
  float a, b, c;
  bool tie;
  void init(const Vtx& v0, const Vtx& v1) {  // EdgeEquation.h:37-43
    a = v0.y - v1.y;
    b = v1.x - v0.x;
    c = -(a * (v0.x + v1.x) + b * (v0.y + v1.y)) / 2;
    tie = a != 0 ? a > 0 : b > 0;
  }
  float eval(float x, float y) const { return a * x + b * y + c; }
  bool test(float v) const { return v > 0 || (v == 0 && tie); }  // EdgeEquation.h:58-61
};

// ParameterEquation (ParameterEquation.h:29-75).
struct Param {
  float a, b, c;
  void init(float p0, float p1, float p2, const Edge& e0, const Edge& e1, const Edge& e2,
            float f) {  // ParameterEquation.h:36-48
    a = f * (p0 * e0.a + p1 * e1.a + p2 * e2.a);
    b = f * (p0 * e0.b + p1 * e1.b + p2 * e2.b);
    c = f * (p0 * e0.c + p1 * e1.c + p2 * e2.c);
  }
  float eval(float x, float y) const { return a * x + b * y + c; }
};

// TriangleEquations (TriangleEquations.h:35-72); the counts are the pixel shader's.
struct TriEq {
  float area2;
  Edge e0, e1, e2;
  Param z, invw, avar[kMaxVars], pvar[kMaxVars];
  void init(const Vtx& v0, const Vtx& v1, const Vtx& v2, int na, int np) {
    e0.init(v1, v2);
    e1.init(v2, v0);
    e2.init(v0, v1);
    area2 = e0.c + e1.c + e2.c;
    if (area2 <= 0) return;  // TriangleEquations.h:56-57
    const float factor = 1.0f / area2;
    z.init(v0.z, v1.z, v2.z, e0, e1, e2, factor);
    const float iw0 = 1.0f / v0.w, iw1 = 1.0f / v1.w, iw2 = 1.0f / v2.w;
    invw.init(iw0, iw1, iw2, e0, e1, e2, factor);
    for (int i = 0; i < na; ++i) avar[i].init(v0.avar[i], v1.avar[i], v2.avar[i], e0, e1, e2, factor);
    for (int i = 0; i < np; ++i)
      pvar[i].init(v0.pvar[i] * iw0, v1.pvar[i] * iw1, v2.pvar[i] * iw2, e0, e1, e2, factor);
  }
};

// PixelData (PixelData.h:35-146), state carried by incremental stepping.
template <class PS>
struct Pix {
  int x, y;
  float z, w, invw;
  float avar[kMaxVars], pvar[kMaxVars], pvarTemp[kMaxVars];
  const TriEq* eq = nullptr;  // PixelData::equations (set by init; null for points and lines)
  enum { NA = PS::AVarCount, NP = PS::PVarCount, IZ = PS::InterpolateZ,
         IW = PS::InterpolateW || PS::PVarCount > 0 };
  void init(const TriEq& e, float fx, float fy) {  // PixelData.h:61-79
    eq = &e;
    if (IZ) z = e.z.eval(fx, fy);
    if (IW) { invw = e.invw.eval(fx, fy); w = 1.0f / invw; }
    for (int i = 0; i < NA; ++i) avar[i] = e.avar[i].eval(fx, fy);
    for (int i = 0; i < NP; ++i) { pvarTemp[i] = e.pvar[i].eval(fx, fy); pvar[i] = pvarTemp[i] * w; }
  }
  void stepX(const TriEq& e) {  // PixelData.h:82-103
    if (IZ) z = z + e.z.a;
    if (IW) { invw = invw + e.invw.a; w = 1.0f / invw; }
    for (int i = 0; i < NA; ++i) avar[i] = avar[i] + e.avar[i].a;
    for (int i = 0; i < NP; ++i) { pvarTemp[i] = pvarTemp[i] + e.pvar[i].a; pvar[i] = pvarTemp[i] * w; }
  }
  void stepY(const TriEq& e) {  // PixelData.h:106-125
    if (IZ) z = z + e.z.b;
    if (IW) { invw = invw + e.invw.b; w = 1.0f / invw; }
    for (int i = 0; i < NA; ++i) avar[i] = avar[i] + e.avar[i].b;
    for (int i = 0; i < NP; ++i) { pvarTemp[i] = pvarTemp[i] + e.pvar[i].b; pvar[i] = pvarTemp[i] * w; }
  }
};

// PixelData::computePerspectiveDerivatives (PixelData.h:128-145) for the shared shaders
// (found by argument-dependent lookup).
template <class PS>
void swr_persp_deriv(const Pix<PS>& p, int i, float& ddx, float& ddy) {
  if (!p.eq) {
    ddx = ddy = 0.0f;
    return;
  }
  const float pv[3] = {p.eq->pvar[i].a, p.eq->pvar[i].b, p.eq->pvar[i].c};
  const float iw[3] = {p.eq->invw.a, p.eq->invw.b, p.eq->invw.c};
  swr_persp_deriv_eq(pv, iw, p.x, p.y, ddx, ddy);
}

struct Counters {
  uint64_t frags = 0, outside = 0, prims = 0, batches = 0;
  int32_t* prim_src = nullptr;  // optional: source triangle per primitive id
  uint64_t prim_src_cap = 0;
  bool src_overflow = false;
};

// Rasterizer restatement (Rasterizer.h:52-446) for pixel shader PS.
template <class PS>
struct Raster {
  int minX, maxX, minY, maxY;  // scissor (Rasterizer::setScissorRect, Rasterizer.h:81-87)
  int mode;                    // 0 Span, 1 Block, 2 Adaptive
  const SwrUniforms* u;
  Counters* cnt;

  // One drawPixel call (PixelShaderBase.h:116) applied to the pixel's framebuffer.
  template <class PD>
  void emit(const PD& p, int prim, uint64_t& frags, uint64_t& outside) const {
    if (p.x < 0 || p.y < 0 || p.x >= u->width || p.y >= u->height) { outside++; return; }
    typename PS::State s;
    PS::load(s, p.x, p.y, *u);
    PS::drawPixel(p, prim, s, *u);
    PS::store(s, p.x, p.y, *u);
    frags++;
  }

  bool scissor(float x, float y) const {  // Rasterizer.h:144-147
    return x >= minX && x < maxX && y >= minY && y < maxY;
  }

  // Rasterizer::pixelDataFromVertex (Rasterizer.h:161-173).
  Pix<PS> fromVertex(const Vtx& v) const {
    Pix<PS> p;
    p.x = (int)v.x;
    p.y = (int)v.y;
    if (PS::InterpolateZ) p.z = v.z;
    if (PS::InterpolateW) { p.w = v.w; p.invw = 1.0f / v.w; }
    for (int i = 0; i < PS::AVarCount; ++i) p.avar[i] = v.avar[i];
    for (int i = 0; i < PS::PVarCount; ++i) p.pvar[i] = v.pvar[i];
    return p;
  }

  void point(const Vtx& v, int prim) const {  // Rasterizer.h:150-158
    if (!scissor(v.x, v.y)) return;
    emit(fromVertex(v), prim, cnt->frags, cnt->outside);
  }

  void line(const Vtx& v0, const Vtx& v1, int prim) const {  // Rasterizer.h:176-222
    const int adx = abs((int)v1.x - (int)v0.x);
    const int ady = abs((int)v1.y - (int)v0.y);
    int steps = adx > ady ? adx : ady;
    Vtx st;
    st.x = (v1.x - v0.x) / steps;
    st.y = (v1.y - v0.y) / steps;
    if (PS::InterpolateZ) st.z = (v1.z - v0.z) / steps;
    if (PS::InterpolateW) st.w = (v1.w - v0.w) / steps;
    for (int i = 0; i < PS::AVarCount; ++i) st.avar[i] = (v1.avar[i] - v0.avar[i]) / steps;
    for (int i = 0; i < PS::PVarCount; ++i) st.pvar[i] = (v1.pvar[i] - v0.pvar[i]) / steps;
    Vtx v = v0;
    while (steps-- > 0) {
      Pix<PS> p = fromVertex(v);
      if (scissor(v.x, v.y)) emit(p, prim, cnt->frags, cnt->outside);
      v.x += st.x;
      v.y += st.y;
      if (PS::InterpolateZ) v.z += st.z;
      if (PS::InterpolateW) v.w += st.w;
      for (int i = 0; i < PS::AVarCount; ++i) v.avar[i] += st.avar[i];
      for (int i = 0; i < PS::PVarCount; ++i) v.pvar[i] += st.pvar[i];
    }
  }

  // PixelShaderBase::drawSpan (PixelShaderBase.h:96-112).
  void span(const TriEq& e, int x, int y, int x2, int prim, uint64_t& frags, uint64_t& outside) const {
    Pix<PS> p;
    p.y = y;
    p.init(e, x + 0.5f, y + 0.5f);
    while (x < x2) {
      p.x = x;
      emit(p, prim, frags, outside);
      p.stepX(e);
      x++;
    }
  }

  // Per-pixel edge values stepped like EdgeData (EdgeData.h:37-80).
  struct EdgeVals {
    float v0, v1, v2;
    void init(const TriEq& e, float x, float y) { v0 = e.e0.eval(x, y); v1 = e.e1.eval(x, y); v2 = e.e2.eval(x, y); }
    void stepX(const TriEq& e) { v0 = v0 + e.e0.a; v1 = v1 + e.e1.a; v2 = v2 + e.e2.a; }
    void stepY(const TriEq& e) { v0 = v0 + e.e0.b; v1 = v1 + e.e1.b; v2 = v2 + e.e2.b; }
    void stepX(const TriEq& e, float s) { v0 = v0 + e.e0.a * s; v1 = v1 + e.e1.a * s; v2 = v2 + e.e2.a * s; }
    void stepY(const TriEq& e, float s) { v0 = v0 + e.e0.b * s; v1 = v1 + e.e1.b * s; v2 = v2 + e.e2.b * s; }
    bool test(const TriEq& e) const { return e.e0.test(v0) && e.e1.test(v1) && e.e2.test(v2); }
  };

  // PixelShaderBase::drawBlock<TestEdges> (PixelShaderBase.h:55-94).  The row copy
  // (copyPixelData, PixelShaderBase.h:122-136) carries the stepped row-start state.
  template <bool TestEdges>
  void block(const TriEq& e, int x, int y, int prim, uint64_t& frags, uint64_t& outside) const {
    const float xf = x + 0.5f, yf = y + 0.5f;
    Pix<PS> po;
    po.init(e, xf, yf);
    EdgeVals eo;
    if (TestEdges) eo.init(e, xf, yf);
    for (int yy = y; yy < y + kBlock; yy++) {
      Pix<PS> pi = po;
      EdgeVals ei = eo;
      for (int xx = x; xx < x + kBlock; xx++) {
        if (!TestEdges || ei.test(e)) {
          pi.x = xx;
          pi.y = yy;
          emit(pi, prim, frags, outside);
        }
        pi.stepX(e);
        if (TestEdges) ei.stepX(e);
      }
      po.stepY(e);
      if (TestEdges) eo.stepY(e);
    }
  }

  void triBlock(const Vtx& v0, const Vtx& v1, const Vtx& v2, int prim) const {  // Rasterizer.h:225-306
    TriEq e;
    e.init(v0, v1, v2, PS::AVarCount, PS::PVarCount);
    if (e.area2 <= 0) return;
    int bx0 = (int)swr_minf(swr_minf(v0.x, v1.x), v2.x);
    int bx1 = (int)swr_maxf(swr_maxf(v0.x, v1.x), v2.x);
    int by0 = (int)swr_minf(swr_minf(v0.y, v1.y), v2.y);
    int by1 = (int)swr_maxf(swr_maxf(v0.y, v1.y), v2.y);
    bx0 = swr_maxi(bx0, minX);
    bx1 = swr_mini(bx1, maxX);
    by0 = swr_maxi(by0, minY);
    by1 = swr_mini(by1, maxY);
    bx0 &= ~(kBlock - 1);
    bx1 &= ~(kBlock - 1);
    by0 &= ~(kBlock - 1);
    by1 &= ~(kBlock - 1);
    const float s = kBlock - 1;
    const int stepsX = (bx1 - bx0) / kBlock + 1;
    const int stepsY = (by1 - by0) / kBlock + 1;
    uint64_t frags = 0, outside = 0;
    auto blk = [&](int i, uint64_t& frags, uint64_t& outside) {
      const int sx = i % stepsX, sy = i / stepsX;
      const int x = bx0 + sx * kBlock, y = by0 + sy * kBlock;
      const float xf = x + 0.5f, yf = y + 0.5f;
      EdgeVals c00; c00.init(e, xf, yf);
      EdgeVals c01 = c00; c01.stepY(e, s);
      EdgeVals c10 = c00; c10.stepX(e, s);
      EdgeVals c11 = c01; c11.stepX(e, s);
      const bool a0 = e.e0.test(c00.v0), a1 = e.e1.test(c00.v1), a2 = e.e2.test(c00.v2);
      const bool b0 = e.e0.test(c01.v0), b1 = e.e1.test(c01.v1), b2 = e.e2.test(c01.v2);
      const bool d0 = e.e0.test(c10.v0), d1 = e.e1.test(c10.v1), d2 = e.e2.test(c10.v2);
      const bool f0 = e.e0.test(c11.v0), f1 = e.e1.test(c11.v1), f2 = e.e2.test(c11.v2);
      const int inside = (a0 && a1 && a2) + (b0 && b1 && b2) + (d0 && d1 && d2) + (f0 && f1 && f2);
      if (inside == 0) {
        // Rasterizer.h:287-293: ((t0 == t1) == t2) per corner.
        const bool sa = (a0 == a1) == a2, sb = (b0 == b1) == b2;
        const bool sd = (d0 == d1) == d2, sf = (f0 == f1) == f2;
        if (!sa || !sb || !sd || !sf) block<true>(e, x, y, prim, frags, outside);
      } else if (inside == 4) {
        block<false>(e, x, y, prim, frags, outside);
      } else {
        block<true>(e, x, y, prim, frags, outside);
      }
    };
    // The reference's OpenMP loop over blocks (Rasterizer.h:257); a one-thread run skips
    // the team fork per triangle, as the reference built without OpenMP does.
    if (omp_get_max_threads() > 1) {
#pragma omp parallel for reduction(+ : frags, outside)
      for (int i = 0; i < stepsX * stepsY; ++i) blk(i, frags, outside);
    } else {
      for (int i = 0; i < stepsX * stepsY; ++i) blk(i, frags, outside);
    }
    cnt->frags += frags;
    cnt->outside += outside;
  }

  // drawBottomFlatTriangle (Rasterizer.h:361-385).
  void bottomFlat(const TriEq& e, const Vtx& v0, const Vtx& v1, const Vtx& v2, int prim) const {
    const float is1 = (v1.x - v0.x) / (v1.y - v0.y);
    const float is2 = (v2.x - v0.x) / (v2.y - v0.y);
    uint64_t frags = 0, outside = 0;
    const int y0 = int(v0.y + 0.5f), y1 = int(v1.y + 0.5f);
    auto row = [&](int y, uint64_t& frags, uint64_t& outside) {
      const float dy = (y - v0.y) + 0.5f;
      const float cx1 = v0.x + is1 * dy + 0.5f;
      const float cx2 = v0.x + is2 * dy + 0.5f;
      const int xl = swr_maxi(minX, (int)cx1);
      const int xr = swr_mini(maxX, (int)cx2);
      span(e, xl, y, xr, prim, frags, outside);
    };
    if (omp_get_max_threads() > 1) {  // OpenMP over scanlines (Rasterizer.h:369)
#pragma omp parallel for reduction(+ : frags, outside)
      for (int y = y0; y < y1; y++) row(y, frags, outside);
    } else {
      for (int y = y0; y < y1; y++) row(y, frags, outside);
    }
    cnt->frags += frags;
    cnt->outside += outside;
  }

  // drawTopFlatTriangle (Rasterizer.h:388-411).
  void topFlat(const TriEq& e, const Vtx& v0, const Vtx& v1, const Vtx& v2, int prim) const {
    const float is1 = (v2.x - v0.x) / (v2.y - v0.y);
    const float is2 = (v2.x - v1.x) / (v2.y - v1.y);
    uint64_t frags = 0, outside = 0;
    const int ytop = int(v2.y - 0.5f), yend = int(v0.y - 0.5f);
    auto row = [&](int y, uint64_t& frags, uint64_t& outside) {
      const float dy = (y - v2.y) + 0.5f;
      const float cx1 = v2.x + is1 * dy + 0.5f;
      const float cx2 = v2.x + is2 * dy + 0.5f;
      const int xl = swr_maxi(minX, (int)cx1);
      const int xr = swr_mini(maxX, (int)cx2);
      span(e, xl, y, xr, prim, frags, outside);
    };
    if (omp_get_max_threads() > 1) {  // OpenMP over scanlines (Rasterizer.h:396)
#pragma omp parallel for reduction(+ : frags, outside)
      for (int y = ytop; y > yend; y--) row(y, frags, outside);
    } else {
      for (int y = ytop; y > yend; y--) row(y, frags, outside);
    }
    cnt->frags += frags;
    cnt->outside += outside;
  }

  void triSpan(const Vtx& v0, const Vtx& v1, const Vtx& v2, int prim) const {  // Rasterizer.h:309-358
    TriEq e;
    e.init(v0, v1, v2, PS::AVarCount, PS::PVarCount);
    if (e.area2 <= 0) return;
    const Vtx* t = &v0;
    const Vtx* m = &v1;
    const Vtx* b = &v2;
    if (t->y > m->y) std::swap(t, m);
    if (m->y > b->y) std::swap(m, b);
    if (t->y > m->y) std::swap(t, m);
    const float dy = b->y - t->y;
    const float iy = m->y - t->y;
    if (m->y == t->y) {
      const Vtx* l = m;
      const Vtx* r = t;
      if (l->x > r->x) std::swap(l, r);
      topFlat(e, *l, *r, *b, prim);
    } else if (m->y == b->y) {
      const Vtx* l = m;
      const Vtx* r = b;
      if (l->x > r->x) std::swap(l, r);
      bottomFlat(e, *t, *l, *r, prim);
    } else {
      // Only x and y of the split vertex reach the span walkers.
      Vtx v4;
      v4.y = m->y;
      v4.x = t->x + ((b->x - t->x) / dy) * iy;
      const Vtx* l = m;
      const Vtx* r = &v4;
      if (l->x > r->x) std::swap(l, r);
      bottomFlat(e, *t, *l, *r, prim);
      topFlat(e, *l, *r, *b, prim);
    }
  }

  void triangle(const Vtx& v0, const Vtx& v1, const Vtx& v2, int prim) const {  // Rasterizer.h:414-446
    if (mode == 0) {
      triSpan(v0, v1, v2, prim);
    } else if (mode == 1) {
      triBlock(v0, v1, v2, prim);
    } else {
      const float bminX = swr_minf(swr_minf(v0.x, v1.x), v2.x);
      const float bmaxX = swr_maxf(swr_maxf(v0.x, v1.x), v2.x);
      const float bminY = swr_minf(swr_minf(v0.y, v1.y), v2.y);
      const float bmaxY = swr_maxf(swr_maxf(v0.y, v1.y), v2.y);
      const float orient = (bmaxX - bminX) / (bmaxY - bminY);
      if (orient > 0.4 && orient < 1.6) triBlock(v0, v1, v2, prim);
      else triSpan(v0, v1, v2, prim);
    }
  }

  // Rasterizer::draw{Point,Line,Triangle}List (Rasterizer.h:116-141).
  void list(int draw_mode, const Vtx* v, const int* idx, size_t n) const {
    if (draw_mode == 0) {
      for (size_t i = 0; i < n; ++i) {
        if (idx[i] == -1) continue;
        point(v[idx[i]], (int)cnt->prims++);
      }
    } else if (draw_mode == 1) {
      for (size_t i = 0; i + 2 <= n; i += 2) {
        if (idx[i] == -1) continue;
        line(v[idx[i]], v[idx[i + 1]], (int)cnt->prims++);
      }
    } else {
      for (size_t i = 0; i + 3 <= n; i += 3) {
        if (idx[i] == -1) continue;
        triangle(v[idx[i]], v[idx[i + 1]], v[idx[i + 2]], (int)cnt->prims++);
      }
    }
  }
};

typedef void (*ListFn)(const void* raster, int draw_mode, const Vtx* v, const int* idx, size_t n);

template <class PS>
void list_thunk(const void* r, int dm, const Vtx* v, const int* idx, size_t n) {
  ((const Raster<PS>*)r)->list(dm, v, idx, n);
}

// Helper::interpolateVertex (PolyClipper.h:34-48).
static Vtx lerp_vtx(const Vtx& v0, const Vtx& v1, float t, int na, int np) {
  Vtx r;
  r.x = v0.x * (1.0f - t) + v1.x * t;
  r.y = v0.y * (1.0f - t) + v1.y * t;
  r.z = v0.z * (1.0f - t) + v1.z * t;
  r.w = v0.w * (1.0f - t) + v1.w * t;
  for (int i = 0; i < na; ++i) r.avar[i] = v0.avar[i] * (1.0f - t) + v1.avar[i] * t;
  for (int i = 0; i < np; ++i) r.pvar[i] = v0.pvar[i] * (1.0f - t) + v1.pvar[i] * t;
  return r;
}

static inline float plane_dist(const Vtx& v, float a, float b, float c, float d) {
  return a * v.x + b * v.y + c * v.z + d * v.w;
}

static inline int sgnf(float v) { return (0.0f < v) - (v < 0.0f); }

// Outcodes (VertexProcessor.cpp:122-132).
static int outcode(const Vtx& v) {
  int m = 0;
  if (v.w - v.x < 0) m |= 0x01;
  if (v.x + v.w < 0) m |= 0x02;
  if (v.w - v.y < 0) m |= 0x04;
  if (v.y + v.w < 0) m |= 0x08;
  if (v.w - v.z < 0) m |= 0x10;
  if (v.z + v.w < 0) m |= 0x20;
  return m;
}

static const float kPlanes[6][4] = {{-1, 0, 0, 1}, {1, 0, 0, 1}, {0, -1, 0, 1},
                                    {0, 1, 0, 1},  {0, 0, -1, 1}, {0, 0, 1, 1}};

// VertexProcessor state and per-batch processing (VertexProcessor.cpp:78-377).
struct VP {
  float px, py, ox, oy, dn, df;
  int cull;
  int na, np;
  int draw_mode;
  std::vector<Vtx> verts;
  std::vector<int> idx;
  std::vector<int> src;  // per triangle of idx: its source triangle in the draw's index list
  std::vector<int> mask;
  std::vector<char> done;
  const void* raster;
  ListFn list;
  Counters* cnt;

  // PolyClipper::clipToPlane (PolyClipper.cpp:45-81) over index lists.
  void clip_poly(std::vector<int>& in, std::vector<int>& out, const float* pl) {
    if (in.size() < 3) return;
    out.clear();
    int iprev = in[0];
    in.push_back(iprev);
    float dprev = plane_dist(verts[iprev], pl[0], pl[1], pl[2], pl[3]);
    for (size_t i = 1; i < in.size(); ++i) {
      const int icur = in[i];
      const float dcur = plane_dist(verts[icur], pl[0], pl[1], pl[2], pl[3]);
      if (dprev >= 0) out.push_back(iprev);
      if (sgnf(dcur) != sgnf(dprev)) {
        const float t = dcur < 0 ? dprev / (dprev - dcur) : -dprev / (dcur - dprev);
        const Vtx nv = lerp_vtx(verts[iprev], verts[icur], t, na, np);
        verts.push_back(nv);
        out.push_back((int)verts.size() - 1);
      }
      iprev = icur;
      dprev = dcur;
    }
    std::swap(in, out);
  }

  void compute_masks() {
    mask.assign(verts.size(), 0);
    for (size_t i = 0; i < verts.size(); ++i) mask[i] = outcode(verts[i]);
  }

  void clip_triangles() {  // VertexProcessor.cpp:217-263
    compute_masks();
    std::vector<int> poly, tmp;
    const size_t n = idx.size();
    for (size_t i = 0; i < n; i += 3) {
      const int i0 = idx[i], i1 = idx[i + 1], i2 = idx[i + 2];
      const int m = mask[i0] | mask[i1] | mask[i2];
      poly.assign({i0, i1, i2});
      for (int p = 0; p < 6; ++p)
        if (m & (1 << p)) clip_poly(poly, tmp, kPlanes[p]);
      if (poly.size() < 3) {
        idx[i] = idx[i + 1] = idx[i + 2] = -1;
        continue;
      }
      idx[i] = poly[0];
      idx[i + 1] = poly[1];
      idx[i + 2] = poly[2];
      for (size_t k = 3; k < poly.size(); ++k) {
        idx.push_back(poly[0]);
        idx.push_back(poly[k - 1]);
        idx.push_back(poly[k]);
        src.push_back(src[i / 3]);
      }
    }
  }

  void clip_lines() {  // VertexProcessor.cpp:167-215 with LineClipper.cpp:30-56
    compute_masks();
    for (size_t i = 0; i < idx.size(); i += 2) {
      const int i0 = idx[i], i1 = idx[i + 1];
      const Vtx v0 = verts[i0], v1 = verts[i1];
      const int m = mask[i0] | mask[i1];
      float t0 = 0.0f, t1 = 1.0f;
      bool gone = false;
      for (int p = 0; p < 6 && !gone; ++p) {
        if (!(m & (1 << p))) continue;
        const float* pl = kPlanes[p];
        const float d0 = plane_dist(v0, pl[0], pl[1], pl[2], pl[3]);
        const float d1 = plane_dist(v1, pl[0], pl[1], pl[2], pl[3]);
        const bool n0 = d0 < 0, n1 = d1 < 0;
        if (n0 && n1) { gone = true; break; }
        if (n0) {
          const float t = -d0 / (d1 - d0);
          t0 = (t0 < t) ? t : t0;
        } else {
          const float t = d0 / (d0 - d1);
          t1 = (t < t1) ? t : t1;
        }
      }
      if (gone) {
        idx[i] = idx[i + 1] = -1;
        continue;
      }
      if (mask[i0]) {
        verts.push_back(lerp_vtx(v0, v1, t0, na, np));
        idx[i] = (int)verts.size() - 1;
      }
      if (mask[i1]) {
        verts.push_back(lerp_vtx(v0, v1, t1, na, np));
        idx[i + 1] = (int)verts.size() - 1;
      }
    }
  }

  void clip_points() {  // VertexProcessor.cpp:152-165
    compute_masks();
    for (size_t i = 0; i < idx.size(); ++i)
      if (mask[idx[i]]) idx[i] = -1;
  }

  void transform() {  // VertexProcessor.cpp:347-377
    done.assign(verts.size(), 0);
    for (size_t i = 0; i < idx.size(); ++i) {
      const int k = idx[i];
      if (k == -1 || done[k]) continue;
      Vtx& v = verts[k];
      const float iw = 1.0f / v.w;
      v.x *= iw;
      v.y *= iw;
      v.z *= iw;
      v.x = (px * v.x + ox);
      v.y = (py * -v.y + oy);
      v.z = 0.5f * (df - dn) * v.z + 0.5f * (dn + df);
      done[k] = 1;
    }
  }

  void cull_triangles() {  // VertexProcessor.cpp:319-345
    for (size_t i = 0; i + 3 <= idx.size(); i += 3) {
      if (idx[i] == -1) continue;
      const Vtx& v0 = verts[idx[i]];
      const Vtx& v1 = verts[idx[i + 1]];
      const Vtx& v2 = verts[idx[i + 2]];
      const float facing = (v0.x - v1.x) * (v2.y - v1.y) - (v2.x - v1.x) * (v0.y - v1.y);
      if (facing < 0) {
        if (cull == 2) idx[i] = idx[i + 1] = idx[i + 2] = -1;
      } else {
        if (cull == 1) idx[i] = idx[i + 1] = idx[i + 2] = -1;
        else std::swap(idx[i], idx[i + 2]);
      }
    }
  }

  void process() {  // VertexProcessor::processPrimitives (VertexProcessor.cpp:281-317)
    cnt->batches++;
    if (draw_mode == 0) clip_points();
    else if (draw_mode == 1) clip_lines();
    else clip_triangles();
    transform();
    if (draw_mode == 2) cull_triangles();
    if (draw_mode == 2 && cnt->prim_src) {
      // the rasterizer numbers the surviving triangles in idx order
      uint64_t k = cnt->prims;
      for (size_t i = 0; i + 3 <= idx.size(); i += 3) {
        if (idx[i] == -1) continue;
        if (k < cnt->prim_src_cap) cnt->prim_src[k] = src[i / 3];
        else cnt->src_overflow = true;
        ++k;
      }
    }
    list(raster, draw_mode, verts.data(), idx.data(), idx.size());
  }
};

template <class VS>
void draw_elements(VP& vp, const OracleDraw& d) {  // VertexProcessor.cpp:78-120
  vp.verts.clear();
  vp.idx.clear();
  vp.src.clear();
  int cache_in[16], cache_out[16];  // VertexCache (VertexCache.h:29-63)
  for (int i = 0; i < 16; ++i) cache_in[i] = -1;
  const int per = d.draw_mode == 0 ? 1 : (d.draw_mode == 1 ? 2 : 3);
  for (uint64_t i = 0; i < d.count; ++i) {
    const int index = d.indices[i];
    const int slot = index % 16;
    int out = cache_in[slot] == index ? cache_out[slot] : -1;
    if (out == -1) {
      SwrVertexInput in;
      for (int a = 0; a < VS::AttribCount; ++a)
        in.p[a] = (const char*)d.attrib[a] + (size_t)d.attrib_stride[a] * (size_t)index;
      out = (int)vp.verts.size();
      vp.verts.resize(vp.verts.size() + 1);
      VS::processVertex(in, &vp.verts.back(), *d.uniforms);
      cache_in[slot] = index;
      cache_out[slot] = out;
    }
    vp.idx.push_back(out);
    if (per == 3 && i % 3 == 2) vp.src.push_back((int)(i / 3));
    if ((int)(vp.idx.size() / per) >= kBatchPrims) {
      vp.process();
      vp.verts.clear();
      vp.idx.clear();
      vp.src.clear();
      for (int k = 0; k < 16; ++k) cache_in[k] = -1;
    }
  }
  vp.process();
}

template <class PS>
int run_ps(const OracleDraw& d, Counters& cnt) {
  Raster<PS> r;
  r.minX = d.scissor[0];
  r.minY = d.scissor[1];
  r.maxX = d.scissor[0] + d.scissor[2];
  r.maxY = d.scissor[1] + d.scissor[3];
  r.mode = d.raster_mode;
  r.u = d.uniforms;
  r.cnt = &cnt;
  if (d.raster_vertices) {
    // Direct Rasterizer path: vertices are already in screen space.
    uint64_t maxi = 0;
    for (uint64_t i = 0; i < d.count; ++i)
      if (d.indices[i] >= 0 && (uint64_t)d.indices[i] + 1 > maxi) maxi = (uint64_t)d.indices[i] + 1;
    std::vector<Vtx> v(maxi);
    if (maxi) memcpy(v.data(), d.raster_vertices, maxi * sizeof(Vtx));
    r.list(d.draw_mode, v.data(), d.indices, (size_t)d.count);
    cnt.batches = 0;
    return 0;
  }
  VP vp;
  vp.px = d.viewport[2] / 2.0f;  // VertexProcessor::setViewport (VertexProcessor.cpp:43-54)
  vp.py = d.viewport[3] / 2.0f;
  vp.ox = (d.viewport[0] + vp.px);
  vp.oy = (d.viewport[1] + vp.py);
  vp.dn = d.depth_range[0];
  vp.df = d.depth_range[1];
  vp.cull = d.cull_mode;
  vp.draw_mode = d.draw_mode;
  vp.raster = &r;
  vp.list = &list_thunk<PS>;
  vp.cnt = &cnt;
  switch (d.vs_id) {
    case SWR_VS_POS_UV: vp.na = VsPosUV::AVarCount; vp.np = VsPosUV::PVarCount; draw_elements<VsPosUV>(vp, d); break;
    case SWR_VS_POS_NRM_UV: vp.na = VsPosNrmUV::AVarCount; vp.np = VsPosNrmUV::PVarCount; draw_elements<VsPosNrmUV>(vp, d); break;
    case SWR_VS_POS_RGB: vp.na = VsPosRGB::AVarCount; vp.np = VsPosRGB::PVarCount; draw_elements<VsPosRGB>(vp, d); break;
    case SWR_VS_POS_RGB_AFFINE: vp.na = VsPosRGBAffine::AVarCount; vp.np = VsPosRGBAffine::PVarCount; draw_elements<VsPosRGBAffine>(vp, d); break;
    case SWR_VS_POS_RGB_UV: vp.na = VsPosRGBUV::AVarCount; vp.np = VsPosRGBUV::PVarCount; draw_elements<VsPosRGBUV>(vp, d); break;
    default: return 2;
  }
  return 0;
}

}  // namespace port

#ifdef _OPENMP
#include <omp.h>
#endif

extern "C" int oracle_draw(const OracleDraw* d, OracleStats* st) {
  using namespace port;
  if (!d || !d->uniforms) return 1;
  const uint64_t per = d->draw_mode == 0 ? 1 : (d->draw_mode == 1 ? 2 : 3);
  if (d->draw_mode < 0 || d->draw_mode > 2 || d->count % per) return 1;
  for (uint64_t i = 0; i < d->count; ++i)
    if (d->indices[i] < (d->raster_vertices ? -1 : 0)) return 1;
#ifdef _OPENMP
  if (d->threads > 0) omp_set_num_threads(d->threads);
#endif
  Counters cnt;
  cnt.prim_src = d->raster_vertices ? nullptr : d->prim_src;
  cnt.prim_src_cap = d->prim_src_cap;
  int rc;
  switch (d->ps_id) {
    case SWR_PS_TEX_NEAREST: rc = run_ps<PsTexNearest>(*d, cnt); break;
    case SWR_PS_LAMBERT: rc = run_ps<PsLambert>(*d, cnt); break;
    case SWR_PS_VCOLOR: rc = run_ps<PsVColor>(*d, cnt); break;
    case SWR_PS_VCOLOR_AFFINE: rc = run_ps<PsVColorAffine>(*d, cnt); break;
    case SWR_PS_LAMBERT_TEX: rc = run_ps<PsLambertTex>(*d, cnt); break;
    case SWR_PS_DIFF: rc = run_ps<PsDiff>(*d, cnt); break;
    case SWR_PS_TEX_MIP: rc = d->draw_mode == 2 ? run_ps<PsTexMip>(*d, cnt) : 1; break;
    case SWR_PS_PERSP_DERIV: rc = d->draw_mode == 2 ? run_ps<PsPerspDeriv>(*d, cnt) : 1; break;
    default: rc = 2;
  }
  if (st) {
    st->fragments = cnt.frags;
    st->outside = cnt.outside;
    st->primitives = cnt.prims;
    st->batches = cnt.batches;
  }
  if (!rc && cnt.src_overflow) rc = 3;
  return rc;
}

extern "C" float oracle_fold(float v, float a, int k) { return swr_fold(v, a, k); }

// swr_log2 and the mip-mapped sampler exposed for the tests of the texture subsystem.
extern "C" void oracle_log2(const float* x, float* out, uint64_t n) {
  for (uint64_t i = 0; i < n; ++i) out[i] = swr_log2(x[i]);
}

// swr_tex_sample (the sampler the GPU shader PsTexMip runs) over a mip chain of a w x h
// texture: q holds n records {u, v, dudx, dvdx, dudy, dvdy}.
extern "C" void oracle_tex_sample(const uint32_t* chain, int w, int h, int max_aniso, const float* q, uint32_t* out,
                                  uint64_t n) {
  SwrUniforms u;
  memset(&u, 0, sizeof(u));
  u.tex = chain;
  u.tex_w = w;
  u.tex_h = h;
  u.max_aniso = max_aniso;
  for (uint64_t i = 0; i < n; ++i) {
    const float* r = q + 6 * i;
    out[i] = swr_tex_sample(u, r[0], r[1], r[2], r[3], r[4], r[5]);
  }
}

// Randomized check of swr_fold against plain serial stepping: returns the number of
// (v, a, k) cases where they differ (NaN results compare equal).  Cases mix arbitrary bit
// patterns, moderate magnitudes, powers of two and their neighbours (binade edges),
// subnormals, and increments placed on or next to half-ulp ties of v.
extern "C" uint64_t oracle_fold_selftest(uint64_t iters, uint64_t seed) {
  uint64_t s = seed * 0x9E3779B97F4A7C15ull + 88172645463325252ull;
  auto rnd = [&]() { s ^= s << 13; s ^= s >> 7; s ^= s << 17; return s; };
  auto bits = [](uint32_t b) { float f; memcpy(&f, &b, 4); return f; };
  auto pick = [&]() -> float {
    switch (rnd() % 7) {
      case 0: return bits((uint32_t)rnd());
      case 1: return bits(((uint32_t)rnd() & 0x807fffffu) | ((uint32_t)(100 + rnd() % 56) << 23));
      case 2: return (float)((double)(rnd() % 2000001) / 1000.0 - 1000.0);
      case 3: {
        float f = bits((uint32_t)(97 + rnd() % 60) << 23);
        if (rnd() & 1) f = -f;
        uint32_t b; memcpy(&b, &f, 4);
        b += (uint32_t)(rnd() % 3) - 1;
        return bits(b);
      }
      case 4: return bits(((uint32_t)rnd() & 0x80000000u) | (uint32_t)(rnd() % 64));
      case 5: return (float)((double)((int)(rnd() % 200001) - 100000) / (double)(1u << (rnd() % 30)));
      default: return bits(((uint32_t)rnd() & 0x807fffffu) | ((uint32_t)(110 + rnd() % 30) << 23));
    }
  };
  uint64_t bad = 0;
  for (uint64_t it = 0; it < iters; ++it) {
    float v = pick(), a = pick();
    if (rnd() % 4 == 0) {  // increments of (q + 1/2 or q + f) ulps of v: ties and near-ties
      uint32_t vb; memcpy(&vb, &v, 4);
      const int e = (int)((vb >> 23) & 0xff) - 150;
      const double u = e > -150 ? ldexp(1.0, e) : ldexp(1.0, -149);
      const double q = (double)(rnd() % 64) + ((rnd() & 1) ? 0.5 : (double)(rnd() % 1000) / 1000.0);
      a = (float)(q * u * (double)(1u << (rnd() % 5)));
      if (rnd() & 1) a = -a;
    }
    const int k = (int)(rnd() % ((rnd() % 3 == 0) ? 5000 : 300));
    float ref = v;
    for (int i = 0; i < k; ++i) ref = ref + a;
    const float got = swr_fold(v, a, k);
    uint32_t rb, gb;
    memcpy(&rb, &ref, 4);
    memcpy(&gb, &got, 4);
    if (rb != gb && !(ref != ref && got != got)) bad++;
  }
  return bad;
}
