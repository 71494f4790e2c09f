// Test infrastructure: CPU reference of the differentiable-rendering backward, in double.
//
// The forward is the pixel shader PsDiff (swr_programs.h): colour = (vertex rgb) * bilinear
// RGBA32F texel, with rgb and uv interpolated perspective-correct.  With visibility held
// fixed (the winner buffer and the primitive-source map of a forward draw), the colour of
// a covered pixel is a smooth function of the vertex records and the texels; this file
// evaluates it directly from the triangle's clip-space vertices and differentiates it.
//
// Perspective-correct barycentrics in homogeneous window coordinates: with clip
// positions (X, Y, Z, W), viewport (px, py, ox, oy) as VertexProcessor::setViewport sets
// it (VertexProcessor.cpp:43-54; window x = px * X/W + ox, y = -py * Y/W + oy,
// VertexProcessor.cpp:370-376) and the pixel centre (xp, yp) = (x + 0.5, y + 0.5)
// (PixelShaderBase.h:68-111 evaluate at +0.5), let
//   D_k = (px * X_k + (ox - xp) * W_k,  -py * Y_k + (oy - yp) * W_k)   ( = W_k * (s_k - p) )
//   e_0 = D_1 x D_2,  e_1 = D_2 x D_0,  e_2 = D_0 x D_1,  b_k = e_k / (e_0 + e_1 + e_2),
// the weights of the perspective-correct interpolation that PixelData's 1/w stepping
// evaluates (PixelData.h:84-103).  No division by W is needed, so the form also holds for
// triangles that clipping split.  The bilinear sampler follows the reference's example
// texture (Texture.h:146-181): px = u * (w - 1) on u clamped to [0, 1], x0 = floor,
// x1 = min(w - 1, x0 + 1).
//
// Only tests use this file.
#include <math.h>
#include <stdint.h>
#include <string.h>

#include <vector>

#include "../oracle_abi.h"

#ifdef _OPENMP
#include <omp.h>
#endif

namespace {

struct Eval {
  const OracleDiffScene* s;
  int kind;        // perturbed parameter: -1 none, 0 vertex-record component, 1 texel component
  uint64_t index;  // 8 * vertex + component, or 4 * texel + channel
  double delta;

  double vtx(uint64_t v, int c) const {
    const uint64_t k = v * 8 + (uint64_t)c;
    return s->vertices[k] + (kind == 0 && index == k ? delta : 0.0);
  }
  double tex(uint64_t t, int c) const {
    const uint64_t k = t * 4 + (uint64_t)c;
    return s->texture[k] + (kind == 1 && index == k ? delta : 0.0);
  }
};

struct Pixel {
  uint64_t vi[3];
  double P[3][3], rgb[3][3], uv[3][2];
  double X[3], Y[3], W[3], D[3][2], e[3], E, b[3];
  double crgb[3], cu, cv;
  double fx, fy;
  int x0, x1, y0, y1;
  double c00[4], c10[4], c01[4], c11[4], t[4];
  double color[4];
};

double cross2(const double* a, const double* b) { return a[0] * b[1] - a[1] * b[0]; }

// Colour of pixel (x, y) covered by source triangle `tri` of the scene; false when the
// triangle is degenerate at the pixel or an index is out of range.
bool shade(const Eval& ev, const OracleDiffView& v, int x, int y, uint64_t tri, Pixel& q) {
  const OracleDiffScene& s = *ev.s;
  for (int k = 0; k < 3; ++k) {
    const int32_t i = s.indices[3 * tri + (uint64_t)k];
    if (i < 0 || (uint64_t)i >= s.nverts) return false;
    q.vi[k] = (uint64_t)i;
    for (int j = 0; j < 3; ++j) q.P[k][j] = ev.vtx(q.vi[k], j);
    for (int j = 0; j < 3; ++j) q.rgb[k][j] = ev.vtx(q.vi[k], 3 + j);
    for (int j = 0; j < 2; ++j) q.uv[k][j] = ev.vtx(q.vi[k], 6 + j);
  }
  const float* m = v.mvp;
  const double px = v.viewport[2] / 2.0, py = v.viewport[3] / 2.0;
  const double ox = v.viewport[0] + px, oy = v.viewport[1] + py;
  const double ax = ox - (x + 0.5), ay = oy - (y + 0.5);
  for (int k = 0; k < 3; ++k) {
    const double* P = q.P[k];
    q.X[k] = m[0] * P[0] + m[1] * P[1] + m[2] * P[2] + m[3];
    q.Y[k] = m[4] * P[0] + m[5] * P[1] + m[6] * P[2] + m[7];
    q.W[k] = m[12] * P[0] + m[13] * P[1] + m[14] * P[2] + m[15];
    q.D[k][0] = px * q.X[k] + ax * q.W[k];
    q.D[k][1] = -py * q.Y[k] + ay * q.W[k];
  }
  q.e[0] = cross2(q.D[1], q.D[2]);
  q.e[1] = cross2(q.D[2], q.D[0]);
  q.e[2] = cross2(q.D[0], q.D[1]);
  q.E = q.e[0] + q.e[1] + q.e[2];
  if (!(q.E != 0.0) || !std::isfinite(q.E)) return false;
  for (int k = 0; k < 3; ++k) q.b[k] = q.e[k] / q.E;
  for (int j = 0; j < 3; ++j) q.crgb[j] = q.b[0] * q.rgb[0][j] + q.b[1] * q.rgb[1][j] + q.b[2] * q.rgb[2][j];
  q.cu = q.b[0] * q.uv[0][0] + q.b[1] * q.uv[1][0] + q.b[2] * q.uv[2][0];
  q.cv = q.b[0] * q.uv[0][1] + q.b[1] * q.uv[1][1] + q.b[2] * q.uv[2][1];
  const int tw = s.tex_w, th = s.tex_h;
  const double fu = q.cu < 0.0 ? 0.0 : (q.cu > 1.0 ? 1.0 : q.cu);
  const double fv = q.cv < 0.0 ? 0.0 : (q.cv > 1.0 ? 1.0 : q.cv);
  const double sx = fu * (tw - 1), sy = fv * (th - 1);
  q.x0 = (int)floor(sx);
  q.y0 = (int)floor(sy);
  if (q.x0 > tw - 1) q.x0 = tw - 1;
  if (q.y0 > th - 1) q.y0 = th - 1;
  q.x1 = q.x0 + 1 < tw - 1 ? q.x0 + 1 : tw - 1;
  q.y1 = q.y0 + 1 < th - 1 ? q.y0 + 1 : th - 1;
  q.fx = sx - q.x0;
  q.fy = sy - q.y0;
  const uint64_t w = (uint64_t)tw;
  for (int c = 0; c < 4; ++c) {
    q.c00[c] = ev.tex((uint64_t)q.y0 * w + (uint64_t)q.x0, c);
    q.c10[c] = ev.tex((uint64_t)q.y0 * w + (uint64_t)q.x1, c);
    q.c01[c] = ev.tex((uint64_t)q.y1 * w + (uint64_t)q.x0, c);
    q.c11[c] = ev.tex((uint64_t)q.y1 * w + (uint64_t)q.x1, c);
    const double top = q.c00[c] * (1.0 - q.fx) + q.c10[c] * q.fx;
    const double bot = q.c01[c] * (1.0 - q.fx) + q.c11[c] * q.fx;
    q.t[c] = top * (1.0 - q.fy) + bot * q.fy;
  }
  for (int j = 0; j < 3; ++j) q.color[j] = q.crgb[j] * q.t[j];
  q.color[3] = q.t[3];
  return true;
}

// Accumulates dL/d(vertex records) and dL/d(texels) of one pixel with dL/d(colour) = g.
void backward(const OracleDiffScene& s, const OracleDiffView& v, int x, int y, const Pixel& q, const double* g,
              double* gv, double* gt) {
  // colour = (crgb * t.rgb, t.a)
  double gt4[4], grgb[3];
  for (int j = 0; j < 3; ++j) {
    gt4[j] = g[j] * q.crgb[j];
    grgb[j] = g[j] * q.t[j];
  }
  gt4[3] = g[3];
  const uint64_t w = (uint64_t)s.tex_w;
  if (gt) {
    const double w00 = (1.0 - q.fx) * (1.0 - q.fy), w10 = q.fx * (1.0 - q.fy);
    const double w01 = (1.0 - q.fx) * q.fy, w11 = q.fx * q.fy;
    for (int c = 0; c < 4; ++c) {
      gt[4 * ((uint64_t)q.y0 * w + (uint64_t)q.x0) + (uint64_t)c] += w00 * gt4[c];
      gt[4 * ((uint64_t)q.y0 * w + (uint64_t)q.x1) + (uint64_t)c] += w10 * gt4[c];
      gt[4 * ((uint64_t)q.y1 * w + (uint64_t)q.x0) + (uint64_t)c] += w01 * gt4[c];
      gt[4 * ((uint64_t)q.y1 * w + (uint64_t)q.x1) + (uint64_t)c] += w11 * gt4[c];
    }
  }
  if (!gv) return;
  // texture coordinate derivatives (zero where the clamp is active)
  double gu = 0.0, gvv = 0.0;
  for (int c = 0; c < 4; ++c) {
    const double dx = (1.0 - q.fy) * (q.c10[c] - q.c00[c]) + q.fy * (q.c11[c] - q.c01[c]);
    const double dy = (1.0 - q.fx) * (q.c01[c] - q.c00[c]) + q.fx * (q.c11[c] - q.c10[c]);
    gu += gt4[c] * dx;
    gvv += gt4[c] * dy;
  }
  gu = (q.cu > 0.0 && q.cu < 1.0) ? gu * (s.tex_w - 1) : 0.0;
  gvv = (q.cv > 0.0 && q.cv < 1.0) ? gvv * (s.tex_h - 1) : 0.0;
  double G[3];
  for (int k = 0; k < 3; ++k)
    G[k] = grgb[0] * q.rgb[k][0] + grgb[1] * q.rgb[k][1] + grgb[2] * q.rgb[k][2] + gu * q.uv[k][0] +
           gvv * q.uv[k][1];
  const double Gb = q.b[0] * G[0] + q.b[1] * G[1] + q.b[2] * G[2];
  double H[3];
  for (int k = 0; k < 3; ++k) H[k] = (G[k] - Gb) / q.E;
  const double(*D)[2] = q.D;
  double gD[3][2];
  gD[0][0] = H[1] * -D[2][1] + H[2] * D[1][1];
  gD[0][1] = H[1] * D[2][0] + H[2] * -D[1][0];
  gD[1][0] = H[0] * D[2][1] + H[2] * -D[0][1];
  gD[1][1] = H[0] * -D[2][0] + H[2] * D[0][0];
  gD[2][0] = H[0] * -D[1][1] + H[1] * D[0][1];
  gD[2][1] = H[0] * D[1][0] + H[1] * -D[0][0];
  const double px = v.viewport[2] / 2.0, py = v.viewport[3] / 2.0;
  const double ax = v.viewport[0] + px - (x + 0.5), ay = v.viewport[1] + py - (y + 0.5);
  const float* m = v.mvp;
  for (int k = 0; k < 3; ++k) {
    const double gX = px * gD[k][0], gY = -py * gD[k][1], gW = ax * gD[k][0] + ay * gD[k][1];
    double* o = gv + 8 * q.vi[k];
    for (int j = 0; j < 3; ++j) o[j] += m[j] * gX + m[4 + j] * gY + m[12 + j] * gW;
    for (int j = 0; j < 3; ++j) o[3 + j] += q.b[k] * grgb[j];
    o[6] += q.b[k] * gu;
    o[7] += q.b[k] * gvv;
  }
}

// Source triangle of pixel i of view v, -1 for none, -2 for an invalid id.
int64_t source_of(const OracleDiffScene& s, const OracleDiffView& v, uint64_t i) {
  const int32_t w = v.winner[i];
  if (w < 0) return -1;
  if ((uint64_t)w >= v.nprims) return -2;
  const int32_t t = v.prim_src[w];
  if (t < 0 || (uint64_t)t >= s.count / 3) return -2;
  return t;
}

bool valid(const OracleDiffScene* s, const OracleDiffView* v, int n) {
  if (!s || !v || n < 0 || !s->vertices || !s->indices || !s->texture || s->count % 3 || s->tex_w < 1 ||
      s->tex_h < 1)
    return false;
  for (int i = 0; i < n; ++i)
    if (!v[i].winner || !v[i].prim_src || v[i].width <= 0 || v[i].height <= 0) return false;
  return true;
}

}  // namespace

extern "C" int oracle_diff_eval(const OracleDiffScene* s, const OracleDiffView* views, int nviews, double* loss,
                                double* grad_vertices, double* grad_texture) {
  if (!valid(s, views, nviews)) return 1;
  Eval ev{s, -1, 0, 0.0};
  double L = 0.0;
  for (int vi = 0; vi < nviews; ++vi) {
    const OracleDiffView& v = views[vi];
    if (!v.grad_color && !v.target) return 1;
    for (int y = 0; y < v.height; ++y)
      for (int x = 0; x < v.width; ++x) {
        const uint64_t i = (uint64_t)y * (uint64_t)v.width + (uint64_t)x;
        const int64_t t = source_of(*s, v, i);
        if (t == -2) return 2;
        if (t < 0) continue;
        Pixel q;
        if (!shade(ev, v, x, y, (uint64_t)t, q)) continue;
        double g[4];
        for (int c = 0; c < 4; ++c) {
          const double d = v.target ? q.color[c] - v.target[4 * i + (uint64_t)c] : 0.0;
          L += d * d;
          g[c] = v.grad_color ? (double)v.grad_color[4 * i + (uint64_t)c] : 2.0 * d;
        }
        if (grad_vertices || grad_texture) backward(*s, v, x, y, q, g, grad_vertices, grad_texture);
      }
  }
  if (loss) *loss = L;
  return 0;
}

extern "C" int oracle_diff_fd(const OracleDiffScene* s, const OracleDiffView* views, int nviews,
                              const int32_t* kind, const uint64_t* index, int n, double h, double* out,
                              int threads) {
  if (!valid(s, views, nviews) || n < 0 || (n && (!kind || !index || !out)) || !(h > 0.0)) return 1;
  for (int vi = 0; vi < nviews; ++vi)
    if (!views[vi].target) return 1;
  for (int p = 0; p < n; ++p)
    if (kind[p] < 0 || kind[p] > 1 ||
        index[p] >= (kind[p] == 0 ? 8 * s->nverts : 4 * (uint64_t)s->tex_w * (uint64_t)s->tex_h))
      return 1;
  int bad = 0;
#ifdef _OPENMP
  if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(dynamic, 1) reduction(| : bad)
#endif
  for (int p = 0; p < n; ++p) {
    const Eval e0{s, -1, 0, 0.0}, ep{s, kind[p], index[p], h}, em{s, kind[p], index[p], -h};
    const uint64_t vert = index[p] / 8, texel = index[p] / 4;
    const uint64_t tw = (uint64_t)s->tex_w;
    double acc = 0.0;
    for (int vi = 0; vi < nviews; ++vi) {
      const OracleDiffView& v = views[vi];
      for (int y = 0; y < v.height; ++y)
        for (int x = 0; x < v.width; ++x) {
          const uint64_t i = (uint64_t)y * (uint64_t)v.width + (uint64_t)x;
          const int64_t t = source_of(*s, v, i);
          if (t == -2) bad = 1;
          if (t < 0) continue;
          // pixels the parameter cannot reach contribute exactly zero
          if (kind[p] == 0) {
            const int32_t* tri = s->indices + 3 * (uint64_t)t;
            if ((uint64_t)tri[0] != vert && (uint64_t)tri[1] != vert && (uint64_t)tri[2] != vert) continue;
          } else {
            Pixel q0;
            if (!shade(e0, v, x, y, (uint64_t)t, q0)) continue;
            const uint64_t tx = texel % tw, ty = texel / tw;
            if ((tx != (uint64_t)q0.x0 && tx != (uint64_t)q0.x1) || (ty != (uint64_t)q0.y0 && ty != (uint64_t)q0.y1))
              continue;
          }
          Pixel qp, qm;
          const bool okp = shade(ep, v, x, y, (uint64_t)t, qp), okm = shade(em, v, x, y, (uint64_t)t, qm);
          if (!okp || !okm) continue;
          for (int c = 0; c < 4; ++c) {
            const double tg = v.target[4 * i + (uint64_t)c];
            const double dp = qp.color[c] - tg, dm = qm.color[c] - tg;
            acc += dp * dp - dm * dm;
          }
        }
    }
    out[p] = acc / (2.0 * h);
  }
  return bad ? 2 : 0;
}
