// Backward of the differentiable-rendering pixel shader PsDiff (swr_programs.h):
// colour = (interpolated vertex rgb) * bilinear RGBA32F texel, alpha = texel alpha.
//
// Visibility is held fixed: each covered pixel keeps the primitive that won it in the
// forward draw (SwrUniforms.winner), mapped to its source triangle by the primitive-source
// output of the draw.  One CTA per 16 x 16 pixel tile of one view recomputes, per pixel,
// the triangle's clip-space vertices and its perspective-correct barycentrics in
// homogeneous window coordinates (no per-pixel state is kept from the forward):
//   D_k = (px * X_k + (ox - xp) * W_k,  -py * Y_k + (oy - yp) * W_k)    ( = W_k * (s_k - p) )
//   e_0 = D_1 x D_2,  e_1 = D_2 x D_0,  e_2 = D_0 x D_1,   b_k = e_k / (e_0 + e_1 + e_2)
// with (px, py, ox, oy) the viewport transform of VertexProcessor::setViewport
// (VertexProcessor.cpp:43-54, window y = -py * Y/W + oy) and (xp, yp) the pixel centre.
// These b_k are the weights that PixelData's 1/w interpolation evaluates
// (PixelData.h:84-103); no division by W is needed, so triangles split by clipping need no
// special case.  The chain rule through b_k gives the gradients of the clip coordinates
// (X, Y, W) and, through the view's mvp, of the object-space positions.  The texture
// coordinate derivative is that of the bilinear sampler (Texture.h:146-181 addressing),
// zero where u or v is clamped.
//
// Gradients accumulate with vector float atomics (red.global.add.v4.f32): two per vertex
// (x y z r | g b u v) and one per texel of the 2 x 2 footprint.  The fused L2 mode derives
// dL/d(colour) = 2 * scale * (colour - target) in the kernel and reduces the loss per CTA.
#include <string.h>

#include "../../include/swr_gb300.h"
#include "swr_context.h"
#include "swr_device.cuh"

namespace swr {
namespace {

constexpr int kTile = 16;
constexpr int kViewsPerLaunch = 16;

struct BwdView {
  float m[16];
  float px, py, ox, oy;
  int32_t width, height, tiles_x, tiles;
  const int32_t* winner;
  const int32_t* prim_src;
  const float4* grad;
  const float4* color;
  const float4* target;
  uint32_t nprims;
  float gscale;  // 2 * loss_scale
  float lscale;  // loss_scale
  int32_t _pad;
};

struct BwdViews {
  BwdView v[kViewsPerLaunch];
};

struct BwdArgs {
  const float4* verts;  // 2 per vertex: (x, y, z, r), (g, b, u, v)
  const uint32_t* indices;
  const float4* tex;
  float4* gverts;
  float4* gtex;
  double* loss;
  uint32_t* status;
  uint32_t nverts, ntris;
  int32_t tw, th;
};

__device__ __forceinline__ float cross2(float ax, float ay, float bx, float by) { return ax * by - ay * bx; }

__device__ __forceinline__ float4 f4(float a, float b, float c, float d) { return make_float4(a, b, c, d); }

__device__ __forceinline__ void pixel_backward(const BwdView& V, const BwdArgs& a, int x, int y, int32_t w, float4 g) {
  if ((uint32_t)w >= V.nprims) {
    atomicOr(a.status, SWR_F_BAD_GRAD_INPUT);
    return;
  }
  const int32_t t = V.prim_src[w];
  if (t < 0 || (uint32_t)t >= a.ntris) {
    atomicOr(a.status, SWR_F_BAD_GRAD_INPUT);
    return;
  }
  uint32_t vi[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) vi[k] = a.indices[3 * (size_t)t + k];
  if (vi[0] >= a.nverts || vi[1] >= a.nverts || vi[2] >= a.nverts) {
    atomicOr(a.status, SWR_F_BAD_GRAD_INPUT);
    return;
  }
  float4 A[3], B[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    A[k] = __ldg(a.verts + 2 * (size_t)vi[k]);
    B[k] = __ldg(a.verts + 2 * (size_t)vi[k] + 1);
  }
  const float* m = V.m;
  const float ax = V.ox - ((float)x + 0.5f), ay = V.oy - ((float)y + 0.5f);
  float Dx[3], Dy[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float X = m[0] * A[k].x + m[1] * A[k].y + m[2] * A[k].z + m[3];
    const float Y = m[4] * A[k].x + m[5] * A[k].y + m[6] * A[k].z + m[7];
    const float W = m[12] * A[k].x + m[13] * A[k].y + m[14] * A[k].z + m[15];
    Dx[k] = V.px * X + ax * W;
    Dy[k] = -V.py * Y + ay * W;
  }
  const float e0 = cross2(Dx[1], Dy[1], Dx[2], Dy[2]);
  const float e1 = cross2(Dx[2], Dy[2], Dx[0], Dy[0]);
  const float e2 = cross2(Dx[0], Dy[0], Dx[1], Dy[1]);
  const float E = e0 + e1 + e2;
  if (!(E != 0.0f) || !isfinite(E)) return;
  const float iE = 1.0f / E;
  const float b[3] = {e0 * iE, e1 * iE, e2 * iE};
  const float cr = b[0] * A[0].w + b[1] * A[1].w + b[2] * A[2].w;
  const float cg = b[0] * B[0].x + b[1] * B[1].x + b[2] * B[2].x;
  const float cb = b[0] * B[0].y + b[1] * B[1].y + b[2] * B[2].y;
  const float cu = b[0] * B[0].z + b[1] * B[1].z + b[2] * B[2].z;
  const float cv = b[0] * B[0].w + b[1] * B[1].w + b[2] * B[2].w;
  // bilinear footprint
  const float sx = fminf(fmaxf(cu, 0.0f), 1.0f) * (float)(a.tw - 1);
  const float sy = fminf(fmaxf(cv, 0.0f), 1.0f) * (float)(a.th - 1);
  const int x0 = min((int)sx, a.tw - 1), y0 = min((int)sy, a.th - 1);  // sx, sy >= 0: truncation is floor
  const int x1 = min(a.tw - 1, x0 + 1), y1 = min(a.th - 1, y0 + 1);
  const float fx = sx - (float)x0, fy = sy - (float)y0, gx = 1.0f - fx, gy = 1.0f - fy;
  const size_t tw = (size_t)a.tw;
  const size_t i00 = (size_t)y0 * tw + x0, i10 = (size_t)y0 * tw + x1;
  const size_t i01 = (size_t)y1 * tw + x0, i11 = (size_t)y1 * tw + x1;
  const float4 c00 = __ldg(a.tex + i00), c10 = __ldg(a.tex + i10);
  const float4 c01 = __ldg(a.tex + i01), c11 = __ldg(a.tex + i11);
  const float tr = (c00.x * gx + c10.x * fx) * gy + (c01.x * gx + c11.x * fx) * fy;
  const float tg = (c00.y * gx + c10.y * fx) * gy + (c01.y * gx + c11.y * fx) * fy;
  const float tb = (c00.z * gx + c10.z * fx) * gy + (c01.z * gx + c11.z * fx) * fy;
  // dL/d(texel) and dL/d(interpolated rgb)
  const float4 gt = f4(g.x * cr, g.y * cg, g.z * cb, g.w);
  const float grr = g.x * tr, grg = g.y * tg, grb = g.z * tb;
  {
    const float w00 = gx * gy, w10 = fx * gy, w01 = gx * fy, w11 = fx * fy;
    atomicAdd(a.gtex + i00, f4(gt.x * w00, gt.y * w00, gt.z * w00, gt.w * w00));
    atomicAdd(a.gtex + i10, f4(gt.x * w10, gt.y * w10, gt.z * w10, gt.w * w10));
    atomicAdd(a.gtex + i01, f4(gt.x * w01, gt.y * w01, gt.z * w01, gt.w * w01));
    atomicAdd(a.gtex + i11, f4(gt.x * w11, gt.y * w11, gt.z * w11, gt.w * w11));
  }
  // dL/d(u, v) through the bilinear weights
  float gu = 0.0f, gv = 0.0f;
  if (cu > 0.0f && cu < 1.0f) {
    const float dx = gt.x * (gy * (c10.x - c00.x) + fy * (c11.x - c01.x)) +
                     gt.y * (gy * (c10.y - c00.y) + fy * (c11.y - c01.y)) +
                     gt.z * (gy * (c10.z - c00.z) + fy * (c11.z - c01.z)) +
                     gt.w * (gy * (c10.w - c00.w) + fy * (c11.w - c01.w));
    gu = dx * (float)(a.tw - 1);
  }
  if (cv > 0.0f && cv < 1.0f) {
    const float dy = gt.x * (gx * (c01.x - c00.x) + fx * (c11.x - c10.x)) +
                     gt.y * (gx * (c01.y - c00.y) + fx * (c11.y - c10.y)) +
                     gt.z * (gx * (c01.z - c00.z) + fx * (c11.z - c10.z)) +
                     gt.w * (gx * (c01.w - c00.w) + fx * (c11.w - c10.w));
    gv = dy * (float)(a.th - 1);
  }
  // dL/db_k, then through b = e / sum(e) to the edge values e_k
  float G[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) G[k] = grr * A[k].w + grg * B[k].x + grb * B[k].y + gu * B[k].z + gv * B[k].w;
  const float Gb = b[0] * G[0] + b[1] * G[1] + b[2] * G[2];
  const float H0 = (G[0] - Gb) * iE, H1 = (G[1] - Gb) * iE, H2 = (G[2] - Gb) * iE;
  float gDx[3], gDy[3];
  gDx[0] = -H1 * Dy[2] + H2 * Dy[1];
  gDy[0] = H1 * Dx[2] - H2 * Dx[1];
  gDx[1] = H0 * Dy[2] - H2 * Dy[0];
  gDy[1] = -H0 * Dx[2] + H2 * Dx[0];
  gDx[2] = -H0 * Dy[1] + H1 * Dy[0];
  gDy[2] = H0 * Dx[1] - H1 * Dx[0];
#pragma unroll
  for (int k = 0; k < 3; ++k) {
    const float gX = V.px * gDx[k], gY = -V.py * gDy[k], gW = ax * gDx[k] + ay * gDy[k];
    const float p0 = m[0] * gX + m[4] * gY + m[12] * gW;
    const float p1 = m[1] * gX + m[5] * gY + m[13] * gW;
    const float p2 = m[2] * gX + m[6] * gY + m[14] * gW;
    atomicAdd(a.gverts + 2 * (size_t)vi[k], f4(p0, p1, p2, b[k] * grr));
    atomicAdd(a.gverts + 2 * (size_t)vi[k] + 1, f4(b[k] * grg, b[k] * grb, b[k] * gu, b[k] * gv));
  }
}

__global__ void __launch_bounds__(256, 4) k_backward(const __grid_constant__ BwdViews views, const BwdArgs a) {
  __shared__ float red[8];
  const BwdView& V = views.v[blockIdx.y];  // kernel parameter space: uniform constant loads
  if ((int)blockIdx.x >= V.tiles) return;  // uniform per CTA
  const int tx = (int)blockIdx.x % V.tiles_x, ty = (int)blockIdx.x / V.tiles_x;
  const int x = tx * kTile + (int)(threadIdx.x % kTile), y = ty * kTile + (int)(threadIdx.x / kTile);
  float lsum = 0.0f;
  if (x < V.width && y < V.height) {
    const size_t i = (size_t)y * (size_t)V.width + (size_t)x;
    float4 g;
    if (V.grad) {
      g = V.grad[i];
    } else {
      const float4 c = V.color[i], t = V.target[i];
      const float d0 = c.x - t.x, d1 = c.y - t.y, d2 = c.z - t.z, d3 = c.w - t.w;
      lsum = d0 * d0 + d1 * d1 + d2 * d2 + d3 * d3;
      g = f4(V.gscale * d0, V.gscale * d1, V.gscale * d2, V.gscale * d3);
    }
    const int32_t w = V.winner[i];
    if (w >= 0) pixel_backward(V, a, x, y, w, g);
  }
  if (a.loss && !V.grad) {  // uniform per CTA
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) lsum += __shfl_xor_sync(0xffffffffu, lsum, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = lsum;
    __syncthreads();
    if (threadIdx.x == 0) {
      float s = 0.0f;
      for (int k = 0; k < (int)(blockDim.x >> 5); ++k) s += red[k];
      atomicAdd(a.loss, (double)s * (double)V.lscale);
    }
  }
}

bool aligned16(const void* p) { return ((uintptr_t)p & 15u) == 0; }

}  // namespace
}  // namespace swr

extern "C" int swr_backward(swr_context* c, const swr_backward_args* args, const swr_grad_view* views, int nviews,
                            void* stream) {
  using namespace swr;
  if (!c || !args || !views || nviews <= 0) return SWR_EINVAL;
  const swr_backward_args& g = *args;
  if (g.count % 3 || g.count / 3 >= 0x7fffffffull || g.nverts >= 0x3fffffffull) return SWR_EINVAL;
  if ((g.count && !g.indices) || !g.vertices || !g.texture || !g.grad_vertices || !g.grad_texture) return SWR_EINVAL;
  if (g.tex_w < 1 || g.tex_h < 1 || (uint64_t)g.tex_w * (uint64_t)g.tex_h >= 0x7fffffffull) return SWR_EINVAL;
  if (!aligned16(g.vertices) || !aligned16(g.texture) || !aligned16(g.grad_vertices) || !aligned16(g.grad_texture))
    return SWR_EINVAL;
  for (int i = 0; i < nviews; ++i) {
    const swr_grad_view& v = views[i];
    if (v.width <= 0 || v.height <= 0 || !v.winner || (v.nprims && !v.prim_src) || v.nprims > 0xffffffffull)
      return SWR_EINVAL;
    if ((uint64_t)v.width * (uint64_t)v.height >= 0x7fffffffull) return SWR_EINVAL;
    if (v.grad_color ? !aligned16(v.grad_color) : (!v.color || !v.target || !aligned16(v.color) || !aligned16(v.target)))
      return SWR_EINVAL;
  }
  BwdArgs a;
  a.verts = (const float4*)g.vertices;
  a.indices = g.indices;
  a.tex = (const float4*)g.texture;
  a.gverts = (float4*)g.grad_vertices;
  a.gtex = (float4*)g.grad_texture;
  a.loss = g.loss;
  a.status = context_status(c) + SWR_ST_FLAGS;
  a.nverts = (uint32_t)g.nverts;
  a.ntris = (uint32_t)(g.count / 3);
  a.tw = g.tex_w;
  a.th = g.tex_h;
  cudaStream_t s = (cudaStream_t)stream;
  for (int v0 = 0; v0 < nviews; v0 += kViewsPerLaunch) {
    const int nv = nviews - v0 < kViewsPerLaunch ? nviews - v0 : kViewsPerLaunch;
    BwdViews bv;
    memset(&bv, 0, sizeof(bv));
    int max_tiles = 0;
    for (int k = 0; k < nv; ++k) {
      const swr_grad_view& in = views[v0 + k];
      BwdView& o = bv.v[k];
      memcpy(o.m, in.mvp, sizeof(o.m));
      o.px = (float)in.viewport[2] / 2.0f;  // VertexProcessor::setViewport
      o.py = (float)in.viewport[3] / 2.0f;
      o.ox = (float)in.viewport[0] + o.px;
      o.oy = (float)in.viewport[1] + o.py;
      o.width = in.width;
      o.height = in.height;
      o.tiles_x = (in.width + kTile - 1) / kTile;
      o.tiles = o.tiles_x * ((in.height + kTile - 1) / kTile);
      o.winner = in.winner;
      o.prim_src = in.prim_src;
      o.grad = (const float4*)in.grad_color;
      o.color = (const float4*)in.color;
      o.target = (const float4*)in.target;
      o.nprims = (uint32_t)in.nprims;
      o.gscale = 2.0f * in.loss_scale;
      o.lscale = in.loss_scale;
      max_tiles = o.tiles > max_tiles ? o.tiles : max_tiles;
    }
    k_backward<<<dim3((unsigned)max_tiles, (unsigned)nv), 256, 0, s>>>(bv, a);
    context_add_launches(c, 1);
  }
  const cudaError_t e = cudaGetLastError();
  return e == cudaSuccess ? SWR_OK : SWR_ECUDA;
}
