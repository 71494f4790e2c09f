// Pipeline stages of the GB300 rasterizer, templated on the shader programs.
//
//   k_vertex          VertexShader::processVertex once per vertex + outcodes + divide and
//                     viewport (VertexProcessor.cpp:122-150, :347-377)
//   k_assemble_count  one CTA per 1024-primitive batch: outcode OR, polygon clipping
//                     (PolyClipper.cpp:45-81), fan split and culling (VertexProcessor.cpp:
//                     217-263, :319-345); counts survivors per batch
//   k_assemble_emit   writes the surviving triangles in the reference's effective order:
//                     per batch, the input slots in order, then every extra fan triangle
//                     in parent order (VertexProcessor.cpp:254-260)
//   k_setup           TriangleEquations (TriangleEquations.h:47-71) and the raster-mode
//                     decision, bounding boxes and tile counts per primitive
//   k_emit_pairs      (tile, primitive) pairs in primitive order -> stable radix sort
//   k_raster          one CTA per screen tile; each thread owns pixels and walks the
//                     tile's bin in primitive order, reproducing Span (Rasterizer.h:309-411)
//                     and Block (Rasterizer.h:225-306, PixelShaderBase.h:55-112) coverage
//                     and incrementally stepped interpolants exactly, then calls the pixel
//                     shader in the same per-pixel order as the reference.
//
// All arithmetic on the parity path uses the _rn intrinsics (no FMA contraction).
#pragma once
#include "swr_device.cuh"
#include "swr_math.h"

namespace swr {

// ---------------------------------------------------------------------------------
// Post-transform vertex record (floats): 0-3 clip x,y,z,w | 4-6 screen x,y,z | 7 outcode
// | 8.. avar[A] | pvar[P].  Stride rounded to 16 bytes.
template <int A, int P>
struct VLayout {
  enum { NA = A, NP = P, OFF_A = 8, OFF_P = 8 + A, S = ((8 + A + P + 3) / 4) * 4 };
};

template <int A, int P>
struct VsOut {
  float x, y, z, w;
  float avar[A > 0 ? A : 1];
  float pvar[P > 0 ? P : 1];
};

__device__ __forceinline__ int outcode(float x, float y, float z, float w) {
  // VertexProcessor::clipMask (VertexProcessor.cpp:122-132)
  int m = 0;
  if (swr_sub(w, x) < 0.0f) m |= 0x01;
  if (swr_add(x, w) < 0.0f) m |= 0x02;
  if (swr_sub(w, y) < 0.0f) m |= 0x04;
  if (swr_add(y, w) < 0.0f) m |= 0x08;
  if (swr_sub(w, z) < 0.0f) m |= 0x10;
  if (swr_add(z, w) < 0.0f) m |= 0x20;
  return m;
}

// Perspective divide, viewport and depth range (VertexProcessor.cpp:364-373).
__device__ __forceinline__ void to_screen(const SwrDrawDesc& D, float x, float y, float z, float w,
                                          float& sx, float& sy, float& sz) {
  const float iw = swr_div(1.0f, w);
  const float nx = swr_mul(x, iw), ny = swr_mul(y, iw), nz = swr_mul(z, iw);
  sx = swr_add(swr_mul(D.vp_px, nx), D.vp_ox);
  sy = swr_add(swr_mul(D.vp_py, -ny), D.vp_oy);
  sz = swr_add(swr_mul(swr_mul(0.5f, swr_sub(D.df, D.dn)), nz), swr_mul(0.5f, swr_add(D.dn, D.df)));
}

// Vertex shading of every vertex, grid-stride over the launch's threads.
template <class VS>
__device__ __forceinline__ void vertex_stage(const SwrDrawDesc* __restrict__ draws, int ndraws,
                                             const uint32_t* __restrict__ draw_vbase, uint32_t nverts,
                                             float* __restrict__ ptv) {
  typedef VLayout<VS::AVarCount, VS::PVarCount> L;
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < nverts; v += gridDim.x * blockDim.x) {
    const int d = ndraws > 1 ? swr_find_le(draw_vbase, ndraws, v) : 0;
    const SwrDrawDesc& D = draws[d];
    const uint32_t local = v - D.vbase;
    SwrVertexInput in;
#pragma unroll
    for (int a = 0; a < VS::AttribCount; ++a)
      in.p[a] = (const char*)D.attrib[a] + (size_t)D.attrib_stride[a] * (size_t)local;
    VsOut<VS::AVarCount, VS::PVarCount> o;
    VS::processVertex(in, &o, D.u);
    float rec[L::S];
    rec[0] = o.x; rec[1] = o.y; rec[2] = o.z; rec[3] = o.w;
    to_screen(D, o.x, o.y, o.z, o.w, rec[4], rec[5], rec[6]);
    rec[7] = __int_as_float(outcode(o.x, o.y, o.z, o.w));
#pragma unroll
    for (int i = 0; i < VS::AVarCount; ++i) rec[L::OFF_A + i] = o.avar[i];
#pragma unroll
    for (int i = 0; i < VS::PVarCount; ++i) rec[L::OFF_P + i] = o.pvar[i];
#pragma unroll
    for (int i = 8 + VS::AVarCount + VS::PVarCount; i < L::S; ++i) rec[i] = 0.0f;
    float4* dst = (float4*)(ptv + (size_t)v * L::S);
#pragma unroll
    for (int i = 0; i < L::S / 4; ++i) dst[i] = make_float4(rec[4 * i], rec[4 * i + 1], rec[4 * i + 2], rec[4 * i + 3]);
  }
}

template <class VS>
__global__ void __launch_bounds__(256) k_vertex(const SwrDrawDesc* __restrict__ draws, int ndraws,
                                                const uint32_t* __restrict__ draw_vbase,
                                                uint32_t nverts, float* __restrict__ ptv) {
  swr_pdl_entry();
  vertex_stage<VS>(draws, ndraws, draw_vbase, nverts, ptv);
}

// Direct Rasterizer path: RasterizerVertex (x, y, z, w, avar[16], pvar[16]) records are
// already in screen space; convert them to the post-transform layout of the pixel shader.
template <int A, int P>
__global__ void k_direct_vertices(const float* __restrict__ rv, uint32_t nverts, float* __restrict__ ptv) {
  swr_pdl_entry();
  typedef VLayout<A, P> L;
  for (uint32_t v = blockIdx.x * blockDim.x + threadIdx.x; v < nverts; v += gridDim.x * blockDim.x) {
    const float* s = rv + (size_t)v * 36;
    float* o = ptv + (size_t)v * L::S;
    o[0] = s[0]; o[1] = s[1]; o[2] = s[2]; o[3] = s[3];
    o[4] = s[0]; o[5] = s[1]; o[6] = s[2]; o[7] = __int_as_float(0);
    for (int i = 0; i < A; ++i) o[L::OFF_A + i] = s[4 + i];
    for (int i = 0; i < P; ++i) o[L::OFF_P + i] = s[20 + i];
  }
}

// ---------------------------------------------------------------------------------
// Triangle assembly, clipping and culling.

// Polygon clipper over a per-thread vertex pool (clip-space x,y,z,w + A + P values).
// A convex cut adds one vertex per plane (at most 9 in total); exact zeros in the plane
// distances can add more, so both the polygon and the pool are bounds-checked and a
// polygon that would exceed them is reported (SWR_F_CLIP_COMPLEX) and dropped.
template <int A, int P>
struct Clipper {
  enum { NV = 4 + A + P, POOL = 24, MAXPOLY = 16 };
  float pool[POOL][NV];
  int npool;
  int poly[MAXPOLY + 1];
  int npoly;
  bool bad;

  __device__ void lerp(int i0, int i1, float t) {  // Helper::interpolateVertex (PolyClipper.h:34-48)
    const float s = swr_sub(1.0f, t);
    float* r = pool[npool];
#pragma unroll
    for (int k = 0; k < NV; ++k) r[k] = swr_add(swr_mul(pool[i0][k], s), swr_mul(pool[i1][k], t));
    npool++;
  }

  __device__ static float dist(const float* v, float a, float b, float c, float d) {
    return swr_add(swr_add(swr_add(swr_mul(a, v[0]), swr_mul(b, v[1])), swr_mul(c, v[2])), swr_mul(d, v[3]));
  }

  __device__ static int sgn(float v) { return (0.0f < v) - (v < 0.0f); }

  // PolyClipper::clipToPlane (PolyClipper.cpp:45-81).
  __device__ void clip(float a, float b, float c, float d) {
    if (npoly < 3 || bad) return;
    int out[MAXPOLY + 1];
    int nout = 0;
    int iprev = poly[0];
    poly[npoly] = iprev;
    float dprev = dist(pool[iprev], a, b, c, d);
    for (int i = 1; i <= npoly; ++i) {
      const int icur = poly[i];
      const float dcur = dist(pool[icur], a, b, c, d);
      if (dprev >= 0.0f) {
        if (nout >= MAXPOLY) { bad = true; return; }
        out[nout++] = iprev;
      }
      if (sgn(dcur) != sgn(dprev)) {
        if (nout >= MAXPOLY || npool >= POOL) { bad = true; return; }
        const float t = dcur < 0.0f ? swr_div(dprev, swr_sub(dprev, dcur))
                                    : swr_div(-dprev, swr_sub(dcur, dprev));
        lerp(iprev, icur, t);
        out[nout++] = npool - 1;
      }
      iprev = icur;
      dprev = dcur;
    }
    for (int i = 0; i < nout; ++i) poly[i] = out[i];
    npoly = nout;
  }
};

// facing test of VertexProcessor::cullTriangles (VertexProcessor.cpp:330-343):
// returns 0 = drop, 1 = keep, 3 = keep and swap v0 <-> v2.
__device__ __forceinline__ int cull_decision(int cull, float x0, float y0, float x1, float y1,
                                             float x2, float y2) {
  const float facing = swr_sub(swr_mul(swr_sub(x0, x1), swr_sub(y2, y1)),
                               swr_mul(swr_sub(x2, x1), swr_sub(y0, y1)));
  if (facing < 0.0f) return cull == 2 ? 0 : 1;
  return cull == 1 ? 0 : 3;
}

struct AssembleArgs {
  const SwrDrawDesc* draws;
  int ndraws;
  const uint32_t* draw_bbase;
  const float* ptv;
  float* clipv;             // clip-generated vertices (post-transform layout)
  SwrClipEntry* clip_table;
  uint32_t* clip_slot;      // per submitted primitive (valid when clipped)
  uint8_t* tri_flags;       // per submitted primitive: bit0 keep, bit1 swap, bit2 clipped
  uint2* batch_counts;      // per batch: (kept input slots, kept extra fan triangles)
  const uint32_t* batch_base;
  uint4* tris;              // output primitives: v0, v1, v2 references + draw id
  uint2* lp_refs;           // per submitted point / line: endpoint references after clipping
  uint32_t* draw_prim_base; // per draw: index of its first emitted primitive (optional)
  uint32_t* status;
  uint32_t cap_clip_slots, cap_clip_verts, cap_prims;
};

template <int A, int P>
__device__ void assemble_one(const AssembleArgs& g, const SwrDrawDesc& D, uint32_t p, uint32_t i0,
                             uint32_t i1, uint32_t i2, uint32_t& in_kept, uint32_t& ex_kept) {
  typedef VLayout<A, P> L;
  in_kept = ex_kept = 0;
  const uint32_t gp = D.pbase + p;
  if (i0 >= D.nverts || i1 >= D.nverts || i2 >= D.nverts) {
    atomicOr(&g.status[SWR_ST_FLAGS], SWR_F_BAD_INDEX);
    g.tri_flags[gp] = 0;
    return;
  }
  const uint32_t r[3] = {D.vbase + i0, D.vbase + i1, D.vbase + i2};
  const float* v[3] = {g.ptv + (size_t)r[0] * L::S, g.ptv + (size_t)r[1] * L::S, g.ptv + (size_t)r[2] * L::S};
  // words 4-7 of a record (16-byte aligned: S is a multiple of 4): screen x, y, z, outcode
  float4 q[3];
#pragma unroll
  for (int k = 0; k < 3; ++k) q[k] = __ldg((const float4*)(v[k] + 4));
  const int m = __float_as_int(q[0].w) | __float_as_int(q[1].w) | __float_as_int(q[2].w);
  if (m == 0) {
    const int c = cull_decision(D.cull, q[0].x, q[0].y, q[1].x, q[1].y, q[2].x, q[2].y);
    g.tri_flags[gp] = (uint8_t)c;
    in_kept = c & 1;
    return;
  }
  // Clip in the reference's plane order +X, -X, +Y, -Y, +Z, -Z (VertexProcessor.cpp:237-242).
  Clipper<A, P> cp;
  for (int k = 0; k < 3; ++k) {
    cp.pool[k][0] = v[k][0]; cp.pool[k][1] = v[k][1]; cp.pool[k][2] = v[k][2]; cp.pool[k][3] = v[k][3];
    for (int i = 0; i < A; ++i) cp.pool[k][4 + i] = v[k][L::OFF_A + i];
    for (int i = 0; i < P; ++i) cp.pool[k][4 + A + i] = v[k][L::OFF_P + i];
    cp.poly[k] = k;
  }
  cp.npool = 3;
  cp.npoly = 3;
  cp.bad = false;
  if (m & 0x01) cp.clip(-1.0f, 0.0f, 0.0f, 1.0f);
  if (m & 0x02) cp.clip(1.0f, 0.0f, 0.0f, 1.0f);
  if (m & 0x04) cp.clip(0.0f, -1.0f, 0.0f, 1.0f);
  if (m & 0x08) cp.clip(0.0f, 1.0f, 0.0f, 1.0f);
  if (m & 0x10) cp.clip(0.0f, 0.0f, -1.0f, 1.0f);
  if (m & 0x20) cp.clip(0.0f, 0.0f, 1.0f, 1.0f);
  if (cp.bad) atomicOr(&g.status[SWR_ST_FLAGS], SWR_F_CLIP_COMPLEX);
  if (cp.npoly < 3 || cp.bad) {
    g.tri_flags[gp] = 4;  // clipped away entirely
    g.clip_slot[gp] = 0xffffffffu;
    return;
  }
  // Screen positions of the polygon (generated vertices are transformed here).
  float sx[Clipper<A, P>::MAXPOLY], sy[Clipper<A, P>::MAXPOLY], sz[Clipper<A, P>::MAXPOLY];
  int nnew = 0;
  for (int k = 0; k < cp.npoly; ++k) {
    const int pi = cp.poly[k];
    if (pi < 3) {
      sx[k] = v[pi][4]; sy[k] = v[pi][5]; sz[k] = v[pi][6];
    } else {
      to_screen(D, cp.pool[pi][0], cp.pool[pi][1], cp.pool[pi][2], cp.pool[pi][3], sx[k], sy[k], sz[k]);
      nnew++;
    }
  }
  uint32_t keep = 0, swap = 0;  // bit k: fan triangle (p0, p[k+1], p[k+2])
  for (int k = 0; k + 2 < cp.npoly; ++k) {
    const int c = cull_decision(D.cull, sx[0], sy[0], sx[k + 1], sy[k + 1], sx[k + 2], sy[k + 2]);
    if (c & 1) keep |= 1u << k;
    if (c & 2) swap |= 1u << k;
  }
  const uint32_t slot = atomicAdd(&g.status[SWR_ST_CLIP_SLOTS], 1u);
  const uint32_t vb = atomicAdd(&g.status[SWR_ST_CLIP_VERTS], (uint32_t)nnew);
  if (slot >= g.cap_clip_slots || vb + nnew > g.cap_clip_verts) {
    atomicOr(&g.status[SWR_ST_FLAGS], SWR_F_CLIP_OVERFLOW);
    g.tri_flags[gp] = 4;
    g.clip_slot[gp] = 0xffffffffu;
    return;
  }
  SwrClipEntry ent;
  int nv = 0;
  for (int k = 0; k < cp.npoly; ++k) {
    const int pi = cp.poly[k];
    if (pi < 3) {
      ent.ref[k] = r[pi];
    } else {
      const uint32_t id = vb + nv++;
      float* o = g.clipv + (size_t)id * L::S;
      o[0] = cp.pool[pi][0]; o[1] = cp.pool[pi][1]; o[2] = cp.pool[pi][2]; o[3] = cp.pool[pi][3];
      o[4] = sx[k]; o[5] = sy[k]; o[6] = sz[k]; o[7] = __int_as_float(0);
      for (int i = 0; i < A; ++i) o[L::OFF_A + i] = cp.pool[pi][4 + i];
      for (int i = 0; i < P; ++i) o[L::OFF_P + i] = cp.pool[pi][4 + A + i];
      ent.ref[k] = SWR_CLIP_REF | id;
    }
  }
  ent.n = (uint16_t)cp.npoly;
  ent.keep = (uint16_t)keep;
  ent.swap = (uint16_t)swap;
  g.clip_table[slot] = ent;
  g.clip_slot[gp] = slot;
  g.tri_flags[gp] = 4;
  in_kept = keep & 1u;
  ex_kept = __popc(keep >> 1);
}

// Triangles [p0, p0 + count) of a draw, clamped to the draw: their count.
__device__ __forceinline__ uint32_t batch_count(const SwrDrawDesc& D, uint32_t p0, uint32_t count) {
  return p0 < D.nprims ? min(count, D.nprims - p0) : 0u;
}

#define SWR_HALF (SWR_BATCH_PRIMS / 2)  // triangles per assembly CTA (half a batch)

// One CTA per half batch (512 triangles, one per thread): clip / cull and count the
// survivors: batch_counts[h] = (kept input slots, kept extra fan triangles).
template <int A, int P>
__device__ __forceinline__ void assemble_count_block(const AssembleArgs& g, uint32_t hb) {
  __shared__ uint32_t tmp[64];
  const uint32_t b = hb >> 1;
  const int d = g.ndraws > 1 ? swr_find_le(g.draw_bbase, g.ndraws, b) : 0;
  const SwrDrawDesc& D = g.draws[d];
  const uint32_t p0 = (b - D.bbase) * SWR_BATCH_PRIMS + (hb & 1) * SWR_HALF;
  const uint32_t n = batch_count(D, p0, SWR_HALF);
  uint32_t ik = 0, ek = 0;
  const uint32_t q = threadIdx.x;
  if (q < n) {
    const uint32_t* ix = D.indices + (size_t)3 * (p0 + q);
    assemble_one<A, P>(g, D, p0 + q, __ldg(ix), __ldg(ix + 1), __ldg(ix + 2), ik, ek);
  }
  uint32_t tin, tex;
  swr_block_sum2(ik, ek, tmp, tin, tex);
  if (threadIdx.x == 0) g.batch_counts[hb] = make_uint2(tin, tex);
}

template <int A, int P>
__global__ void __launch_bounds__(SWR_HALF) k_assemble_count(AssembleArgs g) {
  swr_pdl_entry();
  assemble_count_block<A, P>(g, blockIdx.x);
}

// Exclusive scan of per-batch totals -> batch bases; primitive total into the status word.
static __global__ void __launch_bounds__(1024) k_batch_scan(const uint2* counts, uint32_t nbatches, uint32_t* base,
                                                     uint32_t* status, uint32_t cap_prims) {
  swr_pdl_entry();
  __shared__ uint32_t tmp[32];
  uint32_t run = 0;
  for (uint32_t b0 = 0; b0 < nbatches; b0 += 1024) {
    const uint32_t b = b0 + threadIdx.x;
    const uint32_t v = b < nbatches ? counts[b].x + counts[b].y : 0u;
    uint32_t tot;
    const uint32_t ex = swr_block_exscan(v, tmp, &tot);
    if (b < nbatches) base[b] = run + ex;
    run += tot;
  }
  if (threadIdx.x == 0) {
    status[SWR_ST_PRIMS] = run;
    if (run > cap_prims) atomicOr(&status[SWR_ST_FLAGS], SWR_F_PRIM_OVERFLOW);
  }
}

// Writes the surviving triangles of one batch at their effective-order positions.  The
// batch base is the sum of the totals of the batches before it; the last batch publishes
// the primitive count (and flags an undersized primitive queue).
template <int A, int P>
__device__ __forceinline__ void assemble_emit_block(const AssembleArgs& g, uint32_t hb, uint32_t nhb) {
  __shared__ uint32_t tmp[64];
  __shared__ uint32_t tmps[32];
  if (g.status[SWR_ST_FLAGS] & SWR_F_ANY_OVERFLOW) return;
  const uint32_t b = hb >> 1, half = hb & 1;
  const int d = g.ndraws > 1 ? swr_find_le(g.draw_bbase, g.ndraws, b) : 0;
  const SwrDrawDesc& D = g.draws[d];
  const uint32_t p0 = (b - D.bbase) * SWR_BATCH_PRIMS + half * SWR_HALF;
  const uint32_t n = batch_count(D, p0, SWR_HALF);
  uint32_t before = 0, dbefore = 0;
  for (uint32_t i = threadIdx.x; i < 2 * b; i += blockDim.x) {
    const uint32_t c = g.batch_counts[i].x + g.batch_counts[i].y;
    before += c;
    if (i < 2 * D.bbase) dbefore += c;
  }
  // base: the batch's first emitted primitive; dbase: the draw's (primitive-source output)
  uint32_t base, dbase;
  swr_block_sum2(before, dbefore, tmp, base, dbase);
  const uint2 c0 = g.batch_counts[2 * b], c1 = g.batch_counts[2 * b + 1];
  const uint32_t batch_in = c0.x + c1.x, batch_total = batch_in + c0.y + c1.y;
  // primitive ids seen by the pixel shader are per draw, as with one drawElements call each
  if (g.draw_prim_base && b == D.bbase && half == 0 && threadIdx.x == 0) g.draw_prim_base[d] = base;
  // effective order within the batch: every kept input slot (first half, then second),
  // then every extra fan triangle (first half's, then second's)
  const uint32_t in_base = base + (half ? c0.x : 0u);
  const uint32_t ex_base = base + batch_in + (half ? c0.y : 0u);
  const uint32_t q = threadIdx.x;
  uint32_t fl = 0, slot = 0xffffffffu, keep = 0, i0 = 0, i1 = 0, i2 = 0;
  if (q < n) {
    const uint32_t* ix = D.indices + (size_t)3 * (p0 + q);  // read early: used after the scan
    i0 = __ldg(ix);
    i1 = __ldg(ix + 1);
    i2 = __ldg(ix + 2);
    fl = g.tri_flags[D.pbase + p0 + q];
    if (fl & 4) {
      slot = g.clip_slot[D.pbase + p0 + q];
      if (slot != 0xffffffffu) keep = g.clip_table[slot].keep;
    } else {
      keep = fl & 1;
    }
  }
  // one scan of (kept input slot, extra fan triangles) packed in 16-bit halves: at most 512
  // and 512 * 13 per half batch, so the low half never carries
  uint32_t tot;
  const uint32_t ex = swr_block_exscan((keep & 1u) | ((uint32_t)__popc(keep >> 1) << 16), tmps, &tot);
  uint32_t rin = (ex & 0xffffu) + in_base;
  uint32_t rex = (ex >> 16) + ex_base;
  if (hb == nhb - 1 && threadIdx.x == 0) {
    g.status[SWR_ST_PRIMS] = base + batch_total;
    if (base + batch_total > g.cap_prims) atomicOr(&g.status[SWR_ST_FLAGS], SWR_F_PRIM_OVERFLOW);
  }
  if (base + batch_total > g.cap_prims) {
    if (threadIdx.x == 0) atomicOr(&g.status[SWR_ST_FLAGS], SWR_F_PRIM_OVERFLOW);
    return;
  }
  // source triangle (draw-relative) of the primitive emitted at global position `at`
  auto record_src = [&](uint32_t at, uint32_t src) {
    if (!D.prim_src) return;
    const uint32_t k = at - dbase;
    if (k < D.prim_src_cap) D.prim_src[k] = (int32_t)src;
    else atomicOr(&g.status[SWR_ST_FLAGS], SWR_F_SRC_OVERFLOW);
  };
  if (keep) {
    if (!(fl & 4)) {
      uint32_t r0 = D.vbase + i0, r1 = D.vbase + i1, r2 = D.vbase + i2;
      if (fl & 2) { const uint32_t t = r0; r0 = r2; r2 = t; }
      record_src(rin, p0 + q);
      g.tris[rin++] = make_uint4(r0, r1, r2, (uint32_t)d);
    } else {
      // first fan triangle in the input slot, the others after all of the batch's slots
      const SwrClipEntry e = g.clip_table[slot];
      for (int k = 0; k + 2 < e.n; ++k) {
        if (!((e.keep >> k) & 1)) continue;
        uint32_t r0 = e.ref[0], r1 = e.ref[k + 1], r2 = e.ref[k + 2];
        if ((e.swap >> k) & 1) { const uint32_t t = r0; r0 = r2; r2 = t; }
        if (k == 0) {
          record_src(rin, p0 + q);
          g.tris[rin++] = make_uint4(r0, r1, r2, (uint32_t)d);
        } else {
          record_src(rex, p0 + q);
          g.tris[rex++] = make_uint4(r0, r1, r2, (uint32_t)d);
        }
      }
    }
  }
}

template <int A, int P>
__global__ void __launch_bounds__(SWR_HALF) k_assemble_emit(AssembleArgs g) {
  swr_pdl_entry();
  assemble_emit_block<A, P>(g, blockIdx.x, gridDim.x);
}

// Grid barrier of a cooperative launch: bar[0] counts arrivals, bar[1] is the generation.
// The wait is bounded: past its limit the barrier sets SWR_F_BARRIER_TIMEOUT and returns
// false, and the caller skips the rest of its work (every CTA ends; none waits forever).
__device__ __forceinline__ bool swr_grid_sync(uint32_t* bar, uint32_t* status) {
  __shared__ int ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile uint32_t* gen = bar + 1;
    const uint32_t g0 = *gen;
    __threadfence();
    ok = 1;
    if (atomicAdd(bar, 1u) == gridDim.x - 1) {
      atomicExch(bar, 0u);  // reset before the release: the next barrier counts from zero
      __threadfence();
      atomicAdd(bar + 1, 1u);
    } else {
      uint32_t spins = 0;
      while (*gen == g0) {
        if (++spins > (1u << 24)) {  // seconds of waiting: give up
          atomicOr(&status[SWR_ST_FLAGS], SWR_F_BARRIER_TIMEOUT);
          ok = 0;
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
  }
  __syncthreads();
  return ok != 0;
}

// The geometry front end of a draw or batch in one persistent cooperative launch: vertex
// shading, then assembly's count and emit over every half batch, the CTAs staying resident
// and meeting at grid barriers between the stages (512 threads, the assembly's CTA size).
template <class VS>
__global__ void __launch_bounds__(SWR_HALF) k_geometry(const SwrDrawDesc* draws, int ndraws, const uint32_t* draw_vbase,
                                                       uint32_t nverts, float* ptv, AssembleArgs g, uint32_t nhb,
                                                       uint32_t* bar) {
  swr_pdl_entry();
  vertex_stage<VS>(draws, ndraws, draw_vbase, nverts, ptv);
  if (!swr_grid_sync(bar, g.status)) return;
  for (uint32_t hb = blockIdx.x; hb < nhb; hb += gridDim.x) {
    assemble_count_block<VS::AVarCount, VS::PVarCount>(g, hb);
    __syncthreads();  // the block's shared scratch is reused by its next half batch
  }
  if (!swr_grid_sync(bar, g.status)) return;
  for (uint32_t hb = blockIdx.x; hb < nhb; hb += gridDim.x) {
    assemble_emit_block<VS::AVarCount, VS::PVarCount>(g, hb, nhb);
    __syncthreads();
  }
}

// Direct Rasterizer path: triangles whose first index is -1 are skipped
// (Rasterizer::drawTriangleList, Rasterizer.h:134-141); others keep their order.
static __global__ void k_direct_flags(const int32_t* __restrict__ idx, uint32_t nprims, int per,
                               uint32_t* __restrict__ keep) {
  swr_pdl_entry();
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < nprims; p += gridDim.x * blockDim.x)
    keep[p] = idx[(size_t)per * p] != -1 ? 1u : 0u;
}

static __global__ void k_direct_emit(const int32_t* __restrict__ idx, uint32_t nprims, int per, uint32_t nverts,
                              const uint32_t* __restrict__ keep, const uint32_t* __restrict__ pos,
                              uint4* __restrict__ tris, uint32_t* status) {
  swr_pdl_entry();
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < nprims; p += gridDim.x * blockDim.x) {
    if (!keep[p]) continue;
    uint32_t r[3] = {0, 0, 0};
    for (int k = 0; k < per; ++k) {
      const int32_t i = idx[(size_t)per * p + k];
      if (i < 0 || (uint32_t)i >= nverts) {
        atomicOr(&status[SWR_ST_FLAGS], SWR_F_BAD_INDEX);
        r[k] = 0;
      } else {
        r[k] = (uint32_t)i;
      }
    }
    tris[pos[p]] = make_uint4(r[0], r[1], r[2], 0u);
  }
}

// ---------------------------------------------------------------------------------
// Triangle setup.

// Setup record layout for pixel shader PS (32-bit words).
template <class PS>
struct Rec {
  enum {
    NA = PS::AVarCount,
    NP = PS::PVarCount,
    IZ = PS::InterpolateZ ? 1 : 0,
    IW = (PS::InterpolateW || PS::PVarCount > 0) ? 1 : 0,
    NEQ = IZ + IW + NA + NP,
    EQ0 = 18,
    R = ((EQ0 + 3 * NEQ + 3) / 4) * 4,
    EQ_Z = 0,
    EQ_W = IZ,
    EQ_A = IZ + IW,
    EQ_P = IZ + IW + NA
  };
  // word 0 flags: bit0 drawable, bit1 block mode, bits2-4 tie of e0..e2, bit5 bottom half,
  //               bit6 top half
  // word 1 draw id; words 2-5 pixel bbox x0, y0, x1, y1 (inclusive, clamped to target)
  // block: words 6-14 e0.a e0.b e0.c e1.a e1.b e1.c e2.a e2.b e2.c
  // span:  words 6-11 bottom half yb0 yb1 t.x t.y is1 is2; 12-17 top half yt_hi yt_lo b.x b.y is1 is2
  // words 18.. (a, b, c) per interpolated equation: z, invw, avar[NA], pvar[NP]
};

struct Edge {
  float a, b, c;
  bool tie;
};

__device__ __forceinline__ Edge make_edge(float x0, float y0, float x1, float y1) {
  // EdgeEquation::init (EdgeEquation.h:37-43)
  Edge e;
  e.a = swr_sub(y0, y1);
  e.b = swr_sub(x1, x0);
  e.c = swr_div(-swr_add(swr_mul(e.a, swr_add(x0, x1)), swr_mul(e.b, swr_add(y0, y1))), 2.0f);
  e.tie = e.a != 0.0f ? e.a > 0.0f : e.b > 0.0f;
  return e;
}

// EdgeEquation::test (EdgeEquation.h): v > 0, or v == 0 on a tie edge.  Written as one
// comparison against a per-edge threshold: with denormals kept (no flush to zero) no float
// lies strictly between 0 and 2^-149, so v > 0 is v >= 2^-149; v == 0 (either zero) with
// the tie is v >= 0; NaN fails both, as it fails the reference's two comparisons.
__device__ __forceinline__ bool edge_test(float v, bool tie) { return v >= (tie ? 0.0f : 0x1p-149f); }

__device__ __forceinline__ void param_eq(float p0, float p1, float p2, const Edge& e0, const Edge& e1,
                                         const Edge& e2, float f, float* o) {
  // ParameterEquation::init (ParameterEquation.h:36-48)
  o[0] = swr_mul(f, swr_add(swr_add(swr_mul(p0, e0.a), swr_mul(p1, e1.a)), swr_mul(p2, e2.a)));
  o[1] = swr_mul(f, swr_add(swr_add(swr_mul(p0, e0.b), swr_mul(p1, e1.b)), swr_mul(p2, e2.b)));
  o[2] = swr_mul(f, swr_add(swr_add(swr_mul(p0, e0.c), swr_mul(p1, e1.c)), swr_mul(p2, e2.c)));
}

struct SetupArgs {
  const uint4* tris;
  const uint32_t* status;  // SWR_ST_PRIMS = primitive count
  uint32_t cap_prims;
  const float* ptv;
  const float* clipv;
  int S, off_a, off_p, vs_a, vs_p;
  const SwrDrawDesc* draws;
  const SwrTargetDesc* targets;
  float* recs;
  uint32_t* tile_count;
  int tile;  // tile edge in pixels
  uint32_t* cell_count;  // per (tile, primitive segment): bin entries (counted with atomics)
  int seg_shift;         // primitive segment = primitive index >> seg_shift (< SWR_SEGS)
};

struct SpanHalf {
  float ox, oy, is1, is2;
  int y0, y1;  // bottom: rows [y0, y1); top: rows (y1, y0]
};

// x extent (xl of the first pixel, xr exclusive) of row y of a span half.
__device__ __forceinline__ void span_row(const SpanHalf& h, int y, int minx, int maxx, int& xl, int& xr) {
  const float dy = swr_add(swr_sub((float)y, h.oy), 0.5f);
  const float c1 = swr_add(swr_add(h.ox, swr_mul(h.is1, dy)), 0.5f);
  const float c2 = swr_add(swr_add(h.ox, swr_mul(h.is2, dy)), 0.5f);
  xl = swr_maxi(minx, swr_trunc_int(c1));
  xr = swr_mini(maxx, swr_trunc_int(c2));
}

// Records are assembled in shared memory and written out as contiguous float4 runs
// (one record per thread would be a 4-byte store per 160-byte stride).
constexpr int kSetupThreads = 128;

template <class PS>
__global__ void __launch_bounds__(kSetupThreads) k_setup(SetupArgs g) {
  swr_pdl_entry();
  typedef Rec<PS> RL;
  // records staged with an odd stride, so the threads' scalar stores of one field fall in
  // 32 different banks (a stride of R = 40 words put 32 threads in 4 banks)
  constexpr int RS = RL::R + 1;
  __shared__ float stage[kSetupThreads * RS];
  if (g.status[SWR_ST_FLAGS] & SWR_F_ANY_OVERFLOW) return;
  uint32_t np = g.status[SWR_ST_PRIMS];
  if (np > g.cap_prims) np = g.cap_prims;
  for (uint32_t p0 = blockIdx.x * kSetupThreads; p0 < np; p0 += gridDim.x * kSetupThreads) {
  const uint32_t p = p0 + threadIdx.x;
  if (p < np) {
    const uint4 t = g.tris[p];
    const SwrDrawDesc& D = g.draws[t.w];
    const SwrTargetDesc& T = g.targets[D.target];
    const uint32_t rr[3] = {t.x, t.y, t.z};
    float x[3], y[3], z[3], w[3];
    float av[3][RL::NA > 0 ? RL::NA : 1], pv[3][RL::NP > 0 ? RL::NP : 1];
    // Post-transform records (16-byte aligned): words 0-3 clip position, 4-6 screen x, y, z,
    // then the vertex shader's avars and pvars.  Records of at most 16 words with the avars
    // at word 8 and 0 or 3 of them (every built-in vertex shader) are read as float4s;
    // scattered scalar reads of 9 words per vertex made the stage L1-wavefront bound.
    const bool vec = g.S <= 16 && g.off_a == 8 && g.off_p == 8 + g.vs_a && (g.vs_a == 0 || g.vs_a == 3);
    for (int k = 0; k < 3; ++k) {
      const float* vp = (rr[k] & SWR_CLIP_REF) ? g.clipv + (size_t)(rr[k] & ~SWR_CLIP_REF) * g.S
                                               : g.ptv + (size_t)rr[k] * g.S;
      if (vec) {
        const float4 q0 = __ldg((const float4*)vp), q1 = __ldg((const float4*)vp + 1);
        const float4 q2 = g.S > 8 ? __ldg((const float4*)vp + 2) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        const float4 q3 = g.S > 12 ? __ldg((const float4*)vp + 3) : make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        const float at[8] = {q2.x, q2.y, q2.z, q2.w, q3.x, q3.y, q3.z, q3.w};
        w[k] = q0.w;
        x[k] = q1.x; y[k] = q1.y; z[k] = q1.z;
#pragma unroll
        for (int i = 0; i < RL::NA; ++i) av[k][i] = i < g.vs_a ? at[i] : 0.0f;
#pragma unroll
        for (int i = 0; i < RL::NP; ++i) pv[k][i] = i < g.vs_p ? (g.vs_a ? at[(3 + i) & 7] : at[i]) : 0.0f;
      } else {
        x[k] = vp[4]; y[k] = vp[5]; z[k] = vp[6]; w[k] = vp[3];
        for (int i = 0; i < RL::NA; ++i) av[k][i] = i < g.vs_a ? vp[g.off_a + i] : 0.0f;
        for (int i = 0; i < RL::NP; ++i) pv[k][i] = i < g.vs_p ? vp[g.off_p + i] : 0.0f;
      }
    }
    float* rec = stage + threadIdx.x * RS;
    uint32_t tiles = 0;
    // TriangleEquations: e0 = (v1, v2), e1 = (v2, v0), e2 = (v0, v1)
    const Edge e0 = make_edge(x[1], y[1], x[2], y[2]);
    const Edge e1 = make_edge(x[2], y[2], x[0], y[0]);
    const Edge e2 = make_edge(x[0], y[0], x[1], y[1]);
    const float area2 = swr_add(swr_add(e0.c, e1.c), e2.c);
    int flags = 0;
    int bx0 = 0, by0 = 0, bx1 = -1, by1 = -1;
    if (!(area2 <= 0.0f)) {
      flags = 1 | (e0.tie ? 4 : 0) | (e1.tie ? 8 : 0) | (e2.tie ? 16 : 0);
      const float factor = swr_div(1.0f, area2);
      float* eq = rec + RL::EQ0;
      if (RL::IZ) param_eq(z[0], z[1], z[2], e0, e1, e2, factor, eq + 3 * RL::EQ_Z);
      const float iw0 = swr_div(1.0f, w[0]), iw1 = swr_div(1.0f, w[1]), iw2 = swr_div(1.0f, w[2]);
      if (RL::IW) param_eq(iw0, iw1, iw2, e0, e1, e2, factor, eq + 3 * RL::EQ_W);
      for (int i = 0; i < RL::NA; ++i) param_eq(av[0][i], av[1][i], av[2][i], e0, e1, e2, factor, eq + 3 * (RL::EQ_A + i));
      for (int i = 0; i < RL::NP; ++i)
        param_eq(swr_mul(pv[0][i], iw0), swr_mul(pv[1][i], iw1), swr_mul(pv[2][i], iw2), e0, e1, e2, factor,
                 eq + 3 * (RL::EQ_P + i));
      // Raster mode (Rasterizer.h:414-446); Adaptive compares the float ratio as double.
      bool block = D.raster_mode == 1;
      if (D.raster_mode == 2) {
        const float fx0 = swr_minf(swr_minf(x[0], x[1]), x[2]), fx1 = swr_maxf(swr_maxf(x[0], x[1]), x[2]);
        const float fy0 = swr_minf(swr_minf(y[0], y[1]), y[2]), fy1 = swr_maxf(swr_maxf(y[0], y[1]), y[2]);
        const float orient = swr_div(swr_sub(fx1, fx0), swr_sub(fy1, fy0));
        block = (double)orient > 0.4 && (double)orient < 1.6;
      }
      if (block) {
        flags |= 2;
        // Rasterizer.h:235-255
        int mnx = swr_trunc_int(swr_minf(swr_minf(x[0], x[1]), x[2]));
        int mxx = swr_trunc_int(swr_maxf(swr_maxf(x[0], x[1]), x[2]));
        int mny = swr_trunc_int(swr_minf(swr_minf(y[0], y[1]), y[2]));
        int mxy = swr_trunc_int(swr_maxf(swr_maxf(y[0], y[1]), y[2]));
        mnx = swr_maxi(mnx, D.sc_minx);
        mxx = swr_mini(mxx, D.sc_maxx);
        mny = swr_maxi(mny, D.sc_miny);
        mxy = swr_mini(mxy, D.sc_maxy);
        mnx &= ~(SWR_BLOCK - 1);
        mxx &= ~(SWR_BLOCK - 1);
        mny &= ~(SWR_BLOCK - 1);
        mxy &= ~(SWR_BLOCK - 1);
        const int sx = (mxx - mnx) / SWR_BLOCK + 1, sy = (mxy - mny) / SWR_BLOCK + 1;
        // Blocks visited by i in [0, sx*sy): (mnx + (i % sx) * 8, mny + (i / sx) * 8).
        if (sx > 0 && sy > 0) {
          bx0 = mnx; bx1 = mnx + SWR_BLOCK * (sx - 1) + SWR_BLOCK - 1;
          by0 = mny; by1 = mny + SWR_BLOCK * (sy - 1) + SWR_BLOCK - 1;
        } else if (sx < 0 && sy < 0) {
          bx0 = mnx; bx1 = mnx + SWR_BLOCK * (-sx - 1) + SWR_BLOCK - 1;
          by0 = mny - SWR_BLOCK * (-sy - 1); by1 = mny + SWR_BLOCK - 1;
        }
        rec[6] = e0.a; rec[7] = e0.b; rec[8] = e0.c;
        rec[9] = e1.a; rec[10] = e1.b; rec[11] = e1.c;
        rec[12] = e2.a; rec[13] = e2.b; rec[14] = e2.c;
      } else {
        // Rasterizer.h:318-357
        int it = 0, im = 1, ib = 2;
        if (y[it] > y[im]) { const int q = it; it = im; im = q; }
        if (y[im] > y[ib]) { const int q = im; im = ib; ib = q; }
        if (y[it] > y[im]) { const int q = it; it = im; im = q; }
        const float dy = swr_sub(y[ib], y[it]);
        const float iy = swr_sub(y[im], y[it]);
        SpanHalf bot, top;
        bool has_bot = false, has_top = false;
        float lx, ly, rx, ry;
        if (y[im] == y[it]) {
          lx = x[im]; ly = y[im]; rx = x[it]; ry = y[it];
          if (lx > rx) { float q = lx; lx = rx; rx = q; q = ly; ly = ry; ry = q; }
          has_top = true;
        } else if (y[im] == y[ib]) {
          lx = x[im]; ly = y[im]; rx = x[ib]; ry = y[ib];
          if (lx > rx) { float q = lx; lx = rx; rx = q; q = ly; ly = ry; ry = q; }
          has_bot = true;
        } else {
          const float v4x = swr_add(x[it], swr_mul(swr_div(swr_sub(x[ib], x[it]), dy), iy));
          lx = x[im]; ly = y[im]; rx = v4x; ry = y[im];
          if (lx > rx) { float q = lx; lx = rx; rx = q; q = ly; ly = ry; ry = q; }
          has_bot = has_top = true;
        }
        if (has_bot) {  // drawBottomFlatTriangle(t, l, r) (Rasterizer.h:361-385)
          bot.ox = x[it]; bot.oy = y[it];
          bot.is1 = swr_div(swr_sub(lx, x[it]), swr_sub(ly, y[it]));
          bot.is2 = swr_div(swr_sub(rx, x[it]), swr_sub(ry, y[it]));
          bot.y0 = swr_trunc_int(swr_add(y[it], 0.5f));
          bot.y1 = swr_trunc_int(swr_add(ly, 0.5f));
        } else {
          bot.ox = bot.oy = bot.is1 = bot.is2 = 0.0f;
          bot.y0 = bot.y1 = 0;
        }
        if (has_top) {  // drawTopFlatTriangle(l, r, b) (Rasterizer.h:388-411)
          top.ox = x[ib]; top.oy = y[ib];
          top.is1 = swr_div(swr_sub(x[ib], lx), swr_sub(y[ib], ly));
          top.is2 = swr_div(swr_sub(x[ib], rx), swr_sub(y[ib], ry));
          top.y0 = swr_trunc_int(swr_sub(y[ib], 0.5f));
          top.y1 = swr_trunc_int(swr_sub(ly, 0.5f));
        } else {
          top.ox = top.oy = top.is1 = top.is2 = 0.0f;
          top.y0 = top.y1 = 0;
        }
        if (has_bot) flags |= 32;
        if (has_top) flags |= 64;
        rec[6] = __int_as_float(bot.y0); rec[7] = __int_as_float(bot.y1);
        rec[8] = bot.ox; rec[9] = bot.oy; rec[10] = bot.is1; rec[11] = bot.is2;
        rec[12] = __int_as_float(top.y0); rec[13] = __int_as_float(top.y1);
        rec[14] = top.ox; rec[15] = top.oy; rec[16] = top.is1; rec[17] = top.is2;
        // Conservative pixel box: rows inside the target, x from the end rows of each
        // half (the span edges are linear in y up to rounding, hence the 2 px margin).
        int rx0 = 0x7fffffff, rx1 = -0x7fffffff, ry0 = 0x7fffffff, ry1 = -0x7fffffff;
        for (int hh = 0; hh < 2; ++hh) {
          const SpanHalf& h = hh ? top : bot;
          if (!(hh ? has_top : has_bot)) continue;
          int lo = hh ? h.y1 + 1 : h.y0, hi = hh ? h.y0 : h.y1 - 1;
          lo = swr_maxi(lo, 0);
          hi = swr_mini(hi, T.height - 1);
          if (lo > hi) continue;
          ry0 = swr_mini(ry0, lo);
          ry1 = swr_maxi(ry1, hi);
          for (int e = 0; e < 2; ++e) {
            int xl, xr;
            span_row(h, e ? hi : lo, D.sc_minx, D.sc_maxx, xl, xr);
            rx0 = swr_mini(rx0, xl);
            rx1 = swr_maxi(rx1, xr - 1);
          }
        }
        if (ry0 <= ry1) {
          bx0 = swr_maxi(rx0 - 2, D.sc_minx);
          bx1 = swr_mini(rx1 + 2, D.sc_maxx - 1);
          by0 = ry0;
          by1 = ry1;
        }
      }
      bx0 = swr_maxi(bx0, 0);
      by0 = swr_maxi(by0, 0);
      bx1 = swr_mini(bx1, T.width - 1);
      by1 = swr_mini(by1, T.height - 1);
      if (bx0 <= bx1 && by0 <= by1) {
        const int tx0 = bx0 / g.tile, tx1 = bx1 / g.tile, ty0 = by0 / g.tile, ty1 = by1 / g.tile;
        tiles = (uint32_t)((tx1 - tx0 + 1) * (ty1 - ty0 + 1));
        if (g.cell_count) {
          const uint32_t seg = p >> g.seg_shift;
          for (int ty = ty0; ty <= ty1; ++ty)
            for (int tx = tx0; tx <= tx1; ++tx)
              atomicAdd(&g.cell_count[(T.tile_base + (uint32_t)(ty * T.tiles_x + tx)) * SWR_SEGS + seg], 1u);
        }
      } else {
        flags = 0;
      }
    }
    rec[0] = __int_as_float(flags);
    rec[1] = __int_as_float((int)t.w);
    rec[2] = __int_as_float(bx0); rec[3] = __int_as_float(by0);
    rec[4] = __int_as_float(bx1); rec[5] = __int_as_float(by1);
    g.tile_count[p] = flags ? tiles : 0u;
  }
  __syncthreads();
  const uint32_t cnt = min((uint32_t)kSetupThreads, np - p0);
  float4* dst = (float4*)(g.recs + (size_t)p0 * RL::R);
  for (uint32_t i = threadIdx.x; i < cnt * (RL::R / 4); i += kSetupThreads) {
    const uint32_t t = i / (RL::R / 4);
    const float* src = stage + t * RS + (i - t * (RL::R / 4)) * 4;
    dst[i] = make_float4(src[0], src[1], src[2], src[3]);
  }
  __syncthreads();
  }
}

// (tile, primitive) pairs in primitive order.
template <class PS>
__global__ void __launch_bounds__(256) k_emit_pairs(const uint32_t* status, uint32_t cap_prims, const float* recs,
                                                    const uint32_t* tile_count, const uint32_t* pair_off,
                                                    const uint32_t* npairs, uint32_t cap_pairs,
                                                    const SwrDrawDesc* draws, const SwrTargetDesc* targets,
                                                    int tile, uint32_t* keys, uint32_t* vals,
                                                    uint32_t* status_w) {
  swr_pdl_entry();
  typedef Rec<PS> RL;
  if (status[SWR_ST_FLAGS] & SWR_F_ANY_OVERFLOW) return;
  if (*npairs > cap_pairs) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      atomicOr(&status_w[SWR_ST_FLAGS], SWR_F_PAIR_OVERFLOW);
      status_w[SWR_ST_PAIRS] = *npairs;
    }
    return;
  }
  uint32_t np = status[SWR_ST_PRIMS];
  if (np > cap_prims) np = cap_prims;
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) {
    if (!tile_count[p]) continue;
    const float* rec = recs + (size_t)p * RL::R;
    const int d = __float_as_int(rec[1]);
    const SwrTargetDesc& T = targets[draws[d].target];
    const int tx0 = __float_as_int(rec[2]) / tile, ty0 = __float_as_int(rec[3]) / tile;
    const int tx1 = __float_as_int(rec[4]) / tile, ty1 = __float_as_int(rec[5]) / tile;
    uint32_t o = pair_off[p];
    for (int ty = ty0; ty <= ty1; ++ty)
      for (int tx = tx0; tx <= tx1; ++tx) {
        keys[o] = T.tile_base + (uint32_t)(ty * T.tiles_x + tx);
        vals[o] = p;
        o++;
      }
  }
}

// Segmented binning.  The primitive list is cut into SWR_SEGS contiguous segments; a
// (tile, segment) cell holds the segment's primitives that touch the tile.  Cells are laid
// out tile-major, so a tile's bin is one contiguous range ordered by segment; inside a cell
// the fill order is arbitrary and k_sort_cells restores increasing primitive order.
template <class PS>
__global__ void __launch_bounds__(256) k_fill_bins(const uint32_t* status, uint32_t cap_prims, const float* recs,
                                                   uint32_t* cell_count,
                                                   const uint32_t* cell_start, uint32_t ncells, int seg_shift,
                                                   uint32_t cap_pairs, const SwrDrawDesc* draws,
                                                   const SwrTargetDesc* targets, int tile, uint32_t* bin,
                                                   uint32_t* status_w) {
  swr_pdl_entry();
  typedef Rec<PS> RL;
  // cell_count is all zero between draws: every entry counted by k_setup is taken back
  // here, and a draw that stops early zeroes the counts instead
  const uint32_t total = cell_start[ncells];
  const bool overflow = status[SWR_ST_FLAGS] & SWR_F_ANY_OVERFLOW;
  if (overflow || total > cap_pairs) {
    if (!overflow && blockIdx.x == 0 && threadIdx.x == 0) {
      atomicOr(&status_w[SWR_ST_FLAGS], SWR_F_PAIR_OVERFLOW);
      status_w[SWR_ST_PAIRS] = total;
    }
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < ncells; i += gridDim.x * blockDim.x) cell_count[i] = 0u;
    return;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) status_w[SWR_ST_PAIRS] = total;
  uint32_t np = status[SWR_ST_PRIMS];
  if (np > cap_prims) np = cap_prims;
  // draw 0's target, read up front: every primitive of a single-draw submission uses it
  const SwrTargetDesc& T0 = targets[draws[0].target];
  const uint32_t tb0 = T0.tile_base;
  const int tw0 = T0.tiles_x;
  const int tshift = __ffs(tile) - 1;  // tiles are 16 or 32 pixels; pixel boxes are >= 0
  const int lane = threadIdx.x & 31;
  // one warp per 32 consecutive primitives (the loop is uniform per warp)
  const uint32_t stride = gridDim.x * blockDim.x;
  for (uint32_t p0 = (blockIdx.x * blockDim.x + threadIdx.x) & ~31u; p0 < np; p0 += stride) {
    const uint32_t p = p0 + (uint32_t)lane;
    // record words 0-5: flags (0: no tile, as tile_count), draw, pixel box (two float4
    // reads of the 16-byte aligned record)
    int tx0 = 0, ty0 = 0, nx = 1, cnt = 0;
    uint32_t tbase = tb0;
    int tiles_x = tw0;
    if (p < np) {
      const float4 q0 = __ldg((const float4*)(recs + (size_t)p * RL::R));
      const float4 q1 = __ldg((const float4*)(recs + (size_t)p * RL::R) + 1);
      if (__float_as_int(q0.x)) {
        const int d = __float_as_int(q0.y);
        if (d != 0) {
          const SwrTargetDesc& T = targets[draws[d].target];
          tbase = T.tile_base;
          tiles_x = T.tiles_x;
        }
        tx0 = __float_as_int(q0.z) >> tshift;
        ty0 = __float_as_int(q0.w) >> tshift;
        nx = (__float_as_int(q1.x) >> tshift) - tx0 + 1;
        cnt = nx * ((__float_as_int(q1.y) >> tshift) - ty0 + 1);
      }
    }
    const uint32_t seg = p >> seg_shift;
    auto put = [&](uint32_t prim, uint32_t pseg, uint32_t tb, int tw, int tx, int ty) {
      const uint32_t cell = (tb + (uint32_t)(ty * tw + tx)) * SWR_SEGS + pseg;
      const uint32_t pos = atomicSub(&cell_count[cell], 1u) - 1u;
      bin[cell_start[cell] + pos] = prim;
    };
    if (__reduce_max_sync(0xffffffffu, (uint32_t)cnt) <= 2u) {
      // small primitives (the common case): every lane its own tiles
      for (int i = 0; i < cnt; ++i) put(p, seg, tbase, tiles_x, tx0 + (i < nx ? i : i - nx), ty0 + (i < nx ? 0 : 1));
      continue;
    }
    // some primitive spans more tiles: the warp's (primitive, tile) pairs are spread over its
    // lanes, 32 at a time, so one large primitive does not serialise the warp
    int inc = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o) inc += y;
    }
    const int total = __shfl_sync(0xffffffffu, inc, 31);
    for (int base = 0; base < total; base += 32) {
      const int j = base + lane;
      // owner: the number of lanes whose inclusive count is <= j
      int src = 0;
#pragma unroll
      for (int step = 16; step; step >>= 1) {
        const int v = __shfl_sync(0xffffffffu, inc, src + step - 1);
        if (v <= j) src += step;
      }
      src = src < 31 ? src : 31;
      const int first = __shfl_sync(0xffffffffu, inc - cnt, src);
      const int onx = __shfl_sync(0xffffffffu, nx, src);
      const int otx0 = __shfl_sync(0xffffffffu, tx0, src);
      const int oty0 = __shfl_sync(0xffffffffu, ty0, src);
      const uint32_t otb = __shfl_sync(0xffffffffu, tbase, src);
      const int otw = __shfl_sync(0xffffffffu, tiles_x, src);
      if (j < total) {
        const int local = j - first;
        const int ry = local / onx;
        put(p0 + (uint32_t)src, (p0 + (uint32_t)src) >> seg_shift, otb, otw, otx0 + (local - ry * onx), oty0 + ry);
      }
    }
  }
}

// One warp per tile: every cell of the tile is copied to `out` in increasing primitive
// order.  Lane c owns cell c: cells of up to 16 entries are sorted in registers by the
// lane; cells of up to 64 are ranked by the whole warp (primitive ids are unique); larger
// cells go to `big_list` for k_sort_big when it is given (its capacity is the cell count,
// so it cannot overflow), else the warp ranks them too.
static __global__ void __launch_bounds__(256) k_sort_cells(const uint32_t* status, const uint32_t* cell_start,
                                                          uint32_t ntiles, uint32_t cap_pairs, const uint32_t* in,
                                                          uint32_t* out, uint32_t* big_list, uint32_t* big_count,
                                                          uint32_t self_sorted, uint8_t* quad_flag,
                                                          uint32_t* quad_tiles, uint32_t* quad_count,
                                                          uint32_t quad_cap, uint32_t quad_min) {
  swr_pdl_entry();
  if (status[SWR_ST_FLAGS] & SWR_F_ANY_OVERFLOW) return;
  if (cell_start[(size_t)ntiles * SWR_SEGS] > cap_pairs) return;
  const int lane = threadIdx.x & 31;
  const uint32_t t = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  if (t >= ntiles) return;
  const uint32_t last = cell_start[(size_t)t * SWR_SEGS + SWR_SEGS];
  // heavy tiles: listed for k_raster's quadrant CTAs (quad_count is zeroed before this kernel)
  if (quad_flag && lane == 0) {
    uint8_t f = 0;
    if (last - cell_start[(size_t)t * SWR_SEGS] > quad_min) {
      const uint32_t slot = atomicAdd(quad_count, 1u);
      if (slot < quad_cap) {
        quad_tiles[slot] = t;
        f = 1;
      }
    }
    quad_flag[t] = f;
  }
  // tiles of at most `self_sorted` entries are ordered by the raster kernel itself
  if (last - cell_start[(size_t)t * SWR_SEGS] <= self_sorted) return;  // uniform per warp
  const uint32_t s = cell_start[(size_t)t * SWR_SEGS + lane];
  // every lane takes part in the shuffle; lane 31 then uses the next tile's first start
  const uint32_t nxt = __shfl_down_sync(0xffffffffu, s, 1);
  const uint32_t e = lane < SWR_SEGS - 1 ? nxt : last;
  // starts are an exclusive scan (monotone, bounded by the total <= cap_pairs); anything
  // else leaves the cell empty instead of walking a wrapped length
  const uint32_t m = (e >= s && e <= cap_pairs) ? e - s : 0u;
  constexpr int kSmall = 16;
  if (m <= kSmall) {
    uint32_t v[kSmall];
#pragma unroll
    for (int i = 0; i < kSmall; ++i) v[i] = (uint32_t)i < m ? in[s + i] : 0xffffffffu;
    // odd-even transposition network on 16 registers
#pragma unroll
    for (int r = 0; r < kSmall; ++r)
#pragma unroll
      for (int i = r & 1; i + 1 < kSmall; i += 2)
        if (v[i] > v[i + 1]) { const uint32_t x = v[i]; v[i] = v[i + 1]; v[i + 1] = x; }
#pragma unroll
    for (int i = 0; i < kSmall; ++i)
      if ((uint32_t)i < m) out[s + i] = v[i];
  }
  constexpr uint32_t kListed = 64;  // above this the warp rank sort below costs more than a bitmap
  const bool listed = big_list && m > kListed;
  if (listed) big_list[atomicAdd(big_count, 1u)] = t * SWR_SEGS + (uint32_t)lane;
  uint32_t big = __ballot_sync(0xffffffffu, m > kSmall && !listed);
  while (big) {
    const int c = __ffs(big) - 1;
    big &= big - 1u;
    const uint32_t cs = __shfl_sync(0xffffffffu, s, c), cm = __shfl_sync(0xffffffffu, m, c);
    for (uint32_t i0 = 0; i0 < cm; i0 += 32) {
      const uint32_t i = i0 + lane;
      const uint32_t val = i < cm ? in[cs + i] : 0xffffffffu;
      uint32_t rank = 0;
      for (uint32_t j0 = 0; j0 < cm; j0 += 32) {
        const uint32_t w = j0 + lane < cm ? in[cs + j0 + lane] : 0xffffffffu;
#pragma unroll 8
        for (int l = 0; l < 32; ++l) rank += __shfl_sync(0xffffffffu, w, l) < val;
      }
      if (i < cm) out[cs + rank] = val;
    }
  }
}

// The cells listed by k_sort_cells, one warp per cell (grid-stride over the list): the ids
// of cell (tile, seg) all lie in segment seg's range [seg << shift, (seg + 1) << shift), so
// a bitmap of that range in the warp's slice of shared memory sorts them: set one bit per
// id (only the words between the cell's smallest and largest id are touched), prefix-count
// the words across the lanes, write the set bits out in order.  Dynamic shared memory:
// (1 << shift) / 8 bytes per warp.  big_count[0] is the list length (reset after the draw).
static __global__ void k_sort_big(uint32_t* status, const uint32_t* cell_start, uint32_t ncells,
                                  uint32_t cap_pairs, int seg_shift, const uint32_t* in, uint32_t* out,
                                  const uint32_t* big_list, uint32_t* big_count) {
  swr_pdl_entry();
  extern __shared__ uint32_t smem_bm[];
  const bool skip = (status[SWR_ST_FLAGS] & SWR_F_ANY_OVERFLOW) || cell_start[ncells] > cap_pairs;
  const uint32_t nbig = skip ? 0u : min(*(volatile uint32_t*)big_count, ncells);
  const uint32_t R = 1u << seg_shift;
  const int lane = threadIdx.x & 31, wib = threadIdx.x >> 5;
  uint32_t* bm = smem_bm + (size_t)wib * (R >> 5);
  const uint32_t nwarps = gridDim.x * (blockDim.x >> 5);
  for (uint32_t bi = blockIdx.x * (blockDim.x >> 5) + wib; bi < nbig; bi += nwarps) {
    const uint32_t cell = big_list[bi];
    if (cell >= ncells) continue;  // uniform per warp
    const uint32_t s = cell_start[cell], e = cell_start[cell + 1];
    const uint32_t m = (e >= s && e <= cap_pairs) ? e - s : 0u;
    const uint32_t lo_id = (cell % SWR_SEGS) << seg_shift;
    uint32_t lo = 0xffffffffu, hi = 0u;
    for (uint32_t j = lane; j < m; j += 32) {
      const uint32_t v = in[s + j] - lo_id;
      if (v < R) {
        lo = min(lo, v);
        hi = max(hi, v);
      }
    }
    lo = __reduce_min_sync(0xffffffffu, lo);
    hi = __reduce_max_sync(0xffffffffu, hi);
    if (lo > hi) continue;  // uniform: no valid id
    const uint32_t w0 = lo >> 5, nw = (hi >> 5) - w0 + 1;
    for (uint32_t w = lane; w < nw; w += 32) bm[w0 + w] = 0u;
    __syncwarp();
    for (uint32_t j = lane; j < m; j += 32) {
      const uint32_t v = in[s + j] - lo_id;
      if (v < R) atomicOr(&bm[v >> 5], 1u << (v & 31));
    }
    __syncwarp();
    // lane l owns words [l * per, (l + 1) * per) of the range
    const uint32_t per = (nw + 31) / 32;
    const uint32_t a = min(nw, (uint32_t)lane * per), b = min(nw, a + per);
    uint32_t cnt = 0;
    for (uint32_t w = a; w < b; ++w) cnt += __popc(bm[w0 + w]);
    uint32_t inc = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, inc, o);
      if (lane >= o) inc += y;
    }
    uint32_t pos = inc - cnt;
    for (uint32_t w = a; w < b; ++w) {
      uint32_t bits = bm[w0 + w];
      while (bits) {
        const int bit = __ffs(bits) - 1;
        bits &= bits - 1u;
        if (pos < m) out[s + pos] = lo_id + ((w0 + w) << 5) + (uint32_t)bit;
        ++pos;
      }
    }
    __syncwarp();
  }
  // The last block to finish closes the draw: the list ([length, blocks done]) is consumed,
  // and every counting stage has run (the tile raster counts only fragments).
  __syncthreads();
  if (threadIdx.x == 0) {
    __threadfence();
    if (atomicAdd(&big_count[1], 1u) == gridDim.x - 1) {
      swr_close_status(status);
      big_count[0] = 0u;
      big_count[1] = 0u;
    }
  }
}

// ---------------------------------------------------------------------------------
// Tile rasterization.

template <class PS>
struct GpuPixel {  // PixelData (PixelData.h:35-146) as seen by drawPixel
  int x, y;
  float z, w, invw;
  float avar[PS::AVarCount > 0 ? PS::AVarCount : 1];
  float pvar[PS::PVarCount > 0 ? PS::PVarCount : 1];
  const float* eq;  // the triangle's parameter equations (PixelData::equations); null for points and lines
};

// PixelData::computePerspectiveDerivatives(*equations, i, ddx, ddy) for the pixel shaders
// (found by argument-dependent lookup from swr_programs.h).
template <class PS>
__device__ __forceinline__ void swr_persp_deriv(const GpuPixel<PS>& p, int i, float& ddx, float& ddy) {
  if (!p.eq) {
    ddx = ddy = 0.0f;
    return;
  }
  typedef Rec<PS> RL;
  swr_persp_deriv_eq(p.eq + 3 * (RL::EQ_P + i), p.eq + 3 * RL::EQ_W, p.x, p.y, ddx, ddy);
}

struct RasterArgs {
  const uint32_t* status;
  const uint32_t* tile_start;  // bin start of tile t at tile_start[t * tile_stride] (plus the end)
  uint32_t tile_stride;        // 1 for per-tile starts, SWR_SEGS for per-(tile, segment) cells
  const uint32_t* bin;         // primitive ids, each tile's range in increasing order
  const uint32_t* bin_raw;     // optional: the unsorted ids (cell layout, tile_stride SWR_SEGS);
                               // tiles of <= SWR_RASTER_SORT entries order them in the kernel
                               // (k_sort_cells skips them)
  const float* recs;
  const SwrDrawDesc* draws;
  const SwrTargetDesc* targets;
  const uint32_t* target_tile_base;  // per target, for the tile -> target lookup
  int ntargets;
  const uint32_t* draw_prim_base;    // per draw first primitive (null: a single draw from 0)
  uint32_t* status_w;
  uint32_t ntiles;
  int slices;                        // overwrite shaders: CTAs per tile of more than SWR_RASTER_SORT
                                     // entries (1: no slicing), each over an ordered slice of its bin
  void* slice_state;                 // their per-pixel PS::State, [tile][slice][TILE * TILE]
  int has_span;                      // some draw rasterizes in Span or Adaptive mode (selects k_raster<..., true>)
  // Quadrant CTAs (16-px tiles, shaders other than the overwrite ones): a heavy tile -- more
  // than quad_min bin entries; k_sort_cells lists up to quad_cap of them -- is rasterized by
  // four CTAs, one per 8 x 8 quadrant, each walking the whole bin for its own pixels, so the
  // slowest tiles no longer set the kernel's length.  CTAs [0, 4 quad_cap) take the listed
  // tiles' quadrants first; CTA 4 quad_cap + t takes tile t unless it is listed.  With
  // quad_all every tile is split (CTA 4 t + q: quadrant q of tile t): an 8-px raster tile
  // over 16-px bins.
  const uint8_t* quad_flag;          // per tile: 1 = listed (null: no heavy-tile split)
  const uint32_t* quad_tiles;        // listed tiles
  const uint32_t* quad_count;        // tiles k_sort_cells listed (may exceed quad_cap)
  uint32_t quad_cap;
  int quad_all;
  // Sliced heavy tiles (depth-min shaders, SwrDepthMin): with dslice set, each tile of the
  // same list is rasterized by SWR_DSLICES CTAs instead, each over a run of whole chunks of
  // its ordered bin and from the draw's starting State; each writes its States to
  // dslice_state, and the last of the tile's CTAs to finish merges them in bin order
  // (swr_depth_merge) and stores.  CTAs [0, SWR_DSLICES quad_cap) take the listed tiles'
  // slices; CTA SWR_DSLICES quad_cap + t takes tile t unless it is listed.
  int dslice;
  void* dslice_state;      // [slot][slice][TILE * TILE] PS::State
  uint32_t* dslice_done;   // per slot: the slices finished (zero between draws)
};

// v <- fl(v + a) repeated k times for 0 <= k <= 7 (steps inside one 8x8 block), as
// predicated adds so the lanes of a warp never diverge.
__device__ __forceinline__ float fold7(float v, float a, int k) {
#pragma unroll
  for (int i = 0; i < 7; ++i) v = i < k ? swr_add(v, a) : v;
  return v;
}

// Block classification of Rasterizer.h:263-304 for the block at (bx, by): 0 = skipped,
// 1 = drawBlock<false> (every pixel), 2 = drawBlock<true> (per-pixel edge tests).
__device__ __forceinline__ int block_class(const float* r, int flags, int bx, int by) {
  const float fx = swr_add((float)bx, 0.5f), fy = swr_add((float)by, 0.5f);
  const float s = (float)(SWR_BLOCK - 1);
  bool t00[3], t01[3], t10[3], t11[3];
#pragma unroll
  for (int j = 0; j < 3; ++j) {
    const float ea = r[6 + 3 * j], eb = r[7 + 3 * j], ec = r[8 + 3 * j];
    const bool tie = (flags >> (2 + j)) & 1;
    const float ev = swr_eval(ea, eb, ec, fx, fy);
    const float v01 = swr_add(ev, swr_mul(eb, s));
    const float v10 = swr_add(ev, swr_mul(ea, s));
    const float v11 = swr_add(v01, swr_mul(ea, s));
    t00[j] = edge_test(ev, tie);
    t01[j] = edge_test(v01, tie);
    t10[j] = edge_test(v10, tie);
    t11[j] = edge_test(v11, tie);
  }
  const int inside = (t00[0] && t00[1] && t00[2]) + (t01[0] && t01[1] && t01[2]) +
                     (t10[0] && t10[1] && t10[2]) + (t11[0] && t11[1] && t11[2]);
  if (inside == 4) return 1;
  if (inside == 0) {
    const bool s00 = (t00[0] == t00[1]) == t00[2], s01 = (t01[0] == t01[1]) == t01[2];
    const bool s10 = (t10[0] == t10[1]) == t10[2], s11 = (t11[0] == t11[1]) == t11[2];
    if (s00 && s01 && s10 && s11) return 0;
  }
  return 2;
}

// Row `row` of drawBlock<true> (PixelShaderBase.h:64-93): the row start is the block
// corner's edge value stepped `row` times by b (eo.stepY), pixels step by a (ei.stepX).
// Returns the row's 8 coverage bits.
__device__ __forceinline__ uint32_t block_row_bits(const float* r, int flags, int bx, int by, int row) {
  const float fx = swr_add((float)bx, 0.5f), fy = swr_add((float)by, 0.5f);
  const bool tie0 = (flags >> 2) & 1, tie1 = (flags >> 3) & 1, tie2 = (flags >> 4) & 1;
  float i0 = fold7(swr_eval(r[6], r[7], r[8], fx, fy), r[7], row);
  float i1 = fold7(swr_eval(r[9], r[10], r[11], fx, fy), r[10], row);
  float i2 = fold7(swr_eval(r[12], r[13], r[14], fx, fy), r[13], row);
  uint32_t m = 0;
#pragma unroll
  for (int col = 0; col < SWR_BLOCK; ++col) {
    if (edge_test(i0, tie0) && edge_test(i1, tie1) && edge_test(i2, tie2)) m |= 1u << col;
    i0 = swr_add(i0, r[6]);
    i1 = swr_add(i1, r[9]);
    i2 = swr_add(i2, r[12]);
  }
  return m;
}

// Primitive id handed to the pixel shader: the index within its own draw.
__device__ __forceinline__ int prim_id(const RasterArgs& g, const float* rec, uint32_t p) {
  return (int)(p - (g.draw_prim_base ? g.draw_prim_base[__float_as_int(rec[1])] : 0u));
}

// Position (0-63) of the j-th set bit of m (j < popcount(m)).
__device__ __forceinline__ int nth_bit64(uint64_t m, int j) {
  int off = 0;
  uint32_t w = (uint32_t)m;
  int c = __popc(w);
  if (j >= c) { j -= c; w = (uint32_t)(m >> 32); off = 32; }
  c = __popc(w & 0xffffu); if (j >= c) { j -= c; w >>= 16; off += 16; }
  c = __popc(w & 0xffu);   if (j >= c) { j -= c; w >>= 8; off += 8; }
  c = __popc(w & 0xfu);    if (j >= c) { j -= c; w >>= 4; off += 4; }
  c = __popc(w & 0x3u);    if (j >= c) { j -= c; w >>= 2; off += 2; }
  if (j >= (int)(w & 1u)) off += 1;
  return off;
}

// Rebuilds the reference's incrementally stepped PixelData for pixel (x, y): the value
// at the evaluation point (block corner or span start) stepped kb times along y and ka
// times along x (PixelData::init/stepY/stepX, PixelData.h:61-125).
template <class PS>
__device__ __forceinline__ void build_pixel(const float* eq, bool blockmode, float fx, float fy, int ka, int kb,
                                            GpuPixel<PS>& pd) {
  typedef Rec<PS> RL;
  // Block pixels step kb rows then ka columns from the block corner; Span pixels ka columns
  // from their span start (kb == 0).  The mode is uniform per primitive (and per warp).
  auto stepped = [&](const float* q3) {
    const float e = swr_eval(q3[0], q3[1], q3[2], fx, fy);
    return blockmode ? fold7(fold7(e, q3[1], kb), q3[0], ka) : swr_fold(e, q3[0], ka);
  };
  if (RL::IW) {
    pd.invw = stepped(eq + 3 * RL::EQ_W);
    pd.w = swr_div(1.0f, pd.invw);
  }
#pragma unroll
  for (int i = 0; i < RL::NA; ++i) pd.avar[i] = stepped(eq + 3 * (RL::EQ_A + i));
#pragma unroll
  for (int i = 0; i < RL::NP; ++i) pd.pvar[i] = swr_mul(stepped(eq + 3 * (RL::EQ_P + i)), pd.w);
}

// Depth a depth-tested shader's State holds (the value its depth test compares against).
template <class State>
__device__ __forceinline__ float swr_state_depth(const State& s) {
  return s.depth;
}

// Conservative depth cull of one primitive in one tile.  A covered pixel's z is the z
// equation (a, b, c) evaluated ((a fx) + (b fy)) + c at the walk's start and then stepped k
// times by b or a (build_z).  With u = 2^-24 and every walk coordinate |x| <= X, 0 <= y <= Y,
// the exact plane values along the walk and the evaluation's terms are bounded by
// Q = |a| X + |b| Y + |c|; the evaluation errs by at most 3.0001 u Q (a three-term naive
// dot product) and each step adds at most u (Q + error so far), so for k u <= 1e-3 the
// stepped z is within u Q (3.01 + 1.001 k) + (k + 3) 2^-149 (underflow) of the exact plane
// value, which 2^-23 (k + 4) Q + 2^-126 bounds.  The exact plane minimum over the covered
// pixel centres [x0, x1] x [y0, y1] is bounded from below with downward-rounded arithmetic.
// Returns true when every covered pixel's z is >= dmax.
__device__ __forceinline__ bool z_not_below(float a, float b, float c, float x0, float x1, float y0, float y1,
                                            float X, float Y, int k, float dmax) {
  if (k > 16384) return false;
  const float q = __fadd_ru(__fadd_ru(__fmul_ru(fabsf(a), X), __fmul_ru(fabsf(b), Y)), fabsf(c));
  if (!(q <= 0x1p100f)) return false;  // no overflow anywhere on the walk (and no NaN)
  const float zlo = __fadd_rd(__fadd_rd(__fmul_rd(a, a >= 0.0f ? x0 : x1), __fmul_rd(b, b >= 0.0f ? y0 : y1)), c);
  const float margin = __fadd_ru(__fmul_ru(q, __fmul_ru((float)(k + 4), 0x1p-23f)), 0x1p-126f);
  return __fsub_rd(zlo, margin) >= dmax;
}

// A State written by another CTA of the same launch (after its fence): loaded through L2,
// never from a possibly stale L1 line.
template <class State>
__device__ __forceinline__ void swr_ld_state(State& d, const State* p) {
  static_assert(sizeof(State) % 4 == 0, "States are whole words");
  uint32_t* o = (uint32_t*)&d;
  const uint32_t* i = (const uint32_t*)p;
#pragma unroll
  for (int k = 0; k < (int)(sizeof(State) / 4); ++k) o[k] = __ldcg(i + k);
}

template <class PS>
__device__ __forceinline__ float build_z(const float* eq, bool blockmode, float fx, float fy, int ka, int kb) {
  typedef Rec<PS> RL;
  if (!RL::IZ) return 0.0f;
  const float* q3 = eq + 3 * RL::EQ_Z;
  const float e = swr_eval(q3[0], q3[1], q3[2], fx, fy);
  // Span pixels start from their own row (kb == 0); the mode is uniform per primitive
  return blockmode ? fold7(fold7(e, q3[1], kb), q3[0], ka) : swr_fold(e, q3[0], ka);
}

// One CTA per screen tile, 256 threads.  Per chunk of CH primitives of the tile's bin:
//   A. stage the setup records in shared memory;
//   B. exact coverage masks per (primitive, 8x8 block): one thread per pair classifies
//      Block-mode blocks (the reference's corner test) and builds Span-mode rows from
//      [xl, xr) (kept as each row's interpolation start); partially covered blocks are then
//      finished by 8 lanes each, one row per lane, with the reference's stepped edge tests;
//   C0. depth-tested shaders: per 8 x 4 pixel region, primitives whose z cannot pass any
//      depth test of the chunk there (z_not_below against the region's largest depth) are
//      only counted;
//   C1. small primitives (<= 64 covered pixels in the tile, up to FB fragments per chunk)
//      are compacted: one thread per covered fragment rebuilds the stepped interpolants and
//      evaluates the pixel shader's pure shade() at full SIMT width;
//   C2. each thread walks the chunk in primitive order for the pixels it owns and applies
//      every covering fragment to the pixel's register-resident State: compacted fragments
//      through apply(), others by rebuilding the interpolants in place (z first: a failing
//      depth test needs nothing else) and drawPixel().
// A heavy tile of a depth-min shader (RasterArgs.dslice) is run by up to SWR_DSLICES CTAs,
// each over its own run of whole chunks from the draw's starting State; the last run to
// finish merges the runs' States in bin order (swr_depth_merge) and stores.
template <class PS, int TILE, int CH, bool SPAN>
__global__ void __launch_bounds__(256, SWR_RASTER_MINB ? SWR_RASTER_MINB : SwrRasterOccupancy<PS>::value)
    k_raster(RasterArgs g) {
  swr_pdl_entry();
  typedef Rec<PS> RL;
  typedef typename PS::Color Color;
  constexpr int PPT = TILE * TILE / 256;  // pixels per thread
  constexpr int NBX = TILE / SWR_BLOCK;   // blocks per tile row
  constexpr int NB = NBX * NBX;
  constexpr bool kCompact = !SwrNoCompact<PS>::value;
  constexpr int FB = !kCompact ? 32 : (sizeof(Color) > 4 ? 512 : 1024);  // compacted fragments per chunk
  constexpr int SMALL = 64;
  __shared__ float4 srec4[CH * RL::R / 4];
  float* srec = (float*)srec4;
  __shared__ uint64_t smask[CH * NB];
  __shared__ int2 sspan[SPAN ? CH * TILE : 1];  // Span mode: each tile row's [xl, xr)
  __shared__ uint32_t sids[CH];
  __shared__ uint32_t sex[CH];   // compacted-fragment base (monotone over the chunk)
  __shared__ uint8_t scomp[CH];  // 1: compacted
  __shared__ float sfz[FB];
  __shared__ Color sfc[FB];
  __shared__ uint32_t sfr[32];
  __shared__ uint32_t snc;
  __shared__ uint32_t suncomp;  // some primitive of the chunk covers pixels and was not compacted
  __shared__ uint16_t spart[CH * NB];  // partially covered (primitive, block) pairs
  __shared__ uint32_t snpart;
  __shared__ uint32_t ssorted[SWR_RASTER_SORT];  // the tile's ordered bin (self-sorted tiles)
  __shared__ uint32_t scs[SWR_SEGS + 1];          // its cell starts relative to the bin start
  static_assert(sizeof(srec4) >= SWR_RASTER_SORT * 4, "raw bin staging fits the record area");
  constexpr bool kCull = SWR_DEPTH_CULL && SwrDepthCull<PS>::value;
  // Depth cull regions: the 8 x 4 pixels of one warp in one sub-tile (region q * 8 + warp).
  constexpr int NREG = 8 * PPT;
  __shared__ uint32_t swd[NREG];  // per region: order key of the largest depth it holds
  __shared__ uint32_t scull_on;   // some region holds no +inf depth (0: nothing can be culled)
  constexpr int NW = CH / 32;      // 32-primitive words of a chunk
  static_assert(CH % 32 == 0 && CH <= 128, "chunks of 32, 64, 96 or 128 primitives");
  __shared__ uint32_t sculr[kCull ? NREG * NW : 1];  // per region: primitives only counted there
  __shared__ int sminx[kCull && SPAN ? CH : 1];  // Span mode: leftmost start of a span reaching the tile
  // Per-pixel walk (shaders without the depth cull or overwrite shortcut): each pixel keeps
  // the set of compacted primitives covering it (set in C1), so in C2 every lane visits only
  // its own pixel's primitives instead of all primitives touching its warp's half block.
  constexpr int HW = (CH + 63) / 64;  // 64-primitive words of a chunk
  // (Not for the depth-culling shaders: measured on the 4K soup, whose chunks mix compacted
  // small primitives with large ones, the per-lane loops cost 30 % more raster time.)
  constexpr bool kPixWalk = SWR_PIX_WALK && kCompact && !kCull && !SwrOverwrite<PS>::value;
  __shared__ uint64_t spm[kPixWalk ? TILE * TILE * HW : 1];
  // per (primitive, block): the primitive's covered pixels in the tile's earlier blocks, so a
  // compacted fragment's slot is sex + spre + its rank in the block's mask (a compacted
  // primitive covers at most SMALL = 64 pixels of the tile: its prefixes fit a byte)
  __shared__ uint8_t spre[kCompact ? CH * NB : 1];
  __shared__ int32_t spid[CH];  // the primitives' ids as drawPixel sees them
  if (g.status[SWR_ST_FLAGS] & SWR_F_ANY_OVERFLOW) return;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  uint32_t frags = 0, passes = 0;
  // One CTA per tile (a persistent grid pulling tiles from a counter measured no faster on
  // the dense mesh and slower where few tiles carry the work: they gather on fewer SMs).
  // Overwrite shaders with g.slices > 1: CTA (tile, slice); a tile of more than
  // SWR_RASTER_SORT entries (an ordered bin) is cut into g.slices runs of whole chunks, each
  // rasterized from an empty State into slice_state and merged in order by k_merge_slices;
  // smaller tiles are rasterized whole by slice 0.
  uint32_t tile = blockIdx.x, slice = 0;
  if (SwrOverwrite<PS>::value && g.slices > 1) {
    tile = blockIdx.x / (uint32_t)g.slices;
    slice = blockIdx.x - tile * (uint32_t)g.slices;
  }
  int quad = -1;  // the 8 x 8 quadrant (block) this CTA rasterizes alone, -1: the whole tile
  int dslot = -1;  // sliced heavy tile: its list slot (slice = its run)
  if constexpr (SwrDepthMin<PS>::value) {
    if (g.dslice) {
      const uint32_t nq = SWR_DSLICES * g.quad_cap;
      if (blockIdx.x < nq) {
        const uint32_t slot = blockIdx.x / SWR_DSLICES;
        if (slot >= min(*g.quad_count, g.quad_cap)) return;
        tile = g.quad_tiles[slot];
        slice = blockIdx.x - slot * SWR_DSLICES;
        dslot = (int)slot;
      } else {
        tile = blockIdx.x - nq;
        if (tile < g.ntiles && g.quad_flag[tile]) return;  // rasterized in slices
      }
    }
  }
  if constexpr (TILE == 16 && !SwrOverwrite<PS>::value) {
    if (g.dslice) {
    } else if (g.quad_all) {
      tile = blockIdx.x >> 2;
      quad = (int)(blockIdx.x & 3u);
    } else if (g.quad_flag) {
      const uint32_t nq = 4u * g.quad_cap;
      if (blockIdx.x < nq) {
        const uint32_t slot = blockIdx.x >> 2;
        if (slot >= min(*g.quad_count, g.quad_cap)) return;
        tile = g.quad_tiles[slot];
        quad = (int)(blockIdx.x & 3u);
      } else {
        tile = blockIdx.x - nq;
        if (tile < g.ntiles && g.quad_flag[tile]) return;  // rasterized by its quadrant CTAs
      }
    }
  }
  if (tile >= g.ntiles) return;
  uint32_t b = g.tile_start[(size_t)tile * g.tile_stride], e = g.tile_start[(size_t)(tile + 1) * g.tile_stride];
  bool sliced = false;
  if constexpr (SwrOverwrite<PS>::value) {
    if (g.slices > 1) {
      if (e - b <= (uint32_t)SWR_RASTER_SORT) {
        if (slice) return;
      } else {
        sliced = true;
        const uint32_t nch = (e - b + CH - 1) / CH, ns = (uint32_t)g.slices;
        const uint32_t lo = b + (uint32_t)((uint64_t)nch * slice / ns) * CH;
        const uint32_t hi = min(e, b + (uint32_t)((uint64_t)nch * (slice + 1) / ns) * CH);
        b = lo;
        e = hi > lo ? hi : lo;  // an empty slice still writes its (empty) states
      }
    }
  }
  if (b == e && !sliced) return;  // uniform per CTA
  // the chunks this CTA rasterizes: the whole bin, or a sliced heavy tile's run
  uint32_t cb = b, ce = e;
  int nsl = 1;
  if (dslot >= 0) {
    const uint32_t nch = (e - b + CH - 1) / CH;
    nsl = (int)min(nch, (uint32_t)SWR_DSLICES);
    if ((int)slice >= nsl) return;  // (uniform per tile: these CTAs take no part)
    cb = b + (uint32_t)((uint64_t)nch * slice / (uint32_t)nsl) * CH;
    ce = min(e, b + (uint32_t)((uint64_t)nch * (slice + 1) / (uint32_t)nsl) * CH);
  }
  const int ti = g.ntargets > 1 ? swr_find_le(g.target_tile_base, g.ntargets, tile) : 0;
  const SwrTargetDesc& T = g.targets[ti];
  const SwrUniforms& U = g.draws[T.first_draw].u;
  const uint32_t lt = tile - T.tile_base;
  const int ox = (int)(lt % (uint32_t)T.tiles_x) * TILE, oy = (int)(lt / (uint32_t)T.tiles_x) * TILE;
  // Thread -> pixels: each warp covers an 8 x 4 half block; 16 x 16 sub-tiles repeat.
  int px[PPT], py[PPT], blk[PPT];
  bool in[PPT];
  typename PS::State st[PPT];
#pragma unroll
  for (int q = 0; q < PPT; ++q) {
    const int sxo = (q % (TILE / 16)) * 16, syo = (q / (TILE / 16)) * 16;
    const int hb = warp >> 1;
    const int lx = sxo + (hb & 1) * 8 + (lane & 7);
    const int ly = syo + (hb >> 1) * 8 + (warp & 1) * 4 + (lane >> 3);
    px[q] = ox + lx;
    py[q] = oy + ly;
    blk[q] = (ly >> 3) * NBX + (lx >> 3);
    in[q] = px[q] < T.width && py[q] < T.height && (quad < 0 || blk[q] == quad);
    if (in[q]) PS::load(st[q], px[q], py[q], U);
  }
  // A tile of at most SWR_RASTER_SORT entries orders its own bin: the cells (increasing id
  // segments) are contiguous, so an id's position is its cell's start plus the number of
  // smaller ids in that cell.  The raw ids are staged in the record area (used only later).
  const bool self_sort = g.bin_raw && !sliced && e - b <= (uint32_t)SWR_RASTER_SORT;
  if (self_sort) {
    uint32_t* sraw = (uint32_t*)srec4;
    const uint32_t ntot = e - b;
    if (threadIdx.x <= SWR_SEGS) scs[threadIdx.x] = g.tile_start[(size_t)tile * SWR_SEGS + threadIdx.x] - b;
    for (uint32_t j = threadIdx.x; j < ntot; j += 256) sraw[j] = g.bin_raw[b + j];
    __syncthreads();
    for (uint32_t j = threadIdx.x; j < ntot; j += 256) {
      int lo = 0, hi = SWR_SEGS - 1;  // the cell holding j: last c with scs[c] <= j
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (scs[mid] <= j) lo = mid; else hi = mid - 1;
      }
      const uint32_t v = sraw[j], c_end = scs[lo + 1];
      uint32_t pos = scs[lo];
      for (uint32_t k = scs[lo]; k < c_end; ++k) pos += sraw[k] < v;
      ssorted[pos < ntot ? pos : 0] = v;
    }
  }
  for (uint32_t c0 = cb; c0 < ce; c0 += CH) {
    const int n = (int)min((uint32_t)CH, ce - c0);
    __syncthreads();  // the previous chunk's shared state is no longer read; ssorted is complete
    if (threadIdx.x < n) sids[threadIdx.x] = self_sort ? ssorted[c0 - b + threadIdx.x] : g.bin[c0 + threadIdx.x];
    if (threadIdx.x == 0) snpart = 0;
    if constexpr (kPixWalk) {
#pragma unroll
      for (int q = 0; q < PPT; ++q)
#pragma unroll
        for (int w = 0; w < HW; ++w) spm[((py[q] - oy) * TILE + (px[q] - ox)) * HW + w] = 0ull;
    }
    if (kCull && SPAN && threadIdx.x < CH) sminx[threadIdx.x] = 0x7fffffff;
    // Region depth bounds at the chunk's start (depth-tested shaders, tiles of more than one
    // chunk): per region an order-preserving key of the largest depth its pixels hold (NaN
    // depths, which every fragment fails, and pixels outside the target are ignored; key 0:
    // none usable).  A region holding +inf can cull nothing (z is finite); the barrier's OR
    // tells whether any region can.
    int any_ok = 0;
    bool cull_tile = false;
    bool my_ok = false;
    if constexpr (kCull) {
      cull_tile = ce - cb > (uint32_t)CH;
      if (cull_tile) {
#pragma unroll
        for (int q = 0; q < PPT; ++q) {
          const float dq = swr_state_depth(st[q]);
          const uint32_t u = __float_as_uint(dq);
          const uint32_t kq = (u & 0x80000000u) ? ~u : (u | 0x80000000u);
          const uint32_t key = __reduce_max_sync(0xffffffffu, in[q] && !swr_isnan(dq) ? kq : 0u);
          if (lane == 0) swd[q * 8 + warp] = key;
          my_ok |= key != 0u && key < 0xff800000u;  // uniform per warp
        }
      }
    }
    // A: the chunk's setup records (ids read from the bin directly: sids is published by
    // the barrier below)
    {
      constexpr int R4 = RL::R / 4;
      const float4* recs4 = (const float4*)g.recs;
#pragma unroll 4
      for (int i = threadIdx.x; i < n * R4; i += 256) {
        const int k = i / R4, w = i - k * R4;
        const uint32_t id = self_sort ? ssorted[c0 - b + k] : __ldg(g.bin + c0 + k);
        srec4[i] = recs4[(size_t)id * R4 + w];
      }
    }
    if (cull_tile)
      any_ok = __syncthreads_or(my_ok);
    else
      __syncthreads();
    // B1: coverage per (primitive, block).  Fully covered / skipped blocks and Span rows are
    // finished here; partially covered Block-mode blocks are queued for B2.
    if (kCull && threadIdx.x == 0) scull_on = any_ok;
    for (int i = threadIdx.x; i < n * NB; i += 256) {
      const int k = i / NB, j = i - k * NB;
      const float* r = srec + k * RL::R;
      const int flags = __float_as_int(r[0]);
      if (SPAN && (flags & 3) == 1) continue;  // Span mode: rows below, masks after the barrier
      if (quad >= 0 && j != quad) {  // another CTA's quadrant
        smask[i] = 0;
        continue;
      }
      const int bx = ox + (j % NBX) * SWR_BLOCK, by = oy + (j / NBX) * SWR_BLOCK;
      uint64_t m = 0;
      const bool hit = (flags & 1) && bx <= __float_as_int(r[4]) && bx + SWR_BLOCK - 1 >= __float_as_int(r[2]) &&
                       by <= __float_as_int(r[5]) && by + SWR_BLOCK - 1 >= __float_as_int(r[3]);
      if (hit) {  // Block mode (every valid primitive of a k_raster<..., false> launch)
        const int cls = block_class(r, flags, bx, by);
        if (cls == 1) m = ~0ull;
        if (cls == 2) spart[atomicAdd(&snpart, 1u)] = (uint16_t)i;
      }
      smask[i] = m;
    }
    if constexpr (SPAN) {
      // B1 (Span mode): each tile row's span [xl, xr) of every primitive, once per row (kept
      // as the row's interpolation start); the rows of one primitive are consecutive lanes,
      // and whole warps iterate (the row reduction below shuffles across the warp)
      for (int i = threadIdx.x; i < (n * TILE + 31) / 32 * 32; i += 256) {
        const int k = i / TILE, row = i - k * TILE;
        const float* r = srec + k * RL::R;
        const int flags = k < n ? __float_as_int(r[0]) : 0;
        int2 sp = make_int2(1, 0);
        const int y = oy + row;
        if ((flags & 3) == 1 && y >= __float_as_int(r[3]) && y <= __float_as_int(r[5])) {
          SpanHalf h;
          bool any = true;
          if ((flags & 32) && y >= __float_as_int(r[6]) && y < __float_as_int(r[7])) {
            h.ox = r[8]; h.oy = r[9]; h.is1 = r[10]; h.is2 = r[11];
          } else if ((flags & 64) && y > __float_as_int(r[13]) && y <= __float_as_int(r[12])) {
            h.ox = r[14]; h.oy = r[15]; h.is1 = r[16]; h.is2 = r[17];
          } else {
            any = false;
          }
          if (any) {
            const SwrDrawDesc& D = g.draws[__float_as_int(r[1])];
            span_row(h, y, D.sc_minx, D.sc_maxx, sp.x, sp.y);
          }
        }
        if ((flags & 3) == 1) sspan[k * TILE + row] = sp;
        if (kCull) {
          // leftmost start of a span reaching the tile, over the primitive's TILE rows
          int lmin = (sp.x < sp.y && sp.y > ox) ? sp.x : 0x7fffffff;
#pragma unroll
          for (int o = TILE / 2; o; o >>= 1) lmin = min(lmin, __shfl_xor_sync(0xffffffffu, lmin, o));
          if (row == 0 && lmin != 0x7fffffff) atomicMin(&sminx[k], lmin);
        }
      }
      __syncthreads();
      // B1 (Span mode) masks from the spans: each row's [xl, xr) clipped to the block
      for (int i = threadIdx.x; i < n * NB; i += 256) {
        const int k = i / NB, j = i - k * NB;
        const float* r = srec + k * RL::R;
        const int flags = __float_as_int(r[0]);
        if ((flags & 3) != 1) continue;
        if (quad >= 0 && j != quad) {
          smask[i] = 0;
          continue;
        }
        const int bx = ox + (j % NBX) * SWR_BLOCK, by = oy + (j / NBX) * SWR_BLOCK;
        const bool hit = bx <= __float_as_int(r[4]) && bx + SWR_BLOCK - 1 >= __float_as_int(r[2]) &&
                         by <= __float_as_int(r[5]) && by + SWR_BLOCK - 1 >= __float_as_int(r[3]);
        uint64_t m = 0;
        if (hit) {
#pragma unroll
          for (int rr = 0; rr < SWR_BLOCK; ++rr) {
            const int2 sp = sspan[k * TILE + (by - oy) + rr];
            const int c0b = max(sp.x, bx) - bx, c1b = min(sp.y, bx + SWR_BLOCK) - bx;
            if (c1b > c0b) m |= (((1ull << (c1b - c0b)) - 1ull) << c0b) << (rr * 8);
          }
        }
        smask[i] = m;
      }
    } else {
      __syncthreads();
    }
    // B2: partially covered blocks, one row per lane (8 lanes per block); each lane stores
    // its row's byte of the block's mask (bit row * 8 + col of the little-endian word)
    {
      const int np8 = (int)snpart * SWR_BLOCK;
      for (int t = threadIdx.x; t < np8; t += 256) {
        const int i = spart[t >> 3];
        const int row = t & 7;
        const int k = i / NB, j = i - k * NB;
        const float* r = srec + k * RL::R;
        ((uint8_t*)&smask[i])[row] = (uint8_t)block_row_bits(r, __float_as_int(r[0]), ox + (j % NBX) * SWR_BLOCK,
                                                             oy + (j / NBX) * SWR_BLOCK, row);
      }
    }
    __syncthreads();
    // C0 (depth-tested shaders): per (region, primitive) whether every covered pixel's z is
    // provably not below the region's largest depth at the chunk's start (z_not_below over
    // the covered pixels' box in the region).  Depths only decrease, so such fragments fail
    // their depth tests: the primitive is only counted there.
    if (kCull && scull_on) {
      for (int t = threadIdx.x; t < NREG * CH; t += 256) {
        const int reg = t / CH, k = t - reg * CH;  // reg uniform per warp (CH is a multiple of 32)
        bool culled = false;
        if (k < n && (__float_as_int(srec[k * RL::R]) & 1)) {
          const int q = reg >> 3, w = reg & 7, hb = w >> 1;
          const int lx0 = (q % (TILE / 16)) * 16 + (hb & 1) * 8;
          const int ly0 = (q / (TILE / 16)) * 16 + (hb >> 1) * 8 + (w & 1) * 4;
          const uint32_t mh = (uint32_t)(smask[k * NB + (ly0 >> 3) * NBX + (lx0 >> 3)] >> ((w & 1) * 32));
          const uint32_t key = swd[reg];
          if (mh && key != 0u && key < 0xff800000u) {
            const float dmax = __uint_as_float((key & 0x80000000u) ? (key & 0x7fffffffu) : ~key);
            uint32_t c = mh | (mh >> 16);
            c |= c >> 8;
            c &= 0xffu;
            const int x0 = ox + lx0 + __ffs(c) - 1, x1 = ox + lx0 + 31 - __clz(c);
            const int y0 = oy + ly0 + ((__ffs(mh) - 1) >> 3), y1 = oy + ly0 + ((31 - __clz(mh)) >> 3);
            const float* r = srec + k * RL::R;
            // walk bounds: Block mode steps <= 7 rows then <= 7 columns inside the block;
            // Span mode steps from the row's span start (every covered pixel lies in a row
            // whose span reaches the tile) to the pixel
            int steps = 2 * (SWR_BLOCK - 1);
            float X = (float)x1 + 0.5f;
            if (SPAN && !(__float_as_int(r[0]) & 2)) {
              const int smin = sminx[k];
              steps = max(0, x1 - smin);
              if (smin < 0) X = fmaxf(X, (float)(-smin) + 0.5f);
            }
            const float* zq = r + RL::EQ0 + 3 * RL::EQ_Z;
            const float fy1 = (float)y1 + 0.5f;
            culled = z_not_below(zq[0], zq[1], zq[2], (float)x0 + 0.5f, (float)x1 + 0.5f, (float)y0 + 0.5f, fy1, X,
                                 fy1, steps, dmax);
          }
        }
        const uint32_t bal = __ballot_sync(0xffffffffu, culled);
        if (lane == 0) sculr[reg * NW + (k >> 5)] = bal;
      }
      __syncthreads();
    }
    // C1 set-up (one thread per primitive in warps 0..NW-1, warp 0 scans): compact the small
    // primitives' fragments (a prefix of the chunk's small primitives whose fragments fit in
    // FB), leaving out primitives culled in every region they cover.
    if (warp < NW) {
      const bool try_cull = kCull && scull_on;
      // cnt: the primitive's covered pixels in the tile; culled: culled in every region it
      // covers (its fragments are then left out of the compaction)
      auto prim_info = [&](int k, uint32_t& cnt, bool& culled) {
        cnt = 0;
        culled = false;
        if (k >= n) return;
        const float* r = srec + k * RL::R;
        spid[k] = prim_id(g, r, sids[k]);
        if (!(__float_as_int(r[0]) & 1)) return;
        for (int j = 0; j < NB; ++j) {
          const uint64_t m = smask[k * NB + j];
          if (kCompact) spre[k * NB + j] = (uint8_t)min(cnt, 255u);
          cnt += __popc((uint32_t)m) + __popc((uint32_t)(m >> 32));
        }
        if (kCull && try_cull && cnt) {
          bool all = true;
          for (int reg = 0; reg < NREG; ++reg) {
            const int q = reg >> 3, w = reg & 7, hb = w >> 1;
            const int lx0 = (q % (TILE / 16)) * 16 + (hb & 1) * 8;
            const int ly0 = (q / (TILE / 16)) * 16 + (hb >> 1) * 8 + (w & 1) * 4;
            const uint32_t mh = (uint32_t)(smask[k * NB + (ly0 >> 3) * NBX + (lx0 >> 3)] >> ((w & 1) * 32));
            if (mh && !((sculr[reg * NW + (k >> 5)] >> (k & 31)) & 1u)) all = false;
          }
          culled = all;
        }
      };
      // warps 0..NW-1 measure primitives warp * 32 + lane; warp 0 scans all of them
      uint32_t cnt0;
      bool cul0;
      prim_info(threadIdx.x, cnt0, cul0);
      if (warp > 0) {  // hand the primitive to warp 0 through sex / scomp
        sex[threadIdx.x] = cnt0;
        scomp[threadIdx.x] = cul0;
      }
      if (NW > 1) asm volatile("bar.sync 1, %0;" ::"r"(CH) : "memory");  // warps 0..NW-1 only
      if (warp == 0) {
        // Behind depths already written (a cull tile past its first chunk) most fragments fail
        // their depth test: shading them ahead of the test (compaction) would be wasted, the
        // in-place path tests z first.
        const bool deep = kCull && scull_on;
        uint32_t cnt[NW], cand[NW], inc[NW];
        bool cul[NW];
#pragma unroll
        for (int w = 0; w < NW; ++w) {
          cnt[w] = w ? sex[w * 32 + lane] : cnt0;
          cul[w] = w ? scomp[w * 32 + lane] != 0 : cul0;
          cand[w] = kCompact && cnt[w] <= SMALL && !cul[w] && !deep ? cnt[w] : 0u;
          inc[w] = cand[w];
        }
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {  // inclusive scans over lanes
#pragma unroll
          for (int w = 0; w < NW; ++w) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, inc[w], o);
            if (lane >= o) inc[w] += y;
          }
        }
        uint32_t carry = 0, hi = 0;
        bool unc = false;
#pragma unroll
        for (int w = 0; w < NW; ++w) {
          const uint32_t ex = carry + inc[w] - cand[w];
          carry += __shfl_sync(0xffffffffu, inc[w], 31);
          const bool comp = kCompact && !cul[w] && !deep && cnt[w] <= SMALL && ex + cnt[w] <= FB;
          if (w * 32 + lane < n) {
            sex[w * 32 + lane] = ex;
            scomp[w * 32 + lane] = comp ? 1 : 0;
          }
          if (comp && cnt[w]) hi = max(hi, ex + cnt[w]);
          unc |= !comp && cnt[w] != 0u;
        }
        const uint32_t nc_max = __reduce_max_sync(0xffffffffu, hi);
        const bool any_unc = __any_sync(0xffffffffu, unc);
        if (lane == 0) {
          snc = nc_max;
          suncomp = any_unc ? 1u : 0u;
        }
      }
    }
    __syncthreads();
    // C1: interpolate and shade the compacted fragments
    const int nc = (int)snc;
    for (int f = threadIdx.x; f < nc; f += 256) {
      int lo = 0, hi = n - 1;
      while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if ((int)sex[mid] <= f) lo = mid; else hi = mid - 1;
      }
      const int k = lo;
      int jj = f - (int)sex[k];
      const uint64_t* mk = smask + k * NB;
      int blkj = 0;
      for (; blkj < NB - 1; ++blkj) {
        const int c = __popcll(mk[blkj]);
        if (jj < c) break;
        jj -= c;
      }
      const int bit = nth_bit64(mk[blkj], jj);
      const int x = ox + (blkj % NBX) * SWR_BLOCK + (bit & 7);
      const int y = oy + (blkj / NBX) * SWR_BLOCK + (bit >> 3);
      const float* r = srec + k * RL::R;
      const bool blockmode = !SPAN || (__float_as_int(r[0]) & 2);
      float fx, fy;
      int ka, kb;
      if (blockmode) {
        fx = swr_add((float)(x & ~7), 0.5f);
        fy = swr_add((float)(y & ~7), 0.5f);
        ka = x & 7;
        kb = y & 7;
      } else {
        const int2 sp = sspan[k * TILE + (y - oy)];
        fx = swr_add((float)sp.x, 0.5f);
        fy = swr_add((float)y, 0.5f);
        ka = x - sp.x;
        kb = 0;
      }
      const float* eq = r + RL::EQ0;
      GpuPixel<PS> pd;
      pd.x = x;
      pd.y = y;
      pd.eq = eq;
      pd.z = build_z<PS>(eq, blockmode, fx, fy, ka, kb);
      build_pixel<PS>(eq, blockmode, fx, fy, ka, kb, pd);
      sfz[f] = pd.z;
      sfc[f] = PS::shade(pd, g.draws[__float_as_int(r[1])].u);
      if constexpr (kPixWalk)
        atomicOr((unsigned long long*)&spm[((y - oy) * TILE + (x - ox)) * HW + (k >> 6)], 1ull << (k & 63));
    }
    __syncthreads();
    // C2: fragments in primitive order.  Each warp owns one 8 x 4 half block per sub-tile
    // q; a ballot over the chunk gives the primitives whose masks touch it, visited in
    // increasing order (per-pixel order = primitive order).
#pragma unroll
    for (int q = 0; q < PPT; ++q) {
      const int half = (py[q] >> 2) & 1;
      if constexpr (kPixWalk) {
        // the warp's primitives that were not compacted and touch its half block (ballot),
        // plus this pixel's compacted primitives; visited per lane in increasing order
        uint64_t todo[HW];
#pragma unroll
        for (int w = 0; w < HW; ++w) todo[w] = 0;
        if (suncomp) {  // (uniform; a chunk of compacted primitives only has nothing to ballot)
#pragma unroll
          for (int w = 0; w < NW; ++w) {
            const int k = w * 32 + lane;
            const bool h = k < n && !scomp[k] && ((uint32_t)(smask[k * NB + blk[q]] >> (half * 32)) != 0u);
            todo[w >> 1] |= (uint64_t)__ballot_sync(0xffffffffu, h) << ((w & 1) * 32);
          }
        }
        const int bit = (py[q] & 7) * 8 + (px[q] & 7);
        if (!in[q]) continue;
        const int pix = (py[q] - oy) * TILE + (px[q] - ox);
#pragma unroll
        for (int w = 0; w < HW; ++w) {
          uint64_t t = todo[w] | spm[pix * HW + w];
          while (t) {
            const int k = w * 64 + __ffsll((long long)t) - 1;
            t &= t - 1ull;
            const uint64_t* mk = smask + k * NB;
            const uint64_t m = mk[blk[q]];
            if (!((m >> bit) & 1ull)) continue;
            const float* r = srec + k * RL::R;
            frags++;
            if (scomp[k]) {
              const int f = (int)sex[k] + (int)spre[k * NB + blk[q]] + __popcll(m & ((1ull << bit) - 1ull));
              PS::apply(st[q], sfz[f], sfc[f], spid[k]);
              continue;
            }
            const bool blockmode = !SPAN || (__float_as_int(r[0]) & 2);
            float fx, fy;
            int ka, kb;
            if (blockmode) {
              fx = swr_add((float)(px[q] & ~7), 0.5f);
              fy = swr_add((float)(py[q] & ~7), 0.5f);
              ka = px[q] & 7;
              kb = py[q] & 7;
            } else {
              const int2 sp = sspan[k * TILE + (py[q] - oy)];
              fx = swr_add((float)sp.x, 0.5f);
              fy = swr_add((float)py[q], 0.5f);
              ka = px[q] - sp.x;
              kb = 0;
            }
            const float* eq = r + RL::EQ0;
            GpuPixel<PS> pd;
            pd.x = px[q];
            pd.y = py[q];
            pd.eq = eq;
            pd.z = build_z<PS>(eq, blockmode, fx, fy, ka, kb);
            if (RL::IZ && PS::earlyReject(pd.z, st[q])) continue;
            build_pixel<PS>(eq, blockmode, fx, fy, ka, kb, pd);
            PS::drawPixel(pd, spid[k], st[q], g.draws[__float_as_int(r[1])].u);
          }
        }
        continue;
      }
      uint64_t hw[HW];
#pragma unroll
      for (int w = 0; w < HW; ++w) hw[w] = 0;
#pragma unroll
      for (int w = 0; w < NW; ++w) {
        const int k = w * 32 + lane;
        const bool h = k < n && ((uint32_t)(smask[k * NB + blk[q]] >> (half * 32)) != 0u);
        hw[w >> 1] |= (uint64_t)__ballot_sync(0xffffffffu, h) << ((w & 1) * 32);
      }
      const int bit = (py[q] & 7) * 8 + (px[q] & 7);
      if (kCull && scull_on) {
        // primitives culled in this warp's region: their fragments fail the depth test and
        // are only counted, in any order (counters commute), outside the primitive-order walk
        const uint32_t* cr = sculr + (q * 8 + warp) * NW;
#pragma unroll
        for (int w = 0; w < HW; ++w) {
          const uint64_t cm = (uint64_t)cr[2 * w] | (2 * w + 1 < NW ? (uint64_t)cr[2 * w + 1] << 32 : 0ull);
          uint64_t ch = hw[w] & cm;
          hw[w] &= ~ch;
          while (ch) {
            const int k = w * 64 + __ffsll((long long)ch) - 1;
            ch &= ch - 1ull;
            if (in[q] && ((smask[k * NB + blk[q]] >> bit) & 1ull)) {
              frags++;
              PS::earlyReject(__int_as_float(0x7f800000), st[q]);  // counts the rejected fragment
            }
          }
        }
      }
      uint32_t extra = 0;  // overwrite shaders: covering fragments before the last one
      if (SwrOverwrite<PS>::value) {
        // only the chunk's last covering primitive shades; the others only count
        int last = -1;
        uint32_t cnt = 0;
#pragma unroll
        for (int w = 0; w < HW; ++w) {
          uint64_t h = hw[w];
          while (h) {
            const int k = w * 64 + __ffsll((long long)h) - 1;
            h &= h - 1ull;
            if (in[q] && ((smask[k * NB + blk[q]] >> bit) & 1ull)) {
              ++cnt;
              last = k;
            }
          }
        }
        if (cnt) {
#pragma unroll
          for (int w = 0; w < HW; ++w) hw[w] = (last >> 6) == w ? 1ull << (last & 63) : 0ull;
          extra = cnt - 1;
          frags += extra;
          st[q].frags += extra;
          st[q].writes += extra;
        }
      }
      // primitive-order walk over the words (one copy of the loop body)
      uint64_t hits = hw[0];
      uint64_t later = HW > 1 ? hw[HW - 1] : 0ull;
      int kbase = 0;
      while (true) {
        if (!hits) {
          if (HW == 1 || !later) break;
          hits = later;
          later = 0;
          kbase = 64;
        }
        const int k = kbase + __ffsll((long long)hits) - 1;
        hits &= hits - 1ull;
        const uint64_t* mk = smask + k * NB;
        const uint64_t m = mk[blk[q]];
        if (!in[q] || !((m >> bit) & 1ull)) continue;
        const float* r = srec + k * RL::R;
        frags++;
        if (scomp[k]) {
          const int f = (int)sex[k] + (int)spre[k * NB + blk[q]] + __popcll(m & ((1ull << bit) - 1ull));
          PS::apply(st[q], sfz[f], sfc[f], spid[k]);
          continue;
        }
        const bool blockmode = !SPAN || (__float_as_int(r[0]) & 2);
        float fx, fy;
        int ka, kb;
        if (blockmode) {
          fx = swr_add((float)(px[q] & ~7), 0.5f);
          fy = swr_add((float)(py[q] & ~7), 0.5f);
          ka = px[q] & 7;
          kb = py[q] & 7;
        } else {
          const int2 sp = sspan[k * TILE + (py[q] - oy)];
          fx = swr_add((float)sp.x, 0.5f);
          fy = swr_add((float)py[q], 0.5f);
          ka = px[q] - sp.x;
          kb = 0;
        }
        const float* eq = r + RL::EQ0;
        GpuPixel<PS> pd;
        pd.x = px[q];
        pd.y = py[q];
        pd.eq = eq;
        pd.z = build_z<PS>(eq, blockmode, fx, fy, ka, kb);
        if (RL::IZ && PS::earlyReject(pd.z, st[q])) continue;
        build_pixel<PS>(eq, blockmode, fx, fy, ka, kb, pd);
        PS::drawPixel(pd, spid[k], st[q], g.draws[__float_as_int(r[1])].u);
      }
    }
  }
  if constexpr (SwrDepthMin<PS>::value) {
    if (dslot >= 0) {
      // this run's States, then the last run to finish merges the tile's runs in bin order
      // (each thread owns the same pixels in every run's CTA)
      typename PS::State* ss = (typename PS::State*)g.dslice_state + (size_t)dslot * SWR_DSLICES * (TILE * TILE);
#pragma unroll
      for (int q = 0; q < PPT; ++q)
        if (in[q]) {
          ss[(size_t)slice * (TILE * TILE) + (py[q] - oy) * TILE + (px[q] - ox)] = st[q];
          passes += st[q].writes;
        }
      __threadfence();
      __syncthreads();
      if (threadIdx.x == 0) snc = atomicAdd(&g.dslice_done[dslot], 1u) == (uint32_t)(nsl - 1);
      __syncthreads();
      if (snc) {
        __threadfence();
#pragma unroll
        for (int q = 0; q < PPT; ++q)
          if (in[q]) {
            const int pi = (py[q] - oy) * TILE + (px[q] - ox);
            typename PS::State m;
            swr_ld_state(m, ss + pi);
            for (int sl = 1; sl < nsl; ++sl) {
              typename PS::State o;
              swr_ld_state(o, ss + (size_t)sl * (TILE * TILE) + pi);
              swr_depth_merge(m, o);
            }
            PS::store(m, px[q], py[q], U);
          }
        if (threadIdx.x == 0) g.dslice_done[dslot] = 0u;  // ready for the next draw
      }
      uint32_t tot, ptot;
      swr_block_exscan(frags, sfr, &tot);
      swr_block_exscan(passes, sfr, &ptot);
      if (threadIdx.x == 0 && tot) {
        atomicAdd((unsigned long long*)&g.status_w[SWR_ST_SHADED_LO], (unsigned long long)tot);
        atomicAdd((unsigned long long*)&g.status_w[SWR_ST_PASSES_LO], (unsigned long long)ptot);
      }
      return;
    }
  }
#pragma unroll
  for (int q = 0; q < PPT; ++q)
    if (in[q]) {
      if (sliced) {
        typename PS::State* ss = (typename PS::State*)g.slice_state +
                                 ((size_t)tile * g.slices + slice) * (TILE * TILE);
        ss[(py[q] - oy) * TILE + (px[q] - ox)] = st[q];
      } else {
        PS::store(st[q], px[q], py[q], U);
      }
      passes += st[q].writes;
    }
  // fragment statistics: drawPixel calls and colour writes
  uint32_t tot, ptot;
  swr_block_exscan(frags, sfr, &tot);
  swr_block_exscan(passes, sfr, &ptot);
  if (threadIdx.x == 0 && tot) {
    atomicAdd((unsigned long long*)&g.status_w[SWR_ST_SHADED_LO], (unsigned long long)tot);
    atomicAdd((unsigned long long*)&g.status_w[SWR_ST_PASSES_LO], (unsigned long long)ptot);
  }
}

// Merges the slices of the tiles k_raster sliced (more than SWR_RASTER_SORT entries):
// per pixel the slices' States in bin order (swr_overwrite_merge), then the shader's store.
template <class PS, int TILE>
__global__ void __launch_bounds__(256) k_merge_slices(RasterArgs g) {
  swr_pdl_entry();
  constexpr int PPT = TILE * TILE / 256;
  if (g.status[SWR_ST_FLAGS] & SWR_F_ANY_OVERFLOW) return;
  const uint32_t tile = blockIdx.x;
  if (tile >= g.ntiles) return;
  const uint32_t b = g.tile_start[(size_t)tile * g.tile_stride], e = g.tile_start[(size_t)(tile + 1) * g.tile_stride];
  if (e - b <= (uint32_t)SWR_RASTER_SORT) return;
  const int ti = g.ntargets > 1 ? swr_find_le(g.target_tile_base, g.ntargets, tile) : 0;
  const SwrTargetDesc& T = g.targets[ti];
  const SwrUniforms& U = g.draws[T.first_draw].u;
  const uint32_t lt = tile - T.tile_base;
  const int ox = (int)(lt % (uint32_t)T.tiles_x) * TILE, oy = (int)(lt / (uint32_t)T.tiles_x) * TILE;
  const typename PS::State* ss = (const typename PS::State*)g.slice_state + (size_t)tile * g.slices * (TILE * TILE);
#pragma unroll
  for (int q = 0; q < PPT; ++q) {
    const int i = q * 256 + threadIdx.x;
    const int x = ox + i % TILE, y = oy + i / TILE;
    if (x >= T.width || y >= T.height) continue;
    typename PS::State m;
    PS::load(m, x, y, U);
    for (int sl = 0; sl < g.slices; ++sl) swr_overwrite_merge(m, ss[(size_t)sl * (TILE * TILE) + i]);
    PS::store(m, x, y, U);
  }
}

}  // namespace swr
