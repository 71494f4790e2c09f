// Points and lines: VertexProcessor::clipPoints / clipLines (VertexProcessor.cpp:152-215,
// LineClipper.cpp:30-56) and Rasterizer::drawPointTemplate / drawLineTemplate
// (Rasterizer.h:150-222).
//
//   k_assemble_lp_count / _emit  one CTA per batch: outcodes, parametric line clipping
//                                (endpoints replaced by lerps at t0 / t1), point rejection;
//                                survivors keep submission order
//   k_lp_setup                   per primitive: DDA step count and per-step increments
//   k_lp_frags                   one thread per DDA step: the stepped vertex by exact fold,
//                                the per-step scissor test, the pixel key
//   (stable radix sort of fragments by pixel keeps primitive order, then step order,
//    including a pixel hit twice by one line)
//   k_lp_shade                   one thread per covered pixel applies its fragments in order
#pragma once
#include "swr_stages.cuh"

namespace swr {

// Line / point record for pixel shader PS: steps, draw id, start vertex, per-step increment;
// each vertex is x, y, z, w, avar[NA], pvar[NP].
template <class PS>
struct LpRec {
  enum { NA = PS::AVarCount, NP = PS::PVarCount, NV = 4 + NA + NP, R = 2 + 2 * NV };
};

template <int A, int P>
__device__ uint32_t assemble_lp_one(const AssembleArgs& g, const SwrDrawDesc& D, uint32_t p) {
  typedef VLayout<A, P> L;
  const uint32_t gp = D.pbase + p;
  const int per = D.draw_mode == 0 ? 1 : 2;
  uint32_t idx[2] = {0, 0};
  for (int k = 0; k < per; ++k) {
    idx[k] = D.indices[(size_t)per * p + k];
    if (idx[k] >= D.nverts) {
      atomicOr(&g.status[SWR_ST_FLAGS], SWR_F_BAD_INDEX);
      g.tri_flags[gp] = 0;
      return 0;
    }
  }
  const uint32_t r0 = D.vbase + idx[0], r1 = D.vbase + idx[per - 1];
  const float* v0 = g.ptv + (size_t)r0 * L::S;
  const float* v1 = g.ptv + (size_t)r1 * L::S;
  const int m0 = __float_as_int(v0[7]), m1 = __float_as_int(v1[7]);
  uint2 ref = make_uint2(r0, r1);
  uint32_t kept = 0;
  if (per == 1) {  // clipPoints: any outcode bit rejects
    kept = m0 == 0;
  } else if ((m0 | m1) == 0) {
    kept = 1;
  } else {
    // LineClipper against every plane whose bit is set in either outcode; each test uses
    // the original endpoints, t0 only grows and t1 only shrinks.
    const int m = m0 | m1;
    const float pl[6][4] = {{-1, 0, 0, 1}, {1, 0, 0, 1}, {0, -1, 0, 1}, {0, 1, 0, 1}, {0, 0, -1, 1}, {0, 0, 1, 1}};
    float t0 = 0.0f, t1 = 1.0f;
    bool gone = false;
    for (int k = 0; k < 6 && !gone; ++k) {
      if (!(m & (1 << k))) continue;
      const float d0 = Clipper<A, P>::dist(v0, pl[k][0], pl[k][1], pl[k][2], pl[k][3]);
      const float d1 = Clipper<A, P>::dist(v1, pl[k][0], pl[k][1], pl[k][2], pl[k][3]);
      const bool n0 = d0 < 0.0f, n1 = d1 < 0.0f;
      if (n0 && n1) {
        gone = true;
      } else if (n0) {
        const float t = swr_div(-d0, swr_sub(d1, d0));
        t0 = (t0 < t) ? t : t0;
      } else {
        const float t = swr_div(d0, swr_sub(d0, d1));
        t1 = (t < t1) ? t : t1;
      }
    }
    if (!gone) {
      // endpoints with a non-zero outcode are replaced (VertexProcessor.cpp:201-213)
      const int nnew = (m0 ? 1 : 0) + (m1 ? 1 : 0);
      const uint32_t vb = atomicAdd(&g.status[SWR_ST_CLIP_VERTS], (uint32_t)nnew);
      if (vb + nnew > g.cap_clip_verts) {
        atomicOr(&g.status[SWR_ST_FLAGS], SWR_F_CLIP_OVERFLOW);
        g.tri_flags[gp] = 0;
        return 0;
      }
      uint32_t next = vb;
      for (int e = 0; e < 2; ++e) {
        if (!(e ? m1 : m0)) continue;
        const float t = e ? t1 : t0;  // Helper::interpolateVertex(v0, v1, t)
        const float s = swr_sub(1.0f, t);
        float* o = g.clipv + (size_t)next * L::S;
        for (int c = 0; c < 4; ++c) o[c] = swr_add(swr_mul(v0[c], s), swr_mul(v1[c], t));
        for (int i = 0; i < A; ++i)
          o[L::OFF_A + i] = swr_add(swr_mul(v0[L::OFF_A + i], s), swr_mul(v1[L::OFF_A + i], t));
        for (int i = 0; i < P; ++i)
          o[L::OFF_P + i] = swr_add(swr_mul(v0[L::OFF_P + i], s), swr_mul(v1[L::OFF_P + i], t));
        to_screen(D, o[0], o[1], o[2], o[3], o[4], o[5], o[6]);
        o[7] = __int_as_float(0);
        if (e) ref.y = SWR_CLIP_REF | next; else ref.x = SWR_CLIP_REF | next;
        next++;
      }
      kept = 1;
    }
  }
  g.tri_flags[gp] = (uint8_t)kept;
  g.lp_refs[gp] = ref;
  return kept;
}

template <int A, int P>
__global__ void __launch_bounds__(256) k_assemble_lp_count(AssembleArgs g) {
  swr_pdl_entry();
  __shared__ uint32_t tmp[32];
  const uint32_t b = blockIdx.x;
  const int d = g.ndraws > 1 ? swr_find_le(g.draw_bbase, g.ndraws, b) : 0;
  const SwrDrawDesc& D = g.draws[d];
  const uint32_t p0 = (b - D.bbase) * SWR_BATCH_PRIMS;
  uint32_t sum = 0;
  for (int j = 0; j < 4; ++j) {
    const uint32_t p = p0 + threadIdx.x * 4 + j;
    if (p < D.nprims && p < p0 + SWR_BATCH_PRIMS) sum += assemble_lp_one<A, P>(g, D, p);
  }
  uint32_t tot;
  swr_block_exscan(sum, tmp, &tot);
  if (threadIdx.x == 0) g.batch_counts[b] = make_uint2(tot, 0u);
}

static __global__ void __launch_bounds__(256) k_assemble_lp_emit(AssembleArgs g) {
  swr_pdl_entry();
  __shared__ uint32_t tmp[32];
  if (g.status[SWR_ST_FLAGS] & SWR_F_ANY_OVERFLOW) return;
  const uint32_t b = blockIdx.x;
  const int d = g.ndraws > 1 ? swr_find_le(g.draw_bbase, g.ndraws, b) : 0;
  const SwrDrawDesc& D = g.draws[d];
  const uint32_t p0 = (b - D.bbase) * SWR_BATCH_PRIMS;
  uint32_t keep[4], sum = 0;
  for (int j = 0; j < 4; ++j) {
    const uint32_t p = p0 + threadIdx.x * 4 + j;
    keep[j] = (p < D.nprims && p < p0 + SWR_BATCH_PRIMS) ? g.tri_flags[D.pbase + p] & 1u : 0u;
    sum += keep[j];
  }
  uint32_t tot;
  uint32_t rank = swr_block_exscan(sum, tmp, &tot);
  const uint32_t base = g.batch_base[b];
  for (int j = 0; j < 4; ++j) {
    if (!keep[j]) continue;
    const uint2 r = g.lp_refs[D.pbase + p0 + threadIdx.x * 4 + j];
    g.tris[base + rank] = make_uint4(r.x, r.y, 0u, (uint32_t)d);
    rank++;
  }
}

// Per primitive: start vertex and per-step increment (computeVertexStep, Rasterizer.h:210-222).
template <class PS>
__global__ void __launch_bounds__(256) k_lp_setup(SetupArgs g) {
  swr_pdl_entry();
  typedef LpRec<PS> RL;
  if (g.status[SWR_ST_FLAGS] & SWR_F_ANY_OVERFLOW) return;
  uint32_t np = g.status[SWR_ST_PRIMS];
  if (np > g.cap_prims) np = g.cap_prims;
  for (uint32_t p = blockIdx.x * blockDim.x + threadIdx.x; p < np; p += gridDim.x * blockDim.x) {
    const uint4 t = g.tris[p];
    const SwrDrawDesc& D = g.draws[t.w];
    const float* vp[2];
    const uint32_t rr[2] = {t.x, t.y};
    for (int k = 0; k < 2; ++k)
      vp[k] = (rr[k] & SWR_CLIP_REF) ? g.clipv + (size_t)(rr[k] & ~SWR_CLIP_REF) * g.S : g.ptv + (size_t)rr[k] * g.S;
    float a[RL::NV], s[RL::NV];
    float b[RL::NV];
    for (int k = 0; k < 2; ++k) {
      float* o = k ? b : a;
      o[0] = vp[k][4]; o[1] = vp[k][5]; o[2] = vp[k][6]; o[3] = vp[k][3];
      for (int i = 0; i < RL::NA; ++i) o[4 + i] = i < g.vs_a ? vp[k][g.off_a + i] : 0.0f;
      for (int i = 0; i < RL::NP; ++i) o[4 + RL::NA + i] = i < g.vs_p ? vp[k][g.off_p + i] : 0.0f;
    }
    int steps = 1;
    if (D.draw_mode == 1) {
      const int adx = abs(swr_trunc_int(b[0]) - swr_trunc_int(a[0]));
      const int ady = abs(swr_trunc_int(b[1]) - swr_trunc_int(a[1]));
      steps = adx > ady ? adx : ady;
      const float fs = (float)steps;
      for (int i = 0; i < RL::NV; ++i) s[i] = swr_div(swr_sub(b[i], a[i]), fs);
    } else {
      for (int i = 0; i < RL::NV; ++i) s[i] = 0.0f;
    }
    float* rec = g.recs + (size_t)p * RL::R;
    rec[0] = __int_as_float(steps);
    rec[1] = __int_as_float((int)t.w);
    for (int i = 0; i < RL::NV; ++i) {
      rec[2 + i] = a[i];
      rec[2 + RL::NV + i] = s[i];
    }
    g.tile_count[p] = (uint32_t)(steps > 0 ? steps : 0);
  }
}

// Stepped vertex component i after j steps.  stepVertex (Rasterizer.h:196-207) advances z
// only with InterpolateZ and w only with InterpolateW; x, y and the variables always.
template <class PS>
__device__ __forceinline__ float lp_value(const float* rec, int i, int j) {
  typedef LpRec<PS> RL;
  if ((i == 2 && !PS::InterpolateZ) || (i == 3 && !PS::InterpolateW)) return rec[2 + i];
  return swr_fold(rec[2 + i], rec[2 + RL::NV + i], j);
}

struct LpFragArgs {
  const uint32_t* status;
  uint32_t cap_prims;
  const float* recs;
  const uint32_t* frag_off;   // exclusive scan of steps per primitive
  const uint32_t* nfrags;     // device total
  uint32_t cap_frags;
  const SwrDrawDesc* draws;
  const SwrTargetDesc* targets;
  uint32_t* keys;
  uint32_t* vals;
  uint32_t* status_w;
  uint32_t invalid;           // key of fragments that reach no target pixel (sorts last)
};

template <class PS>
__global__ void __launch_bounds__(256) k_lp_frags(LpFragArgs g) {
  swr_pdl_entry();
  typedef LpRec<PS> RL;
  if (g.status[SWR_ST_FLAGS] & SWR_F_ANY_OVERFLOW) return;
  const uint32_t nf = *g.nfrags;
  if (nf > g.cap_frags) {
    if (blockIdx.x == 0 && threadIdx.x == 0) {
      atomicOr(&g.status_w[SWR_ST_FLAGS], SWR_F_PAIR_OVERFLOW);
      g.status_w[SWR_ST_PAIRS] = nf;
    }
    return;
  }
  uint32_t np = g.status[SWR_ST_PRIMS];
  if (np > g.cap_prims) np = g.cap_prims;
  for (uint32_t f = blockIdx.x * blockDim.x + threadIdx.x; f < nf; f += gridDim.x * blockDim.x) {
    // primitive owning fragment f: last p with frag_off[p] <= f (primitives with zero
    // steps share an offset with their successor, so take the last)
    uint32_t lo = 0, hi = np - 1;
    while (lo < hi) {
      const uint32_t mid = (lo + hi + 1) >> 1;
      if (g.frag_off[mid] <= f) lo = mid; else hi = mid - 1;
    }
    const uint32_t p = lo;
    const int j = (int)(f - g.frag_off[p]);
    const float* rec = g.recs + (size_t)p * RL::R;
    const SwrDrawDesc& D = g.draws[__float_as_int(rec[1])];
    const SwrTargetDesc& T = g.targets[D.target];
    const float x = lp_value<PS>(rec, 0, j), y = lp_value<PS>(rec, 1, j);
    uint32_t key = g.invalid;
    // Rasterizer::scissorTest on the stepped float position (Rasterizer.h:144-147)
    if (x >= (float)D.sc_minx && x < (float)D.sc_maxx && y >= (float)D.sc_miny && y < (float)D.sc_maxy) {
      const int ix = swr_trunc_int(x), iy = swr_trunc_int(y);
      if (ix >= 0 && iy >= 0 && ix < T.width && iy < T.height)
        key = T.pixel_base + (uint32_t)iy * (uint32_t)T.width + (uint32_t)ix;
    }
    g.keys[f] = key;
    g.vals[f] = f;
  }
}

struct LpShadeArgs {
  const uint32_t* status;
  uint32_t cap_prims;
  const float* recs;
  const uint32_t* frag_off;
  const uint32_t* nfrags;
  uint32_t cap_frags;
  const uint32_t* keys;  // sorted
  const uint32_t* vals;  // fragment ids in sorted order
  const SwrDrawDesc* draws;
  const SwrTargetDesc* targets;
  const uint32_t* target_pixel_base;
  int ntargets;
  uint32_t invalid;
  uint32_t* status_w;
};

template <class PS>
__global__ void __launch_bounds__(256) k_lp_shade(LpShadeArgs g) {
  swr_pdl_entry();
  typedef LpRec<PS> RL;
  __shared__ uint32_t sfr[32];
  uint32_t frags = 0, passes = 0;
  const bool ok = !(g.status[SWR_ST_FLAGS] & SWR_F_ANY_OVERFLOW);
  const uint32_t nf = ok ? min(*g.nfrags, g.cap_frags) : 0u;
  uint32_t np = g.status[SWR_ST_PRIMS];
  if (np > g.cap_prims) np = g.cap_prims;
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < nf; i += gridDim.x * blockDim.x) {
    const uint32_t key = g.keys[i];
    if (key == g.invalid || (i > 0 && g.keys[i - 1] == key)) continue;
    const int ti = g.ntargets > 1 ? swr_find_le(g.target_pixel_base, g.ntargets, key) : 0;
    const SwrTargetDesc& T = g.targets[ti];
    const SwrUniforms& U = g.draws[T.first_draw].u;
    const uint32_t local = key - T.pixel_base;
    const int x = (int)(local % (uint32_t)T.width), y = (int)(local / (uint32_t)T.width);
    typename PS::State st;
    PS::load(st, x, y, U);
    for (uint32_t k = i; k < nf && g.keys[k] == key; ++k) {
      const uint32_t f = g.vals[k];
      uint32_t lo = 0, hi = np - 1;
      while (lo < hi) {
        const uint32_t mid = (lo + hi + 1) >> 1;
        if (g.frag_off[mid] <= f) lo = mid; else hi = mid - 1;
      }
      const float* rec = g.recs + (size_t)lo * RL::R;
      const int j = (int)(f - g.frag_off[lo]);
      // Rasterizer::pixelDataFromVertex (Rasterizer.h:161-173)
      GpuPixel<PS> pd;
      pd.x = x;
      pd.y = y;
      pd.eq = nullptr;  // points and lines carry no triangle equations
      if (PS::InterpolateZ) pd.z = lp_value<PS>(rec, 2, j);
      if (PS::InterpolateW) {
        pd.w = lp_value<PS>(rec, 3, j);
        pd.invw = swr_div(1.0f, pd.w);
      }
      for (int a = 0; a < RL::NA; ++a) pd.avar[a] = lp_value<PS>(rec, 4 + a, j);
      for (int a = 0; a < RL::NP; ++a) pd.pvar[a] = lp_value<PS>(rec, 4 + RL::NA + a, j);
      PS::drawPixel(pd, (int)lo, st, g.draws[__float_as_int(rec[1])].u);
      frags++;
    }
    PS::store(st, x, y, U);
    passes += st.writes;
  }
  uint32_t tot, ptot;
  swr_block_exscan(frags, sfr, &tot);
  swr_block_exscan(passes, sfr, &ptot);
  if (threadIdx.x == 0 && tot) {
    atomicAdd((unsigned long long*)&g.status_w[SWR_ST_SHADED_LO], (unsigned long long)tot);
    atomicAdd((unsigned long long*)&g.status_w[SWR_ST_PASSES_LO], (unsigned long long)ptot);
  }
}

}  // namespace swr
