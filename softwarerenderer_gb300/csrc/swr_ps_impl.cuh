// Raster-stage kernels of the built-in pixel shaders: the launch wrappers and the PsOps table
// entry of one shader, instantiated per shader in the swr_ps_*.cu translation units (split
// so that the build compiles them in parallel).
#pragma once
#include "swr_ops.h"

namespace swr {
namespace {

constexpr int kGrid = 152 * 8;

template <class PS>
void run_direct(const float* rv, uint32_t n, float* ptv, cudaStream_t s) {
  if (!n) return;
  const uint32_t want = (n + 255) / 256;
  const int grid = (int)(want < (uint32_t)kGrid ? want : (uint32_t)kGrid);
  swr::launch(k_direct_vertices<PS::AVarCount, PS::PVarCount>, grid, 256, 0, s, rv, n, ptv);
}

template <class PS>
void run_setup(const SetupArgs& a, cudaStream_t s) {
  swr::launch(k_setup<PS>, kGrid, kSetupThreads, 0, s, a);
}

template <class PS>
void run_pairs(const uint32_t* status, uint32_t cap_prims, const float* recs, const uint32_t* tile_count,
               const uint32_t* pair_off, const uint32_t* npairs, uint32_t cap_pairs,
               const SwrDrawDesc* draws, const SwrTargetDesc* targets, int tile, uint32_t* keys,
               uint32_t* vals, uint32_t* status_w, cudaStream_t s) {
  swr::launch(k_emit_pairs<PS>, kGrid, 256, 0, s, status, cap_prims, recs, tile_count, pair_off, npairs, cap_pairs,
                                         draws, targets, tile, keys, vals, status_w);
}

template <class PS>
void run_fill(const uint32_t* status, uint32_t cap_prims, const float* recs,
              uint32_t* cell_count, const uint32_t* cell_start, uint32_t ncells, int seg_shift, uint32_t cap_pairs,
              const SwrDrawDesc* draws, const SwrTargetDesc* targets, int tile, uint32_t* bin, uint32_t* status_w,
              cudaStream_t s) {
  swr::launch(k_fill_bins<PS>, kGrid, 256, 0, s, status, cap_prims, recs, cell_count, cell_start, ncells,
                                        seg_shift, cap_pairs, draws, targets, tile, bin, status_w);
}

template <class PS>
void run_raster(const RasterArgs& a, uint32_t ntiles, int tile, cudaStream_t s) {
  constexpr int kChunk = SwrRasterChunk<PS>::value;  // primitives staged in shared memory per bin chunk
  if (!ntiles) return;
  // one CTA per tile, or per (tile, slice) for sliced overwrite shaders; Block-only
  // submissions run the instantiation without the Span-mode passes
  const bool sliced = SwrOverwrite<PS>::value && a.slices > 1;
  uint32_t grid = sliced ? ntiles * (uint32_t)a.slices : ntiles;
  if (SwrDepthMin<PS>::value && a.dslice) {  // the listed tiles' runs, then the other tiles
    grid = SWR_DSLICES * a.quad_cap + ntiles;
  } else if (tile == 16 && !SwrOverwrite<PS>::value) {  // quadrant CTAs (RasterArgs)
    if (a.quad_all) grid = 4 * ntiles;
    else if (a.quad_flag) grid = 4 * a.quad_cap + ntiles;
  }
  if (tile == 32) {
    if (a.has_span) swr::launch(k_raster<PS, 32, kChunk, true>, grid, 256, 0, s, a);
    else swr::launch(k_raster<PS, 32, kChunk, false>, grid, 256, 0, s, a);
    if constexpr (SwrOverwrite<PS>::value)
      if (sliced) swr::launch(k_merge_slices<PS, 32>, ntiles, 256, 0, s, a);
  } else {
    if (a.has_span) swr::launch(k_raster<PS, 16, kChunk, true>, grid, 256, 0, s, a);
    else swr::launch(k_raster<PS, 16, kChunk, false>, grid, 256, 0, s, a);
    if constexpr (SwrOverwrite<PS>::value)
      if (sliced) swr::launch(k_merge_slices<PS, 16>, ntiles, 256, 0, s, a);
  }
}

template <class PS>
void run_lp_setup(const SetupArgs& a, cudaStream_t s) {
  swr::launch(k_lp_setup<PS>, kGrid, 256, 0, s, a);
}

template <class PS>
void run_lp_frags(const LpFragArgs& a, cudaStream_t s) {
  swr::launch(k_lp_frags<PS>, kGrid, 256, 0, s, a);
}

template <class PS>
void run_lp_shade(const LpShadeArgs& a, cudaStream_t s) {
  swr::launch(k_lp_shade<PS>, kGrid, 256, 0, s, a);
}

template <class PS>
PsOps make_ps() {
  PsOps o;
  o.A = PS::AVarCount;
  o.P = PS::PVarCount;
  o.R = Rec<PS>::R;
  o.S = VLayout<PS::AVarCount, PS::PVarCount>::S;
  o.direct_vertices = &run_direct<PS>;
  o.setup = &run_setup<PS>;
  o.emit_pairs = &run_pairs<PS>;
  o.raster = &run_raster<PS>;
  o.fill_bins = &run_fill<PS>;
  o.lp_R = LpRec<PS>::R;
  o.lp_setup = &run_lp_setup<PS>;
  o.lp_frags = &run_lp_frags<PS>;
  o.lp_shade = &run_lp_shade<PS>;
  o.needs_eq = SwrNeedsEquations<PS>::value;
  o.overwrite = SwrOverwrite<PS>::value;
  o.state_bytes = (int)sizeof(typename PS::State);
  o.depth_min = SwrDepthMin<PS>::value;
  o.slice_chunks = SwrRasterSlices<PS>::value;
  o.chunk = SwrRasterChunk<PS>::value;
  return o;
}

}  // namespace
}  // namespace swr
