// Vertex-stage kernels of one vertex shader: the launch wrappers and the VsOps table entry,
// instantiated per shader -- for the built-in shaders in swr_vs.cu, for a caller's own
// shader in the caller's translation unit (include/swr/Renderer.h).
#pragma once
#include "swr_ops.h"

namespace swr {
namespace {

constexpr int kVsGrid = 152 * 8;

template <class VS>
void run_vertex(const SwrDrawDesc* draws, int ndraws, const uint32_t* draw_vbase, uint32_t nverts,
                float* ptv, cudaStream_t s) {
  if (!nverts) return;
  const uint32_t want = (nverts + 255) / 256;
  const int grid = (int)(want < (uint32_t)kVsGrid ? want : (uint32_t)kVsGrid);
  swr::launch(k_vertex<VS>, grid, 256, 0, s, draws, ndraws, draw_vbase, nverts, ptv);
}

template <class VS>
void run_count(const AssembleArgs& a, uint32_t nbatches, cudaStream_t s) {
  if (nbatches) swr::launch(k_assemble_count<VS::AVarCount, VS::PVarCount>, 2 * nbatches, SWR_HALF, 0, s, a);
}

template <class VS>
void run_emit(const AssembleArgs& a, uint32_t nbatches, cudaStream_t s) {
  if (nbatches) swr::launch(k_assemble_emit<VS::AVarCount, VS::PVarCount>, 2 * nbatches, SWR_HALF, 0, s, a);
}

template <class VS>
void run_lp_count(const AssembleArgs& a, uint32_t nbatches, cudaStream_t s) {
  if (nbatches) swr::launch(k_assemble_lp_count<VS::AVarCount, VS::PVarCount>, nbatches, 256, 0, s, a);
}

inline void run_lp_emit(const AssembleArgs& a, uint32_t nbatches, cudaStream_t s) {
  if (nbatches) swr::launch(k_assemble_lp_emit, nbatches, 256, 0, s, a);
}

// Persistent geometry front end: as many 512-thread CTAs as can be resident at once (a
// cooperative launch, so the grid barriers inside cannot wait on CTAs that never start).
template <class VS>
cudaError_t run_geometry(const SwrDrawDesc* draws, int ndraws, const uint32_t* draw_vbase, uint32_t nverts, float* ptv,
                         const AssembleArgs& a, uint32_t nbatches, uint32_t* bar, cudaStream_t s) {
  static int grid = 0;
  if (!grid) {
    int dev = 0, sms = 0, per_sm = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_geometry<VS>, SWR_HALF, 0) != cudaSuccess ||
        per_sm < 1)
      return cudaErrorLaunchFailure;
    grid = sms * per_sm;
  }
  cudaLaunchConfig_t cfg;
  memset(&cfg, 0, sizeof(cfg));
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3(SWR_HALF);
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeCooperative;
  at[0].val.cooperative = 1;
  cfg.attrs = at;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k_geometry<VS>, draws, ndraws, draw_vbase, nverts, ptv, a, 2 * nbatches, bar);
}

template <class VS>
VsOps make_vs() {
  VsOps o;
  o.attribs = VS::AttribCount;
  o.A = VS::AVarCount;
  o.P = VS::PVarCount;
  o.S = VLayout<VS::AVarCount, VS::PVarCount>::S;
  o.elem_bytes[0] = VS::Bytes0;
  o.elem_bytes[1] = VS::Bytes1;
  o.vertex = &run_vertex<VS>;
  o.assemble_count = &run_count<VS>;
  o.assemble_emit = &run_emit<VS>;
  o.assemble_lp_count = &run_lp_count<VS>;
  o.assemble_lp_emit = &run_lp_emit;
  o.geometry = &run_geometry<VS>;
  return o;
}

}  // namespace
}  // namespace swr
