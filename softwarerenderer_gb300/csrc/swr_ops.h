// Per-program stage launchers: the host side of setVertexShader<VS> / setPixelShader<PS>
// (VertexProcessor.h:77-85, Rasterizer.h:90-96).  Each built-in shader is compiled into
// its own kernels; the context picks the launchers by program id.
#pragma once
#include "swr_lines.cuh"

namespace swr {

struct VsOps {
  int attribs, A, P, S;  // AttribCount, AVarCount, PVarCount, post-transform record stride
  int elem_bytes[2];     // bytes read per element of attribute streams 0 and 1 (0: one whole stride,
                         // for every stream)
  void (*vertex)(const SwrDrawDesc* draws, int ndraws, const uint32_t* draw_vbase, uint32_t nverts,
                 float* ptv, cudaStream_t s);
  void (*assemble_count)(const AssembleArgs& a, uint32_t nbatches, cudaStream_t s);
  void (*assemble_emit)(const AssembleArgs& a, uint32_t nbatches, cudaStream_t s);
  void (*assemble_lp_count)(const AssembleArgs& a, uint32_t nbatches, cudaStream_t s);  // points, lines
  void (*assemble_lp_emit)(const AssembleArgs& a, uint32_t nbatches, cudaStream_t s);
  // vertex shading + assembly count + emit as one persistent cooperative launch (k_geometry);
  // bar: two zeroed words of device memory.  Returns a CUDA error (nothing queued on failure).
  cudaError_t (*geometry)(const SwrDrawDesc* draws, int ndraws, const uint32_t* draw_vbase, uint32_t nverts,
                          float* ptv, const AssembleArgs& a, uint32_t nbatches, uint32_t* bar, cudaStream_t s);
};

struct PsOps {
  int A, P, R, S;  // AVarCount, PVarCount, setup record words, direct-path vertex stride
  void (*direct_vertices)(const float* rv, uint32_t n, float* ptv, cudaStream_t s);
  void (*setup)(const SetupArgs& a, cudaStream_t s);
  void (*emit_pairs)(const uint32_t* status, uint32_t cap_prims, const float* recs,
                     const uint32_t* tile_count, const uint32_t* pair_off, const uint32_t* npairs,
                     uint32_t cap_pairs, const SwrDrawDesc* draws, const SwrTargetDesc* targets,
                     int tile, uint32_t* keys, uint32_t* vals, uint32_t* status_w, cudaStream_t s);
  void (*raster)(const RasterArgs& a, uint32_t ntiles, int tile, cudaStream_t s);
  void (*fill_bins)(const uint32_t* status, uint32_t cap_prims, const float* recs,
                    uint32_t* cell_count, const uint32_t* cell_start, uint32_t ncells, int seg_shift,
                    uint32_t cap_pairs, const SwrDrawDesc* draws, const SwrTargetDesc* targets, int tile,
                    uint32_t* bin, uint32_t* status_w, cudaStream_t s);
  int lp_R;  // point / line record words
  void (*lp_setup)(const SetupArgs& a, cudaStream_t s);
  void (*lp_frags)(const LpFragArgs& a, cudaStream_t s);
  void (*lp_shade)(const LpShadeArgs& a, cudaStream_t s);
  int needs_eq;  // shade() reads the triangle equations: triangles only
  int overwrite;    // SwrOverwrite: large tiles may be rasterized in slices (RasterArgs.slices)
  int state_bytes;  // sizeof(PS::State), per pixel and slice of RasterArgs.slice_state
  int depth_min;    // SwrDepthMin: heavy tiles may be rasterized in runs (RasterArgs.dslice)
  int slice_chunks; // SwrRasterSlices: by default tiles of more than this many chunks are (0: none)
  int chunk;        // SwrRasterChunk: primitives per raster chunk
};

const VsOps* vs_ops(int id);
const PsOps* ps_ops(int id);

}  // namespace swr

// A shader program compiled in a caller's own translation unit (include/swr/Renderer.h):
// the stage-launcher table of one vertex or pixel shader, handed to the library through
// swr_set_vertex_program / swr_set_pixel_program.  The kernels it launches are built from
// these headers in the caller's unit, so the library checks that both sides agree on the
// layout of every structure that crosses between them.
#define SWR_PROGRAM_MAGIC 0x50525753u  // "SWRP"
#define SWR_PROGRAM_ABI 3u             // bumped with any change to VsOps, PsOps or their argument structs
#define SWR_PROGRAM_VERTEX 1u
#define SWR_PROGRAM_PIXEL 2u

struct swr_program {
  uint32_t magic;     // SWR_PROGRAM_MAGIC
  uint32_t abi;       // SWR_PROGRAM_ABI
  uint32_t kind;      // SWR_PROGRAM_VERTEX or SWR_PROGRAM_PIXEL
  uint32_t sizes[10]; // swr_program_layout()
  const swr::VsOps* vs;
  const swr::PsOps* ps;
};

// Sizes of the structures the launchers exchange with the library.
inline void swr_program_layout(uint32_t* s) {
  s[0] = (uint32_t)sizeof(swr::VsOps);
  s[1] = (uint32_t)sizeof(swr::PsOps);
  s[2] = (uint32_t)sizeof(SwrDrawDesc);
  s[3] = (uint32_t)sizeof(SwrTargetDesc);
  s[4] = (uint32_t)sizeof(swr::AssembleArgs);
  s[5] = (uint32_t)sizeof(swr::SetupArgs);
  s[6] = (uint32_t)sizeof(swr::RasterArgs);
  s[7] = (uint32_t)sizeof(swr::LpFragArgs);
  s[8] = (uint32_t)sizeof(swr::LpShadeArgs);
  s[9] = (uint32_t)sizeof(SwrUniforms);
}
