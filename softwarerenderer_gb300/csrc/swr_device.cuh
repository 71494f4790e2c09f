// Device-side data structures and small collective helpers of the GB300 pipeline.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#include "swr_programs.h"

#define SWR_BATCH_PRIMS 1024  // VertexProcessor flushes every 1024 primitives (VertexProcessor.cpp:110-116)
#define SWR_BLOCK 8           // swr::BlockSize (IRasterizer.h:33)
#define SWR_CLIP_REF 0x80000000u  // vertex references with this bit address the clip-vertex buffer
#define SWR_SEGS 32               // primitive segments of the binning (cells per tile)
#ifndef SWR_RASTER_MINB
#define SWR_RASTER_MINB 0         // k_raster CTAs per SM to plan registers for (0: per shader)
#endif
#define SWR_RASTER_SORT 512       // tiles with at most this many bin entries are ordered by k_raster
#define SWR_SLICES_MAX 8          // overwrite shaders: CTAs (ordered bin slices) per tile of more than
                                  // SWR_RASTER_SORT entries, merged by k_merge_slices
#define SWR_DSLICES 4             // depth-min shaders: CTAs (runs of whole chunks) per listed heavy tile
#ifndef SWR_PIX_WALK
#define SWR_PIX_WALK 1            // k_raster's per-pixel primitive walk (shaders without depth cull or overwrite)
#endif
#ifndef SWR_DEPTH_CULL
#define SWR_DEPTH_CULL 1          // k_raster's per-chunk tile depth cull (depth-tested shaders)
#endif

// Status word layout (device memory, reset by every submission).
enum SwrStatusWord {
  SWR_ST_FLAGS = 0,       // error bits, see SwrStatusFlags
  SWR_ST_CLIP_SLOTS = 1,  // clip-table entries requested
  SWR_ST_CLIP_VERTS = 2,  // clip vertices requested
  SWR_ST_PRIMS = 3,       // primitives after clipping and culling
  SWR_ST_PAIRS = 4,       // (tile, primitive) pairs requested
  SWR_ST_FRAGS = 5,       // line/point fragments requested
  SWR_ST_SHADED_LO = 6,   // drawPixel calls (64-bit, low word)
  SWR_ST_SHADED_HI = 7,
  SWR_ST_WORDS = 8,
  SWR_ST_PASSES_LO = 14,  // colour writes (depth-test passes), 64-bit (8-byte aligned), sticky
  SWR_ST_PASSES_HI = 15
};

enum SwrStatusFlags {
  SWR_F_BAD_INDEX = 1,       // an index addressed a vertex beyond the attribute buffers
  SWR_F_CLIP_OVERFLOW = 2,   // clip table or clip-vertex buffer too small
  SWR_F_PRIM_OVERFLOW = 4,   // primitive buffer too small
  SWR_F_PAIR_OVERFLOW = 8,   // bin pair buffer too small
  SWR_F_FRAG_OVERFLOW = 16,  // line/point fragment buffer too small
  SWR_F_CLIP_COMPLEX = 32,   // a clipped polygon exceeded 16 vertices and was dropped
  SWR_F_SRC_OVERFLOW = 64,   // a caller's primitive-source buffer was too small
  SWR_F_BAD_GRAD_INPUT = 128,  // backward: a winner or source id beyond the given counts
  SWR_F_BARRIER_TIMEOUT = 256,  // a grid barrier of a persistent launch gave up waiting
};
#define SWR_F_ANY_OVERFLOW (SWR_F_CLIP_OVERFLOW | SWR_F_PRIM_OVERFLOW | SWR_F_PAIR_OVERFLOW | SWR_F_FRAG_OVERFLOW)
#define SWR_ST_STICKY 8  // words SWR_ST_STICKY + i keep the largest value word i reached (i = CLIP_SLOTS..FRAGS)

// Programmatic dependent launch.  Kernels of a draw are launched so that the next one may
// become resident while the one before it drains (swr::launch); each such kernel begins
// with swr_pdl_entry(): it waits until every kernel before it on the stream has completed
// and its writes are visible (griddepcontrol.wait, a no-op for a kernel launched without
// the attribute), then lets its own dependents launch.  Nothing of a draw's memory is
// touched before the wait, so the order of all reads and writes is unchanged.
__device__ __forceinline__ void swr_pdl_entry() {
  asm volatile("griddepcontrol.wait;" ::: "memory");
  asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

namespace swr {

// Launch with the programmatic-stream-serialization attribute (unless SWR_PDL=0 is set in
// the environment, which launches every kernel fully serialised, as <<<...>>> does).
inline bool pdl_enabled() {
  static const bool on = [] {
    const char* e = getenv("SWR_PDL");
    return !(e && e[0] == '0');
  }();
  return on;
}

template <typename... P, typename... A>
inline void launch(void (*kernel)(P...), dim3 grid, dim3 block, size_t smem, cudaStream_t s, A... args) {
  cudaLaunchConfig_t cfg;
  memset(&cfg, 0, sizeof(cfg));
  cfg.gridDim = grid;
  cfg.blockDim = block;
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute at[1];
  at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  at[0].val.programmaticStreamSerializationAllowed = 1;
  cfg.attrs = at;
  cfg.numAttrs = pdl_enabled() ? 1 : 0;
  cudaLaunchKernelEx(&cfg, kernel, ((P)args)...);
}

}  // namespace swr

// End of a draw: the sticky maxima of the queue sizes it requested (the host grows its
// queues from them after an overflow).  One thread, after every stage that counts.
__device__ __forceinline__ void swr_close_status(uint32_t* st) {
  for (int i = SWR_ST_CLIP_SLOTS; i <= SWR_ST_FRAGS; ++i) {
    const uint32_t v = st[i];
    if (v > st[SWR_ST_STICKY + i]) st[SWR_ST_STICKY + i] = v;
  }
}

// One draw of a submission: the state VertexProcessor and Rasterizer hold for one
// drawElements call (VertexProcessor.h:140-151, Rasterizer.h:54-63).
struct SwrDrawDesc {
  const void* attrib[8];
  int32_t attrib_stride[8];
  const uint32_t* indices;
  uint32_t nidx;      // index count
  uint32_t nverts;    // vertices addressable in every bound attribute stream
  uint32_t vbase;     // first post-transform vertex of this draw
  uint32_t pbase;     // first submitted primitive of this draw (global numbering)
  uint32_t bbase;     // first batch of this draw (global numbering)
  uint32_t nprims;    // submitted primitives
  int32_t target;     // render target index
  int32_t draw_mode;  // 0 Point, 1 Line, 2 Triangle
  int32_t cull;       // 0 None, 1 CCW, 2 CW
  int32_t raster_mode;  // 0 Span, 1 Block, 2 Adaptive
  float vp_px, vp_py, vp_ox, vp_oy;  // VertexProcessor::setViewport (VertexProcessor.cpp:43-54)
  float dn, df;                      // VertexProcessor::setDepthRange
  int32_t sc_minx, sc_miny, sc_maxx, sc_maxy;  // Rasterizer::setScissorRect (Rasterizer.h:81-87)
  int32_t direct;     // 1: vertices are RasterizerVertex records already in screen space
  uint32_t prim_src_cap;  // entries of prim_src
  int32_t* prim_src;  // optional: per emitted primitive (draw-relative id) its source triangle
  SwrUniforms u;
};

// Render target: a tile grid over width x height pixels.  Draws that share a target
// share its tiles, so their primitives meet in one ordered bin per tile.
struct SwrTargetDesc {
  int32_t width, height;
  int32_t tiles_x, tiles_y;
  uint32_t tile_base;
  int32_t first_draw;  // draw whose uniforms carry the framebuffer pointers
  uint32_t pixel_base;  // first global pixel key of this target (point / line fragments)
  int32_t _pad;
};

// Result of clipping one triangle (PolyClipper, PolyClipper.cpp:45-81): a polygon of up
// to 16 vertices emitted as a fan; keep/swap bits per fan triangle from culling.
struct SwrClipEntry {
  uint32_t ref[16];
  uint16_t n;
  uint16_t keep;
  uint16_t swap;
  uint16_t _pad;
};

// Index of the last element of sorted `base[0..n)` that is <= key.
__device__ __forceinline__ int swr_find_le(const uint32_t* base, int n, uint32_t key) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (base[mid] <= key) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// Block-wide sums of two values per thread (blockDim.x multiple of 32, <= 1024), returned
// to every thread.  `tmp` needs 64 words and is not reused by the caller.
__device__ __forceinline__ void swr_block_sum2(uint32_t a, uint32_t b, uint32_t* tmp, uint32_t& sa, uint32_t& sb) {
  a = __reduce_add_sync(0xffffffffu, a);
  b = __reduce_add_sync(0xffffffffu, b);
  if ((threadIdx.x & 31) == 0) {
    tmp[threadIdx.x >> 5] = a;
    tmp[32 + (threadIdx.x >> 5)] = b;
  }
  __syncthreads();
  sa = sb = 0;
  for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
    sa += tmp[w];
    sb += tmp[32 + w];
  }
}

// Block-wide exclusive scan of one value per thread (blockDim.x multiple of 32, <= 1024).
// `tmp` needs 32 words.  Returns the exclusive prefix; *total receives the block sum.
__device__ __forceinline__ uint32_t swr_block_exscan(uint32_t v, uint32_t* tmp, uint32_t* total) {
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int nwarps = blockDim.x >> 5;
  uint32_t x = v;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) tmp[warp] = x;
  __syncthreads();
  if (warp == 0) {
    uint32_t s = lane < nwarps ? tmp[lane] : 0u;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, s, o);
      if (lane >= o) s += y;
    }
    tmp[lane] = s;  // inclusive warp totals
  }
  __syncthreads();
  const uint32_t warp_off = warp ? tmp[warp - 1] : 0u;
  if (total) *total = tmp[nwarps - 1];
  __syncthreads();
  return warp_off + x - v;
}
