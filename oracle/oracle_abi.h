/* Test infrastructure: the plain-C entry point shared by the CPU oracle port
 * (oracle/port/swr_port.cpp) and by the harness that drives the compiled reference
 * library (oracle/ref_harness.cpp).  Both take one draw description, run the
 * reference's VertexProcessor::drawElements (VertexProcessor.cpp:78-120) or, when
 * raster_vertices is set, the Rasterizer::draw*List path (Rasterizer.h:116-141), with
 * the built-in shader programs of swr_programs.h, and report counters.  Only tests,
 * the smoke check and the bench's CPU baseline use this. */
#pragma once
#include <stdint.h>
#include "../softwarerenderer_gb300/csrc/swr_programs.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct OracleDraw {
  int32_t vs_id, ps_id;      /* SwrVsId / SwrPsId */
  int32_t draw_mode;         /* 0 Point, 1 Line, 2 Triangle (DrawMode, VertexProcessor.h:42-46) */
  int32_t cull_mode;         /* 0 None, 1 CCW, 2 CW (CullMode, VertexProcessor.h:49-53) */
  int32_t raster_mode;       /* 0 Span, 1 Block, 2 Adaptive (RasterMode, Rasterizer.h:45-49) */
  int32_t viewport[4];       /* x, y, width, height (VertexProcessor::setViewport) */
  float depth_range[2];      /* n, f (VertexProcessor::setDepthRange) */
  int32_t scissor[4];        /* x, y, width, height (Rasterizer::setScissorRect) */
  int32_t attrib_stride[8];  /* VertexProcessor::setVertexAttribPointer */
  const void* attrib[8];
  const int32_t* indices;
  uint64_t count;
  /* Direct Rasterizer path: RasterizerVertex array (x, y, z, w, avar[16], pvar[16]). */
  const float* raster_vertices;
  const SwrUniforms* uniforms;
  int32_t threads;           /* OpenMP threads for the port (0 = runtime default) */
  int32_t _pad;
  /* Port only (triangles through drawElements): prim_src[k] = source triangle of the k-th
   * primitive handed to the rasterizer; at most prim_src_cap entries are written. */
  int32_t* prim_src;
  uint64_t prim_src_cap;
} OracleDraw;

typedef struct OracleStats {
  uint64_t fragments;   /* drawPixel calls inside the render target */
  uint64_t outside;     /* drawPixel calls outside the render target (dropped) */
  uint64_t primitives;  /* primitives handed to Rasterizer::draw{Point,Line,Triangle} */
  uint64_t batches;     /* VertexProcessor batches processed */
} OracleStats;

/* Returns 0 on success, non-zero on invalid input. */
int oracle_draw(const OracleDraw* d, OracleStats* st);

/* Differentiable rendering reference (port only, oracle/port/swr_diff.cpp), in double.
 * Scene: vertex records {x, y, z, r, g, b, u, v} (the SWR_VS_POS_RGB_UV stream) and an
 * RGBA32F texture, widened to double by the caller.  A view is one forward draw with
 * PsDiff: its mvp, viewport and target size, its winner buffer and primitive-source map
 * (visibility, held fixed), the target image of the L2 loss and/or dL/d(colour). */
typedef struct OracleDiffScene {
  const double* vertices;  /* nverts x 8 */
  uint64_t nverts;
  const int32_t* indices;  /* triangle list */
  uint64_t count;
  const double* texture;   /* tex_h x tex_w x 4 */
  int32_t tex_w, tex_h;
} OracleDiffScene;

typedef struct OracleDiffView {
  float mvp[16];
  int32_t viewport[4];
  int32_t width, height;
  const int32_t* winner;     /* per pixel primitive id, -1 none */
  const int32_t* prim_src;   /* per primitive id its source triangle */
  uint64_t nprims;
  const float* grad_color;   /* dL/d(colour) per pixel (RGBA), or NULL: 2 (colour - target) */
  const float* target;       /* RGBA per pixel, or NULL (then grad_color is required) */
} OracleDiffView;

/* loss (may be NULL) = sum over covered pixels and channels of (colour - target)^2 with the
 * colour recomputed at fixed visibility; grad_vertices (nverts x 8) and grad_texture
 * (tex_h x tex_w x 4), each may be NULL, receive += dL/d(parameter).  Returns 0, 1 for
 * invalid arguments, 2 for a winner or source id beyond the given counts. */
int oracle_diff_eval(const OracleDiffScene* s, const OracleDiffView* views, int nviews, double* loss,
                     double* grad_vertices, double* grad_texture);
/* Central differences (L(p + h) - L(p - h)) / 2h of that loss for n parameters:
 * kind 0 = vertex-record component index (8 * vertex + component), kind 1 = texel
 * component (4 * texel + channel).  OpenMP over parameters (threads 0 = default). */
int oracle_diff_fd(const OracleDiffScene* s, const OracleDiffView* views, int nviews, const int32_t* kind,
                   const uint64_t* index, int n, double h, double* out, int threads);
/* swr_fold exposed for the tests of the fast-forward. */
float oracle_fold(float v, float a, int k);
/* Randomized comparison of swr_fold with serial stepping; returns the mismatch count. */
uint64_t oracle_fold_selftest(uint64_t iters, uint64_t seed);

#ifdef __cplusplus
}
#endif
