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
} OracleDraw;

typedef struct OracleStats {
  uint64_t fragments;   /* drawPixel calls inside the render target */
  uint64_t outside;     /* drawPixel calls outside the render target (dropped) */
  uint64_t primitives;  /* primitives handed to Rasterizer::draw{Point,Line,Triangle} */
  uint64_t batches;     /* VertexProcessor batches processed */
} OracleStats;

/* Returns 0 on success, non-zero on invalid input. */
int oracle_draw(const OracleDraw* d, OracleStats* st);
/* swr_fold exposed for the tests of the fast-forward. */
float oracle_fold(float v, float a, int k);
/* Randomized comparison of swr_fold with serial stepping; returns the mismatch count. */
uint64_t oracle_fold_selftest(uint64_t iters, uint64_t seed);

#ifdef __cplusplus
}
#endif
