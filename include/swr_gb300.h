/* swr_gb300 — C ABI of the GB300 rasterization pipeline.
 *
 * A drop-in for the VertexProcessor + Rasterizer path of trenki2/SoftwareRenderer
 * (src/renderer/).  One swr_context holds the state that a VertexProcessor and a
 * Rasterizer hold together; every entry point names the reference member it replaces.
 * Shaders are compiled into the library as built-in programs (the reference binds them
 * as template arguments, setVertexShader<VS> / setPixelShader<PS>); their uniforms,
 * including the render target buffers that the reference's pixel shaders keep in
 * statics, travel in SwrUniforms (softwarerenderer_gb300/csrc/swr_programs.h).
 *
 * Memory: every buffer pointer passed here (attributes, indices, RasterizerVertex arrays,
 * the colour/depth/texture pointers inside SwrUniforms) is a CUDA device pointer.  The
 * context owns its scratch (post-transform vertices, clip table, bins) and grows it on
 * demand.  Draws are queued asynchronously on the given stream (NULL = legacy default
 * stream); swr_finish() waits and reports.  Errors are returned, never asserted.
 * A context is not reentrant (like VertexProcessor, VertexProcessor.h:146-151): use one
 * context per host thread / stream.
 */
#ifndef SWR_GB300_H
#define SWR_GB300_H

#include <stdint.h>

/* Every entry point is exported; the library's internal symbols (built with hidden
 * visibility) are not, so kernels a caller instantiates from the same headers for its
 * own shaders (include/swr/Renderer.h) never bind to the library's copies or vice versa. */
#if defined(__GNUC__)
#define SWR_API __attribute__((visibility("default")))
#else
#define SWR_API
#endif

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes. */
#define SWR_OK 0
#define SWR_EINVAL 1     /* invalid argument (the reference asserts or has undefined behaviour) */
#define SWR_ENOMEM 2     /* device allocation failed */
#define SWR_EOVERFLOW 3  /* a scratch queue was too small: the draw left its targets untouched,
                            the context has grown the queue; issue the draw again */
#define SWR_ECUDA 4      /* CUDA runtime error */
#define SWR_EINDEX 5     /* an index addressed a vertex beyond the bound attribute buffers */

/* Enumerations carry the reference's values. */
#define SWR_DRAW_POINT 0     /* DrawMode::Point    (VertexProcessor.h:42-46) */
#define SWR_DRAW_LINE 1      /* DrawMode::Line */
#define SWR_DRAW_TRIANGLE 2  /* DrawMode::Triangle */
#define SWR_CULL_NONE 0      /* CullMode::None     (VertexProcessor.h:49-53) */
#define SWR_CULL_CCW 1       /* CullMode::CCW */
#define SWR_CULL_CW 2        /* CullMode::CW (the reference's default) */
#define SWR_RASTER_SPAN 0    /* RasterMode::Span   (Rasterizer.h:45-49, default) */
#define SWR_RASTER_BLOCK 1   /* RasterMode::Block */
#define SWR_RASTER_ADAPTIVE 2 /* RasterMode::Adaptive */

typedef struct swr_context swr_context;
struct SwrUniforms; /* softwarerenderer_gb300/csrc/swr_programs.h */

typedef struct swr_stats {
  uint64_t fragments;   /* drawPixel calls since the last swr_finish */
  uint64_t primitives;  /* primitives handed to the rasterizer by the last draw */
  uint64_t bin_pairs;   /* (tile, primitive) bin entries of the last draw */
  uint32_t clip_polygons;  /* triangles clipped against the frustum in the last draw */
  uint32_t flags;       /* internal status bits (0 when everything succeeded) */
  uint64_t launches;    /* kernels this library launched since the last swr_finish */
  uint64_t passes;      /* colour writes by the pixel shaders (depth-test passes) since the last swr_finish */
} swr_stats;

/* Context lifetime.  Replaces constructing VertexProcessor(IRasterizer*) + Rasterizer()
 * (VertexProcessor.cpp:29-35, Rasterizer.h:67-72): defaults are CullMode::CW, depth range
 * (0, 1), RasterMode::Span, scissor (0, 0, 0, 0), tile size 16. */
SWR_API int swr_create(swr_context** out);
SWR_API int swr_destroy(swr_context* ctx);

/* VertexProcessor::setViewport (VertexProcessor.h:66, VertexProcessor.cpp:43-54). */
SWR_API int swr_set_viewport(swr_context* ctx, int x, int y, int width, int height);
/* VertexProcessor::setDepthRange (VertexProcessor.h:70, VertexProcessor.cpp:56-60). */
SWR_API int swr_set_depth_range(swr_context* ctx, float n, float f);
/* VertexProcessor::setCullMode (VertexProcessor.h:74, VertexProcessor.cpp:62-65). */
SWR_API int swr_set_cull_mode(swr_context* ctx, int mode);
/* VertexProcessor::setVertexShader<VS> (VertexProcessor.h:77-85): built-in VS id. */
SWR_API int swr_set_vertex_shader(swr_context* ctx, int vs_id);
/* VertexProcessor::setVertexAttribPointer (VertexProcessor.h:88, VertexProcessor.cpp:67-76).
 * `bytes` is the buffer size; the vertex count used for index bounds checks is
 * bytes / stride (the reference does not check indices). */
SWR_API int swr_set_vertex_attrib_pointer(swr_context* ctx, int index, int stride, const void* buffer,
                                  uint64_t bytes);
/* VertexProcessor::drawElements (VertexProcessor.h:91, VertexProcessor.cpp:78-120).
 * indices: device uint32 array; values must be < 2^31 - 1 (the reference's int). */
SWR_API int swr_draw_elements(swr_context* ctx, int mode, uint64_t count, const uint32_t* indices,
                      void* stream);

/* Shader programs compiled in the caller's own nvcc translation unit: setVertexShader<VS>
 * (VertexProcessor.h:77-85) and setPixelShader<PS> (Rasterizer.h:90-96) for shaders the
 * library does not ship.  A program is the table of stage launchers that the header-only
 * C++ front-end include/swr/Renderer.h instantiates for one VertexShaderBase- or
 * PixelShaderBase-derived class (swr::program<Shader>()); the library borrows it, so it
 * must outlive the draws that use it.  A program built against other headers (another
 * layout of the structures it exchanges with the library) is rejected with SWR_EINVAL.
 * The id-based setters and these replace each other. */
typedef struct swr_program swr_program;
SWR_API int swr_set_vertex_program(swr_context* ctx, const swr_program* program);
SWR_API int swr_set_pixel_program(swr_context* ctx, const swr_program* program);

/* Rasterizer::setRasterMode (Rasterizer.h:75-78). */
SWR_API int swr_set_raster_mode(swr_context* ctx, int mode);
/* Rasterizer::setScissorRect (Rasterizer.h:81-87). */
SWR_API int swr_set_scissor_rect(swr_context* ctx, int x, int y, int width, int height);
/* Rasterizer::setPixelShader<PS> (Rasterizer.h:90-96): built-in PS id. */
SWR_API int swr_set_pixel_shader(swr_context* ctx, int ps_id);
/* Shader uniforms and render target (the reference's shader statics).  Copied. */
SWR_API int swr_set_uniforms(swr_context* ctx, const struct SwrUniforms* u);
/* IRasterizer::draw{Point,Line,Triangle}List (IRasterizer.h:56-71, Rasterizer.h:116-141):
 * vertices are RasterizerVertex records (x, y, z, w, avar[16], pvar[16]; 36 floats) in
 * screen space; an index of -1 at the start of a primitive skips it. */
SWR_API int swr_draw_list(swr_context* ctx, int mode, const float* vertices, uint64_t nverts,
                  const int32_t* indices, uint64_t count, void* stream);

/* Batched rendering (no reference counterpart: the reference draws one mesh per
 * drawElements call).  One item is the state of one VertexProcessor::drawElements
 * (VertexProcessor.cpp:78-120) call with DrawMode::Triangle; all items of a batch use the
 * same vertex and pixel shader.  Items whose uniforms name the same colour buffer draw
 * into one shared target in item order; every other item gets its own target.  The whole
 * batch is one pass of the pipeline (every kernel covers all items), so per-item results
 * equal separate swr_draw_elements calls. */
typedef struct swr_draw_item {
  int32_t vs_id, ps_id;        /* built-in program ids; 0 = the context's current program */
  int32_t cull_mode, raster_mode;
  int32_t viewport[4];
  float depth_range[2];
  int32_t scissor[4];
  const void* attrib[8];
  int32_t attrib_stride[8];
  uint64_t attrib_bytes[8];
  const uint32_t* indices;
  uint64_t count;
  const struct SwrUniforms* uniforms;
  int32_t* prim_src;           /* optional primitive-source output, see swr_set_primitive_source */
  uint64_t prim_src_capacity;
} swr_draw_item;

SWR_API int swr_draw_batch(swr_context* ctx, const swr_draw_item* items, int n, void* stream);
/* With graph mode on, swr_draw_batch captures its kernel sequence in a CUDA graph the first
 * time a batch layout (item count, sizes, shaders, modes) is seen and replays it for later
 * batches with the same layout; uniforms and buffer pointers are refreshed on every call.
 * Triangle swr_draw_elements calls then run as one-item batches (so they replay too),
 * except while profiling is on (stage events need the launch-by-launch path). */
SWR_API int swr_set_graph_mode(swr_context* ctx, int on);

/* Wait for the stream, report and reset the accumulated status. */
SWR_API int swr_finish(swr_context* ctx, void* stream, swr_stats* stats);
/* Queue sizes (no reference counterpart: the reference grows std::vectors).  A context
 * sizes its primitive queue (triangles after clipping and culling) and its bin-entry queue
 * ((tile, primitive) pairs) ahead of every draw from the submitted count; a draw that
 * needs more is skipped on the device, swr_finish returns SWR_EOVERFLOW with the targets
 * untouched and grows the queue to what the draw asked for, and the caller draws again.
 * swr_set_queue_capacity fixes either size instead (0 keeps the automatic sizing): a
 * caller that knows its scenes (an autotuned batch) pre-sizes the queues once; they are
 * still grown after an overflow.  swr_get_queue_capacity reports the current sizes. */
SWR_API int swr_set_queue_capacity(swr_context* ctx, uint64_t primitives, uint64_t bin_entries);
SWR_API int swr_get_queue_capacity(swr_context* ctx, uint64_t* primitives, uint64_t* bin_entries);
/* Device-memory budget (no reference counterpart): the context's scratch allocations
 * fail with SWR_ENOMEM, queuing nothing, once they would hold more than `bytes` (0: no
 * limit, the default), exactly as when cudaMalloc itself fails; swr_memory_used reports
 * the bytes held. */
SWR_API int swr_set_memory_limit(swr_context* ctx, uint64_t bytes);
SWR_API int swr_memory_used(swr_context* ctx, uint64_t* bytes);
/* Screen tile edge of the bin/tile rasterizer: 16 or 32 pixels, or 8: 16-px bins with every
 * tile rasterized as four 8 x 8 CTAs.  swr_set_tile_split(ctx, 1) rasterizes only the heavy
 * 16-px tiles (more than three raster chunks of bin entries) as four 8 x 8 CTAs; off by
 * default (each such CTA still stages the whole bin, which costs more than it saves on the
 * measured workloads). */
SWR_API int swr_set_tile_size(swr_context* ctx, int tile);
SWR_API int swr_set_tile_split(swr_context* ctx, int on);
/* Heavy-tile slicing (no reference counterpart).  With a built-in depth-tested shader whose
 * result is the first fragment of smallest depth (Lambert, Lambert-textured, vertex colour,
 * nearest texture), a tile of more than `chunks` raster chunks of bin entries is rasterized
 * by four CTAs, each over a run of whole chunks from the draw's starting framebuffer, and
 * the runs are merged in primitive order: colour, depth, winner and fragment counts are
 * those of the sequential draw.  Only the `passes` statistic differs: each run counts its
 * depth-test passes against the depth its run started from.  chunks = 0 turns it off, -1
 * (the default) takes the shader's own setting (the Lambert shader: 1; the others: off). */
SWR_API int swr_set_tile_slicing(swr_context* ctx, int chunks);
/* Persistent geometry front end (no reference counterpart): triangle draws and batches run
 * vertex shading and triangle assembly as one cooperative launch whose CTAs stay resident
 * and meet at grid barriers between the stages, instead of three kernels.  Off by default;
 * a barrier that waits past its limit makes swr_finish return SWR_ECUDA. */
SWR_API int swr_set_persistent_geometry(swr_context* ctx, int on);
/* Test hook of that bounded wait: while on, the persistent launch's grid barrier starts from
 * an arrival count no arrival can complete, so every CTA waits out its limit (about a
 * second), gives up and ends; the draw leaves its targets untouched and swr_finish returns
 * SWR_ECUDA.  The context stays usable. */
SWR_API int swr_test_stall_geometry_barrier(swr_context* ctx, int on);
SWR_API const char* swr_status_string(int status);

/* Tracing (no reference counterpart; the reference has only Benchmark.cpp's chrono).
 * With profiling on, every draw records CUDA events at its stage boundaries on its own
 * stream; swr_stage_times waits for the draws recorded since its previous call and returns
 * their summed durations in ms for 5 stages: vertex shading, clip/cull/assembly, triangle
 * setup, binning, tile raster. */
SWR_API int swr_set_profiling(swr_context* ctx, int on);
SWR_API int swr_stage_times(swr_context* ctx, float* ms5);

/* Primitive sources (no reference counterpart; needed by swr_backward).  While set, each
 * triangle swr_draw_elements call writes out[k] = t, the source triangle (indices
 * [3t, 3t + 3) of its index list) of its k-th rasterized primitive -- k being the id the
 * pixel shaders see and SwrUniforms.winner records (the rasterizer's primitive numbering,
 * VertexProcessor.cpp:281-317 then Rasterizer.h:134-141).  A triangle that clipping splits
 * yields several primitives with one source.  At most `capacity` entries are written; a
 * draw with more primitives makes swr_finish return SWR_EINVAL.  NULL turns it off.
 * (swr_draw_item.prim_src is the same output for one item of a batch.) */
SWR_API int swr_set_primitive_source(swr_context* ctx, int32_t* out, uint64_t capacity);

/* Differentiable rendering (no reference counterpart: the reference renders forward only).
 * The forward is an ordinary draw with vertex shader SWR_VS_POS_RGB_UV and pixel shader
 * SWR_PS_DIFF (colour = interpolated vertex rgb * bilinear RGBA32F texel) that records the
 * winner buffer and the primitive sources.  swr_backward then returns the gradients of a
 * scalar image loss L with respect to the vertex records {x, y, z, r, g, b, u, v} and the
 * texels, with visibility held fixed (each pixel keeps the primitive that won it); the
 * position gradient flows through the perspective-correct barycentrics, which each tile
 * recomputes from the clip-space vertices (nothing per pixel is stored by the forward). */
typedef struct swr_grad_view {
  float mvp[16];            /* the view's SwrUniforms.mvp */
  int32_t viewport[4];      /* the view's viewport: x, y, width, height */
  int32_t width, height;    /* render target size; row pitch == width */
  const int32_t* winner;    /* forward output: per pixel primitive id, -1 = not covered */
  const int32_t* prim_src;  /* forward output: source triangle per primitive id */
  uint64_t nprims;          /* valid entries of prim_src */
  const float* grad_color;  /* dL/d(colour), RGBA32F per pixel; NULL selects the fused L2 loss: */
  const float* color;       /*   forward image, RGBA32F per pixel */
  const float* target;      /*   target image, RGBA32F per pixel */
  float loss_scale;         /*   L = loss_scale * sum over pixels and channels of (color - target)^2 */
  int32_t _pad;
} swr_grad_view;

typedef struct swr_backward_args {
  const float* vertices;    /* nverts records of 8 floats (stride 32 B, 16-byte aligned) */
  uint64_t nverts;
  const uint32_t* indices;  /* the forward's triangle list */
  uint64_t count;
  const float* texture;     /* RGBA32F texels, tex_h rows of tex_w (16-byte aligned) */
  int32_t tex_w, tex_h;
  float* grad_vertices;     /* += dL/d(vertex record): nverts x 8 floats (16-byte aligned) */
  float* grad_texture;      /* += dL/d(texel): tex_h x tex_w x 4 floats (16-byte aligned) */
  double* loss;             /* fused loss only: += L (may be NULL) */
} swr_backward_args;

/* Queues the backward of `nviews` views on `stream`; gradients accumulate (clear them
 * first).  Ids beyond nprims / the triangle count / the vertex count are skipped and make
 * swr_finish return SWR_EINDEX.  Float atomics make the summation order (not the terms)
 * vary from run to run. */
SWR_API int swr_backward(swr_context* ctx, const swr_backward_args* args, const swr_grad_view* views, int nviews,
                 void* stream);

/* Mip-mapped texturing (the reference's example texture, src/examples/Texture.h, used by
 * its Box example).  SWR_PS_TEX_MIP samples SwrUniforms.tex as a mip chain: level 0 of
 * tex_w x tex_h 0x00RRGGBB texels followed by every smaller level down to 1 x 1, each
 * max(1, w/2) x max(1, h/2) of the one before, anisotropically (up to
 * SwrUniforms.max_aniso taps, 0 = 8) with the footprint from
 * PixelData::computePerspectiveDerivatives (PixelData.h:128-145).
 * swr_mip_chain_size gives the level count and the total texels of the chain;
 * swr_build_mip_chain fills it from a level-0 image (Texture::generateMipmaps,
 * Texture.h:220-293; 2 x 2 box filter).  Both buffers are device memory. */
SWR_API int swr_mip_chain_size(int width, int height, int* levels, uint64_t* texels);
SWR_API int swr_build_mip_chain(const uint32_t* base, int width, int height, uint32_t* chain, void* stream);

/* OBJ ingestion: ObjData::loadFromFile + ObjData::toVertexArray of the reference's
 * examples (src/examples/ObjData.cpp:46-199).  A mesh holds the deduplicated vertex array
 * (8 floats per vertex: position xyz, normal xyz, texcoord uv -- ObjData::VertexArrayData)
 * and the fan-triangulated index array, in the reference's order.  Inputs on which the
 * reference has undefined behaviour (indices past their lists, words with more than three
 * '/'-separated parts, empty faces) return SWR_EINVAL.  swr_obj_read copies the arrays to
 * host memory (no GPU needed); swr_obj_upload copies them to device buffers on `stream` and
 * waits for it.  Either array pointer may be NULL. */
typedef struct swr_obj_mesh swr_obj_mesh;
SWR_API int swr_obj_parse(const char* text, uint64_t len, swr_obj_mesh** out);
SWR_API int swr_obj_load(const char* path, swr_obj_mesh** out);
SWR_API int swr_obj_counts(const swr_obj_mesh* mesh, uint64_t* nverts, uint64_t* nindices);
SWR_API int swr_obj_read(const swr_obj_mesh* mesh, float* vdata, int32_t* idata);
SWR_API int swr_obj_upload(const swr_obj_mesh* mesh, float* vdata, int32_t* idata, void* stream);
SWR_API int swr_obj_free(swr_obj_mesh* mesh);

/* Render-target clear (no reference counterpart: its applications clear their own
 * buffers, e.g. Box.cpp's SDL_FillRect): fills the target named by u -- colour
 * (color_bytes = 4 or 16 per pixel, the pattern at clear_color), depth (clear_depth) and,
 * when present, frag_count (0) and winner (-1) -- in one kernel on `stream`.  Buffers must
 * be 16-byte aligned (cudaMalloc is). */
SWR_API int swr_clear_target(const struct SwrUniforms* u, int color_bytes, const void* clear_color, float clear_depth,
                     void* stream);

/* Headless presentation (replaces the SDL window surface of the reference's examples,
 * Box.cpp:170-171, 315): writes width x height pixels -- device or host memory, row pitch
 * == width -- as 8-bit RGB to `path`, binary PPM for a ".ppm" name, PNG for ".png". */
#define SWR_PIXELS_RGBA8 0    /* uint32 per pixel, R in bits 0-7 (the RGBA8 built-in shaders) */
#define SWR_PIXELS_XRGB8 1    /* uint32 0x00RRGGBB (SWR_PS_TEX_MIP, the SDL surface format) */
#define SWR_PIXELS_RGBA32F 2  /* 4 floats per pixel, clamped to [0, 1] and rounded */
SWR_API int swr_write_image(const char* path, const void* pixels, int width, int height, int format);

/* Allocation-free triangle-list draw.  No counterpart in the reference (whose CPU
 * rasterizer needs no device scratch).  It is swr_draw_list(SWR_DRAW_TRIANGLE, ...) for
 * callers that must not allocate device memory -- an application whose device memory is
 * owned by another allocator or capped at start-up, a frame loop that must not stall in
 * the driver's allocator, a plugin handed only a stream and target buffers -- so it takes
 * its state as arguments instead of a swr_context (creating one allocates) and keeps all
 * scratch in one fixed 8 MiB __device__ array inside the library.  It calls no cudaMalloc
 * or cudaFree.  Limits: <= 4096 triangles, <= 12288 vertices, a target of <= 16384 tiles
 * of 16 x 16 pixels (e.g. 2048 x 2048); larger inputs return SWR_EINVAL up front, and more
 * than 262144 (tile, triangle) bin entries return SWR_EOVERFLOW with the target untouched.
 * Synchronous: returns after the stream has drained, so no call can be captured in a CUDA
 * graph (it copies its descriptors from pageable memory and synchronises the stream);
 * *fragments (may be NULL) receives the drawPixel count.  Past the first call it allocates
 * nothing.  The first call on a device is its set-up: it looks up the array's
 * address (cudaGetSymbolAddress), and under lazy module loading (the CUDA default) it is
 * also when the library's device code and the 8 MiB array are loaded, the one call that
 * can allocate -- make it once at start-up, before any stream capture.  After
 * cudaDeviceReset the next call repeats the set-up in the new context.  All calls share
 * the array: calls that overlap on the GPU race, so serialise them. */
SWR_API int swr_draw_triangle_list_noalloc(const struct SwrUniforms* u, int ps_id, int raster_mode,
                                   int scissor_x, int scissor_y, int scissor_w, int scissor_h,
                                   const float* vertices, uint64_t nverts,
                                   const int32_t* indices, uint64_t count, void* stream,
                                   uint64_t* fragments);

#ifdef __cplusplus
}
#endif
#endif /* SWR_GB300_H */
