// swr/Renderer.h -- the reference's C++ API over the GB300 pipeline, header-only.
//
// A drop-in for trenki2/SoftwareRenderer's public API (src/renderer/Renderer.h and the
// headers it includes): VertexShaderBase / PixelShaderBase with AttribCount, AVarCount,
// PVarCount, InterpolateZ and InterpolateW; VertexProcessor with setViewport,
// setDepthRange, setCullMode, setVertexShader<VS>, setVertexAttribPointer and drawElements
// in Point, Line and Triangle modes; Rasterizer with setRasterMode (Span, Block, Adaptive),
// setScissorRect, setPixelShader<PS> and the draw* calls of IRasterizer.  Names, argument
// meaning, defaults and per-pixel results are the reference's.
//
// What changes for an application:
//   * The translation unit that calls setVertexShader<VS>() / setPixelShader<PS>() is
//     compiled by nvcc (-gencode arch=compute_103a,code=sm_103a): those calls instantiate the
//     pipeline's kernels for the shader classes right there, so processVertex and drawPixel
//     run on the GPU inside them.  Mark both __device__ (SWR_SHADER is that qualifier).
//   * What the reference's shaders keep in statics (matrices, framebuffer and texture
//     pointers) lives in __device__ or __constant__ variables of that translation unit, set
//     with cudaMemcpyToSymbol; drawPixel writes the application's own device buffers.
//     Pixels are handed to drawPixel in the reference's order: for every pixel, its
//     fragments in primitive order, one at a time -- the read-modify-write of a depth test
//     on the shader's own buffers is safe.
//   * Vertex attribute, index and RasterizerVertex arrays may be device memory
//     (cudaMalloc / cudaMallocManaged; used in place, bounds from the allocation's extent)
//     or ordinary host memory (copied to the device at every draw: attributes then need
//     host indices, which give the vertex count, and each host attribute array must be
//     readable for (largest index + 1) x stride bytes).
//   * drawElements and the draw* calls return once the draw has finished on the GPU, like
//     the reference's; a failure throws swr::Error (the reference asserts).
//   * The render target is the region [0, scissor x + width) x [0, scissor y + height)
//     -- widened to the viewport for VertexProcessor draws -- and fragments outside it are
//     not shaded (the reference would call drawPixel there).  PixelData carries no
//     pvarTemp, and a triangle's TriangleEquations (PixelData::equations) expose z, invw,
//     avar[] and pvar[] for computePerspectiveDerivatives, without the edge equations.
//
// The C ABI (include/swr_gb300.h) takes the same shader classes through
// swr::vertex_program<VS>() and swr::pixel_program<PS>() with swr_set_vertex_program /
// swr_set_pixel_program.
#pragma once

#ifndef __CUDACC__
#error "swr/Renderer.h instantiates the pipeline's kernels for your shaders: compile this file with nvcc"
#endif

#include <cuda.h>  // CUdeviceptr, CUresult: cuMemGetAddressRange is resolved at run time
#include <cuda_runtime.h>

#include <algorithm>
#include <cstddef>
#include <cstdint>
#include <cstring>
#include <stdexcept>
#include <string>
#include <type_traits>

#include "../swr_gb300.h"
#include "../../softwarerenderer_gb300/csrc/swr_ps_impl.cuh"
#include "../../softwarerenderer_gb300/csrc/swr_vs_impl.cuh"

// Qualifier of processVertex and drawPixel.
#define SWR_SHADER __device__

namespace swr {

// Constants of IRasterizer.h:33-40 and VertexConfig.h:34.
const int BlockSize = 8;
const int MaxAVars = 16;
const int MaxPVars = 16;
const int MaxVertexAttribs = 8;

// IRasterizer.h:42-53: vertex shader output and direct rasterizer input.
struct RasterizerVertex {
  float x, y, z, w;
  float avar[MaxAVars];
  float pvar[MaxPVars];
};
typedef RasterizerVertex VertexShaderOutput;           // VertexConfig.h:37
typedef const void* VertexShaderInput[MaxVertexAttribs];  // VertexConfig.h:40

enum class DrawMode { Point, Line, Triangle };  // VertexProcessor.h:42-46
enum class CullMode { None, CCW, CW };          // VertexProcessor.h:49-53
enum class RasterMode { Span, Block, Adaptive };  // Rasterizer.h:45-49

// ParameterEquation.h:33-62: one interpolant's plane a x + b y + c.
struct ParameterEquation {
  float a, b, c;
  __host__ __device__ float evaluate(float x, float y) const { return swr_eval(a, b, c, x, y); }
  __host__ __device__ float stepX(float v) const { return swr_add(v, a); }
  __host__ __device__ float stepY(float v) const { return swr_add(v, b); }
};

// TriangleEquations.h:39-47 as seen from a pixel shader: the planes of z, 1/w and the
// affine and perspective variables (the latter already multiplied by 1/w) of the triangle
// being drawn.  avar[i] / pvar[i] read the setup record the tile rasterizer holds on chip.
class TriangleEquations {
 public:
  struct Planes {
    const float* q;
    __device__ ParameterEquation operator[](int i) const {
      ParameterEquation e;
      e.a = q[3 * i];
      e.b = q[3 * i + 1];
      e.c = q[3 * i + 2];
      return e;
    }
  };
  ParameterEquation z;
  ParameterEquation invw;
  Planes avar;
  Planes pvar;
};

// PixelData.h:35-146: what drawPixel receives.
struct PixelData {
  int x, y;
  float z;
  float w;
  float invw;
  float avar[MaxAVars];
  float pvar[MaxPVars];
  const TriangleEquations* equations;  // the triangle's equations; null for points and lines

  // PixelData::computePerspectiveDerivatives (PixelData.h:128-145): d(pvar)/dx and
  // d(pvar)/dy at the pixel centre by the quotient rule, in the reference's operation order.
  __device__ void computePerspectiveDerivatives(const TriangleEquations& eqn, int varIndex, float& ddx,
                                                float& ddy) const {
    const float fx = swr_add((float)x, 0.5f), fy = swr_add((float)y, 0.5f);
    const ParameterEquation pv = eqn.pvar[varIndex];
    const float var = pv.evaluate(fx, fy);
    const float inv = eqn.invw.evaluate(fx, fy);
    const float den = swr_mul(inv, inv);
    ddx = swr_div(swr_sub(swr_mul(inv, pv.a), swr_mul(var, eqn.invw.a)), den);
    ddy = swr_div(swr_sub(swr_mul(inv, pv.b), swr_mul(var, eqn.invw.b)), den);
  }
};

// VertexShaderBase.h:33-51.  Derive, redefine the counts and processVertex (__device__).
// Vertex v is shaded when a whole stride of each attribute buffer is there at v.  A shader
// reading a stream interleaved at an offset inside larger records (whose last element ends
// before a full stride) states with `static const int AttribBytes` how many bytes it reads
// per element (at least those it reads from that stream).
template <class Derived>
class VertexShaderBase {
 public:
  static const int AttribCount = 0;
  static const int AVarCount = 0;
  static const int PVarCount = 0;
  SWR_SHADER static void processVertex(VertexShaderInput, VertexShaderOutput*) {}
};

class DummyVertexShader : public VertexShaderBase<DummyVertexShader> {};

// PixelShaderBase.h:40-137.  Derive, redefine the flags and counts and drawPixel
// (__device__).  An optional `static const int RasterOccupancy` (1-8, default 4) sets how
// many 256-thread tile rasterizer blocks per SM the shader's register use must allow, and
// an optional `static const int RasterChunk` (32, 64, 96 or 128, default 64) how many
// binned primitives the tile rasterizer stages at a time.
template <class Derived>
class PixelShaderBase {
 public:
  static const int InterpolateZ = false;
  static const int InterpolateW = false;
  static const int AVarCount = 0;
  static const int PVarCount = 0;
  SWR_SHADER static void drawPixel(const PixelData&) {}
};

class NullPixelShader : public PixelShaderBase<NullPixelShader> {};

// Status of a failed call (the reference asserts where these are thrown).
class Error : public std::runtime_error {
 public:
  Error(int code, const char* what)
      : std::runtime_error(std::string("swr: ") + what + ": " + swr_status_string(code)), code_(code) {}
  int code() const { return code_; }

 private:
  int code_;
};

namespace detail {

inline void check(int rc, const char* what) {
  if (rc != SWR_OK) throw Error(rc, what);
}

// The pipeline's vertex-shader contract (k_vertex) over a VertexShaderBase class.
// Bytes a vertex shader reads from each attribute element: `static const int AttribBytes` in
// the class, else 0 (a whole stride).  A vertex is shaded only if that many bytes of its
// element lie inside every attribute buffer.
template <class VS, class = void>
struct AttribBytes {
  enum { value = 0 };
};
template <class VS>
struct AttribBytes<VS, decltype((void)VS::AttribBytes)> {
  enum { value = VS::AttribBytes };
};

template <class VS>
struct UserVS {
  enum { AttribCount = VS::AttribCount, AVarCount = VS::AVarCount, PVarCount = VS::PVarCount,
         Bytes0 = AttribBytes<VS>::value, Bytes1 = AttribBytes<VS>::value };
  static_assert(VS::AttribCount >= 0 && VS::AttribCount <= MaxVertexAttribs, "AttribCount <= MaxVertexAttribs");
  static_assert(VS::AVarCount >= 0 && VS::AVarCount <= MaxAVars, "AVarCount <= MaxAVars");
  static_assert(VS::PVarCount >= 0 && VS::PVarCount <= MaxPVars, "PVarCount <= MaxPVars");
  template <class Out>
  __device__ static void processVertex(const SwrVertexInput& in, Out* out, const SwrUniforms&) {
    VertexShaderInput p;
#pragma unroll
    for (int i = 0; i < MaxVertexAttribs; ++i) p[i] = i < VS::AttribCount ? in.p[i] : nullptr;
    RasterizerVertex v;
    VS::processVertex(p, &v);
    out->x = v.x;
    out->y = v.y;
    out->z = v.z;
    out->w = v.w;
#pragma unroll
    for (int i = 0; i < VS::AVarCount; ++i) out->avar[i] = v.avar[i];
#pragma unroll
    for (int i = 0; i < VS::PVarCount; ++i) out->pvar[i] = v.pvar[i];
  }
};

// The pipeline's pixel-shader contract over a PixelShaderBase class: drawPixel has its own
// side effects, so the rasterizer calls it once per fragment, in primitive order per pixel
// (NoCompact), and keeps no framebuffer state of its own (State only counts).
template <class PS>
struct UserPS {
  enum { AVarCount = PS::AVarCount, PVarCount = PS::PVarCount, InterpolateZ = PS::InterpolateZ ? 1 : 0,
         InterpolateW = PS::InterpolateW ? 1 : 0, HasDepth = 0, NoCompact = 1,
         RasterOccupancy = SwrRasterOccupancy<PS>::value, RasterChunk = SwrRasterChunk<PS>::value };
  static_assert(PS::AVarCount >= 0 && PS::AVarCount <= MaxAVars, "AVarCount <= MaxAVars");
  static_assert(PS::PVarCount >= 0 && PS::PVarCount <= MaxPVars, "PVarCount <= MaxPVars");
  struct State {
    float depth;
    uint32_t frags, writes;
    int32_t winner;
  };
  typedef uint32_t Color;
  __device__ static void load(State& s, int, int, const SwrUniforms&) {
    s.depth = 0.0f;
    s.frags = 0u;
    s.writes = 0u;
    s.winner = -1;
  }
  __device__ static void store(const State&, int, int, const SwrUniforms&) {}
  __device__ static bool earlyReject(float, State&) { return false; }
  template <class PD>
  __device__ static Color shade(const PD&, const SwrUniforms&) {
    return 0u;  // never used: nothing is shaded ahead of drawPixel (NoCompact)
  }
  __device__ static void apply(State&, float, Color, int) {}
  template <class PD>
  __device__ static void drawPixel(const PD& g, int, State& s, const SwrUniforms&) {
    typedef Rec<UserPS> RL;
    PixelData p;
    p.x = g.x;
    p.y = g.y;
    if (InterpolateZ) p.z = g.z;
    if (RL::IW) {
      p.w = g.w;
      p.invw = g.invw;
    }
#pragma unroll
    for (int i = 0; i < PS::AVarCount; ++i) p.avar[i] = g.avar[i];
#pragma unroll
    for (int i = 0; i < PS::PVarCount; ++i) p.pvar[i] = g.pvar[i];
    TriangleEquations eq;
    p.equations = nullptr;
    if (g.eq) {
      if (RL::IZ) eq.z = ParameterEquation{g.eq[3 * RL::EQ_Z], g.eq[3 * RL::EQ_Z + 1], g.eq[3 * RL::EQ_Z + 2]};
      if (RL::IW) eq.invw = ParameterEquation{g.eq[3 * RL::EQ_W], g.eq[3 * RL::EQ_W + 1], g.eq[3 * RL::EQ_W + 2]};
      eq.avar.q = g.eq + 3 * RL::EQ_A;
      eq.pvar.q = g.eq + 3 * RL::EQ_P;
      p.equations = &eq;
    }
    s.frags++;
    PS::drawPixel(p);
  }
};

inline swr_program make_program(uint32_t kind, const VsOps* vs, const PsOps* ps) {
  swr_program p;
  memset(&p, 0, sizeof(p));
  p.magic = SWR_PROGRAM_MAGIC;
  p.abi = SWR_PROGRAM_ABI;
  p.kind = kind;
  swr_program_layout(p.sizes);
  p.vs = vs;
  p.ps = ps;
  return p;
}

// Bytes of the allocation holding p from p to its end (device or managed memory), 0 if p
// is not in such an allocation.
inline size_t device_extent(const void* p) {
  typedef CUresult (*RangeFn)(CUdeviceptr*, size_t*, CUdeviceptr);
  static RangeFn range = nullptr;
  if (!range) {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuMemGetAddressRange", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !f) {
      cudaGetLastError();
      return 0;
    }
    range = (RangeFn)f;
  }
  CUdeviceptr base = 0;
  size_t size = 0;
  if (range(&base, &size, (CUdeviceptr)(uintptr_t)p) != CUDA_SUCCESS) return 0;
  return (size_t)(base + size - (CUdeviceptr)(uintptr_t)p);
}

// Device (or managed) memory the kernels can read in place?
inline bool on_device(const void* p) {
  cudaPointerAttributes a;
  if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  return a.type == cudaMemoryTypeDevice || a.type == cudaMemoryTypeManaged;
}

// A growable device buffer for copies of host arrays.
struct Staging {
  void* p = nullptr;
  size_t bytes = 0;
  Staging() = default;
  Staging(const Staging&) = delete;
  Staging& operator=(const Staging&) = delete;
  ~Staging() {
    if (p) cudaFree(p);
  }
  void* upload(const void* src, size_t n, cudaStream_t s) {
    if (n > bytes) {
      if (p) cudaFree(p);
      p = nullptr;
      bytes = 0;
      if (cudaMalloc(&p, n) != cudaSuccess) {
        cudaGetLastError();
        throw Error(SWR_ENOMEM, "staging a host array");
      }
      bytes = n;
    }
    check(cudaMemcpyAsync(p, src, n, cudaMemcpyHostToDevice, s) == cudaSuccess ? SWR_OK : SWR_ECUDA,
          "copying a host array to the device");
    return p;
  }
};

// Largest index of the primitives a draw uses (first index != -1), -1 if none.
inline long long max_index(const int* idx, size_t count, int per, bool skip_first_minus_one) {
  long long m = -1;
  for (size_t i = 0; i + (size_t)per <= count; i += (size_t)per) {
    if (skip_first_minus_one && idx[i] == -1) continue;
    for (int k = 0; k < per; ++k)
      if (idx[i + k] > m) m = idx[i + k];
  }
  return m;
}

}  // namespace detail

// Stage-launcher table of a shader class for the C ABI (swr_set_vertex_program /
// swr_set_pixel_program); instantiates the pipeline's kernels for it in this translation
// unit.  The table is a static of this unit.
template <class VertexShader>
const swr_program* vertex_program() {
  static const VsOps ops = make_vs<detail::UserVS<VertexShader>>();
  static const swr_program prog = detail::make_program(SWR_PROGRAM_VERTEX, &ops, nullptr);
  return &prog;
}

template <class PixelShader>
const swr_program* pixel_program() {
  static const PsOps ops = make_ps<detail::UserPS<PixelShader>>();
  static const swr_program prog = detail::make_program(SWR_PROGRAM_PIXEL, nullptr, &ops);
  return &prog;
}

// IRasterizer.h:56-71: the interface VertexProcessor hands its primitives to.
class IRasterizer {
 public:
  virtual ~IRasterizer() {}
  virtual void drawPointList(const RasterizerVertex* vertices, const int* indices, size_t indexCount) const = 0;
  virtual void drawLineList(const RasterizerVertex* vertices, const int* indices, size_t indexCount) const = 0;
  virtual void drawTriangleList(const RasterizerVertex* vertices, const int* indices, size_t indexCount) const = 0;
};

// Rasterizer.h:52-446.  Owns the GPU pipeline's context (swr_context).
class Rasterizer : public IRasterizer {
 public:
  // Rasterizer.h:67-72: Span mode, scissor (0, 0, 0, 0), NullPixelShader.
  Rasterizer() {
    detail::check(swr_create(&ctx_), "creating the pipeline context");
    setRasterMode(RasterMode::Span);
    setScissorRect(0, 0, 0, 0);
    setPixelShader<NullPixelShader>();
  }
  ~Rasterizer() override { swr_destroy(ctx_); }
  Rasterizer(const Rasterizer&) = delete;
  Rasterizer& operator=(const Rasterizer&) = delete;

  void setRasterMode(RasterMode mode) { detail::check(swr_set_raster_mode(ctx_, (int)mode), "setRasterMode"); }

  void setScissorRect(int x, int y, int width, int height) {
    sc_[0] = x;
    sc_[1] = y;
    sc_[2] = width;
    sc_[3] = height;
    detail::check(swr_set_scissor_rect(ctx_, x, y, width, height), "setScissorRect");
  }

  template <class PixelShader>
  void setPixelShader() {
    detail::check(swr_set_pixel_program(ctx_, pixel_program<PixelShader>()), "setPixelShader");
  }

  void drawPoint(const RasterizerVertex& v) const {
    const int idx[1] = {0};
    drawPointList(&v, idx, 1);
  }
  void drawLine(const RasterizerVertex& v0, const RasterizerVertex& v1) const {
    const RasterizerVertex v[2] = {v0, v1};
    const int idx[2] = {0, 1};
    drawLineList(v, idx, 2);
  }
  void drawTriangle(const RasterizerVertex& v0, const RasterizerVertex& v1, const RasterizerVertex& v2) const {
    const RasterizerVertex v[3] = {v0, v1, v2};
    const int idx[3] = {0, 1, 2};
    drawTriangleList(v, idx, 3);
  }

  // Rasterizer.h:116-141: a primitive whose first index is -1 is skipped.
  void drawPointList(const RasterizerVertex* vertices, const int* indices, size_t indexCount) const override {
    drawList(SWR_DRAW_POINT, vertices, indices, indexCount);
  }
  void drawLineList(const RasterizerVertex* vertices, const int* indices, size_t indexCount) const override {
    drawList(SWR_DRAW_LINE, vertices, indices, indexCount);
  }
  void drawTriangleList(const RasterizerVertex* vertices, const int* indices, size_t indexCount) const override {
    drawList(SWR_DRAW_TRIANGLE, vertices, indices, indexCount);
  }

  // GPU additions: the context (for the C ABI), the stream draws run on (default: the
  // legacy default stream) and the statistics of the last draw.
  swr_context* context() const { return ctx_; }
  void setStream(cudaStream_t s) { stream_ = s; }
  cudaStream_t stream() const { return stream_; }
  const swr_stats& lastStats() const { return stats_; }

  // Binds the render-target extent (see the file comment) and runs one queued draw to
  // completion: swr_finish, and a retry when a scratch queue had to grow.
  template <class Queue>
  void run(int ext_w, int ext_h, Queue queue, const char* what) const {
    SwrUniforms u;
    memset(&u, 0, sizeof(u));
    u.width = ext_w;
    u.height = ext_h;
    u.color = (void*)&stats_;  // a target key only: user pixel shaders never touch SwrUniforms
    detail::check(swr_set_uniforms(ctx_, &u), what);
    for (int attempt = 0;; ++attempt) {
      detail::check(queue(), what);
      const int rc = swr_finish(ctx_, (void*)stream_, &stats_);
      if (rc != SWR_EOVERFLOW || attempt == 3) {
        detail::check(rc, what);
        return;
      }
    }
  }

  int extentWidth() const { return sc_[0] + sc_[2] > 0 ? sc_[0] + sc_[2] : 0; }
  int extentHeight() const { return sc_[1] + sc_[3] > 0 ? sc_[1] + sc_[3] : 0; }

 private:
  void drawList(int mode, const RasterizerVertex* vertices, const int* indices, size_t count) const {
    const int per = mode == SWR_DRAW_POINT ? 1 : (mode == SWR_DRAW_LINE ? 2 : 3);
    count -= count % (size_t)per;  // the reference's loops stop at the last whole primitive
    if (!count || extentWidth() <= 0 || extentHeight() <= 0) return;
    const void* dv = vertices;
    const void* di = indices;
    size_t nverts;
    if (detail::on_device(indices)) {
      if (!detail::on_device(vertices)) throw Error(SWR_EINVAL, "host vertices need host indices");
    } else {
      di = idx_.upload(indices, count * sizeof(int), stream_);
    }
    if (detail::on_device(vertices)) {
      nverts = detail::device_extent(vertices) / sizeof(RasterizerVertex);
    } else {
      const long long m = detail::max_index(indices, count, per, true);
      if (m < 0) return;  // every primitive skipped
      nverts = (size_t)m + 1;
      dv = vtx_.upload(vertices, nverts * sizeof(RasterizerVertex), stream_);
    }
    run(extentWidth(), extentHeight(), [&] {
      return swr_draw_list(ctx_, mode, (const float*)dv, nverts, (const int32_t*)di, count, (void*)stream_);
    }, "draw list");
  }

  swr_context* ctx_ = nullptr;
  cudaStream_t stream_ = 0;
  int sc_[4] = {0, 0, 0, 0};
  mutable swr_stats stats_ = {};
  mutable detail::Staging idx_, vtx_;
  friend class VertexProcessor;
};

// VertexProcessor.h:56-151.  Draws through a Rasterizer of this header.
class VertexProcessor {
 public:
  // VertexProcessor.cpp:29-35: CullMode::CW, depth range (0, 1), DummyVertexShader.
  explicit VertexProcessor(Rasterizer* rasterizer) {
    setRasterizer(rasterizer);
    setCullMode(CullMode::CW);
    setDepthRange(0.0f, 1.0f);
    setVertexShader<DummyVertexShader>();
  }

  void setRasterizer(Rasterizer* rasterizer) {
    if (!rasterizer) throw Error(SWR_EINVAL, "setRasterizer");
    r_ = rasterizer;
  }

  void setViewport(int x, int y, int width, int height) {
    vp_[0] = x;
    vp_[1] = y;
    vp_[2] = width;
    vp_[3] = height;
  }

  void setDepthRange(float n, float f) {
    dn_ = n;
    df_ = f;
  }

  void setCullMode(CullMode mode) { cull_ = mode; }

  template <class VertexShader>
  void setVertexShader() {
    static_assert(VertexShader::AttribCount <= MaxVertexAttribs, "AttribCount <= MaxVertexAttribs");
    prog_ = vertex_program<VertexShader>();
    attribs_ = VertexShader::AttribCount;
  }

  void setVertexAttribPointer(int index, int stride, const void* buffer) {
    if (index < 0 || index >= MaxVertexAttribs) throw Error(SWR_EINVAL, "setVertexAttribPointer");
    buf_[index] = buffer;
    stride_[index] = stride;
  }

  // VertexProcessor.cpp:78-120.
  void drawElements(DrawMode mode, size_t count, int* indices) const {
    const int m = (int)mode;
    const int per = m == SWR_DRAW_POINT ? 1 : (m == SWR_DRAW_LINE ? 2 : 3);
    if (count % (size_t)per) throw Error(SWR_EINVAL, "drawElements: count is not a whole number of primitives");
    if (!count) return;
    swr_context* c = r_->ctx_;
    cudaStream_t s = r_->stream_;
    const int ew = std::max(r_->extentWidth(), vp_[0] + vp_[2]);
    const int eh = std::max(r_->extentHeight(), vp_[1] + vp_[3]);
    if (ew <= 0 || eh <= 0) return;
    detail::check(swr_set_viewport(c, vp_[0], vp_[1], vp_[2], vp_[3]), "setViewport");
    detail::check(swr_set_depth_range(c, dn_, df_), "setDepthRange");
    detail::check(swr_set_cull_mode(c, (int)cull_), "setCullMode");
    detail::check(swr_set_vertex_program(c, prog_), "setVertexShader");
    const bool dev_idx = detail::on_device(indices);
    const void* di = dev_idx ? (const void*)indices : idx_.upload(indices, count * sizeof(int), s);
    long long max_idx = -2;  // host indices: their largest value (sizes host attribute copies)
    for (int a = 0; a < attribs_; ++a) {
      const void* b = buf_[a];
      if (!b || stride_[a] <= 0) throw Error(SWR_EINVAL, "drawElements: attribute pointer not set");
      size_t bytes;
      if (detail::on_device(b)) {
        bytes = detail::device_extent(b);
      } else {
        if (dev_idx) throw Error(SWR_EINVAL, "drawElements: host attribute arrays need host indices");
        if (max_idx == -2) max_idx = detail::max_index(indices, count, 1, false);
        if (max_idx < 0) throw Error(SWR_EINDEX, "drawElements: negative index");
        bytes = ((size_t)max_idx + 1) * (size_t)stride_[a];
        b = att_[a].upload(b, bytes, s);
      }
      detail::check(swr_set_vertex_attrib_pointer(c, a, stride_[a], b, bytes), "setVertexAttribPointer");
    }
    r_->run(ew, eh, [&] { return swr_draw_elements(c, m, count, (const uint32_t*)di, (void*)s); }, "drawElements");
  }

 private:
  Rasterizer* r_ = nullptr;
  int vp_[4] = {0, 0, 0, 0};
  float dn_ = 0.0f, df_ = 1.0f;
  CullMode cull_ = CullMode::CW;
  const swr_program* prog_ = nullptr;
  int attribs_ = 0;
  const void* buf_[MaxVertexAttribs] = {};
  int stride_[MaxVertexAttribs] = {};
  mutable detail::Staging idx_, att_[MaxVertexAttribs];
};

}  // namespace swr
