// Test infrastructure: drives the unmodified reference library (trenki2/SoftwareRenderer
// src/renderer, compiled from its own sources by oracle/Makefile with OpenMP, as the
// reference's own build does when OpenMP is found) through the same
// oracle_draw() entry point as the CPU port, using the shared shader programs of
// swr_programs.h wrapped in the reference's VertexShaderBase / PixelShaderBase.
// Used to generate the golden fixtures under tests/golden and to pin the port.
#include <stdint.h>
#include <string.h>
#include <vector>
#include <memory>
#include <omp.h>
#include "Renderer.h"  // reference umbrella header (src/renderer/Renderer.h)
#include "Texture.h"   // the reference's example texture (src/examples/Texture.h) over sdl_shim/SDL.h
#include "oracle_abi.h"

namespace swr {
// The shared shaders ask for derivatives through swr_persp_deriv (argument-dependent
// lookup): here it is the reference's own PixelData::computePerspectiveDerivatives.
inline void swr_persp_deriv(const PixelData& p, int i, float& ddx, float& ddy) {
  p.computePerspectiveDerivatives(*p.equations, i, ddx, ddy);
}
}  // namespace swr

namespace {

const SwrUniforms* g_u = nullptr;  // the reference keeps shader parameters in statics
int g_prim = 0;

// Fragment counters per OpenMP thread (the reference calls drawPixel from its OpenMP teams
// for distinct pixels of one primitive), summed after the draw.
struct alignas(64) Counters {
  uint64_t frags, outside;
};
constexpr int kMaxThreads = 512;
Counters g_count[kMaxThreads];

inline Counters& counters() { return g_count[omp_get_thread_num() & (kMaxThreads - 1)]; }

template <class P>
struct RefPS : public swr::PixelShaderBase<RefPS<P>> {
  static const int AVarCount = P::AVarCount;
  static const int PVarCount = P::PVarCount;
  static const int InterpolateZ = P::InterpolateZ;
  static const int InterpolateW = P::InterpolateW;
  static void drawPixel(const swr::PixelData& p) {
    if (p.x < 0 || p.y < 0 || p.x >= g_u->width || p.y >= g_u->height) {
      counters().outside++;
      return;
    }
    typename P::State s;
    P::load(s, p.x, p.y, *g_u);
    P::drawPixel(p, g_prim, s, *g_u);
    P::store(s, p.x, p.y, *g_u);
    counters().frags++;
  }
};

// The mip-mapped textured shader of the reference's Box example (Box.cpp:38-61) with the
// reference's own sampler: Texture::sample over the chain Texture::generateMipmaps builds
// from the level-0 image (src/examples/Texture.h:35-293), derivatives from
// PixelData::computePerspectiveDerivatives.  Every fragment overwrites the pixel, recorded
// through PsTexMip's State like every other shader here.
std::unique_ptr<swr::Texture> g_texture;

struct RefTexMipPS : public swr::PixelShaderBase<RefTexMipPS> {
  static const int AVarCount = PsTexMip::AVarCount;
  static const int PVarCount = PsTexMip::PVarCount;
  static const int InterpolateZ = PsTexMip::InterpolateZ;
  static const int InterpolateW = PsTexMip::InterpolateW;
  static void drawPixel(const swr::PixelData& p) {
    if (p.x < 0 || p.y < 0 || p.x >= g_u->width || p.y >= g_u->height) {
      counters().outside++;
      return;
    }
    float dudx, dudy, dvdx, dvdy;
    p.computePerspectiveDerivatives(*p.equations, 0, dudx, dudy);
    p.computePerspectiveDerivatives(*p.equations, 1, dvdx, dvdy);
    Uint32 c = 0;
    g_texture->sample(p.pvar[0], p.pvar[1], dudx, dvdx, dudy, dvdy, c);
    PsTexMip::State s;
    PsTexMip::load(s, p.x, p.y, *g_u);
    PsTexMip::apply(s, 0.0f, c, g_prim);
    PsTexMip::store(s, p.x, p.y, *g_u);
    counters().frags++;
  }
};

// swr::Texture from the level-0 image of SwrUniforms.tex (0x00RRGGBB texels).
bool make_reference_texture(const SwrUniforms& u) {
  SDL_Surface* base = SDL_CreateRGBSurface(0, u.tex_w, u.tex_h, 32, 0x00FF0000, 0x0000FF00, 0x000000FF, 0);
  if (!base || !u.tex) return false;
  memcpy(base->pixels, u.tex, (size_t)u.tex_w * (size_t)u.tex_h * 4);
  g_texture.reset(new swr::Texture(base, u.max_aniso > 0 ? u.max_aniso : 8));
  SDL_FreeSurface(base);
  return true;
}

template <class V>
struct RefVS : public swr::VertexShaderBase<RefVS<V>> {
  static const int AttribCount = V::AttribCount;
  static const int AVarCount = V::AVarCount;
  static const int PVarCount = V::PVarCount;
  static void processVertex(swr::VertexShaderInput in, swr::VertexShaderOutput* out) {
    SwrVertexInput vi;
    for (int i = 0; i < V::AttribCount; ++i) vi.p[i] = in[i];
    V::processVertex(vi, out, *g_u);
  }
};

// IRasterizer that numbers the primitives it forwards (the same loops as
// Rasterizer::draw*List) so the pixel shader can record which primitive wrote a pixel.
class NumberingRasterizer : public swr::IRasterizer {
 public:
  explicit NumberingRasterizer(swr::Rasterizer* r) : r_(r) {}
  mutable uint64_t prims = 0;
  void drawPointList(const swr::RasterizerVertex* v, const int* idx, size_t n) const override {
    for (size_t i = 0; i < n; ++i) {
      if (idx[i] == -1) continue;
      g_prim = (int)prims++;
      r_->drawPoint(v[idx[i]]);
    }
  }
  void drawLineList(const swr::RasterizerVertex* v, const int* idx, size_t n) const override {
    for (size_t i = 0; i + 2 <= n; i += 2) {
      if (idx[i] == -1) continue;
      g_prim = (int)prims++;
      r_->drawLine(v[idx[i]], v[idx[i + 1]]);
    }
  }
  void drawTriangleList(const swr::RasterizerVertex* v, const int* idx, size_t n) const override {
    for (size_t i = 0; i + 3 <= n; i += 3) {
      if (idx[i] == -1) continue;
      g_prim = (int)prims++;
      r_->drawTriangle(v[idx[i]], v[idx[i + 1]], v[idx[i + 2]]);
    }
  }

 private:
  swr::Rasterizer* r_;
};

template <class V>
void set_vs(swr::VertexProcessor& vp) {
  vp.setVertexShader<RefVS<V>>();
}

template <class P>
void set_ps(swr::Rasterizer& r) {
  r.setPixelShader<RefPS<P>>();
}

}  // namespace

extern "C" int oracle_draw(const OracleDraw* d, OracleStats* st) {
  if (!d || !d->uniforms) return 1;
  const uint64_t per = d->draw_mode == 0 ? 1 : (d->draw_mode == 1 ? 2 : 3);
  if (d->draw_mode < 0 || d->draw_mode > 2 || d->count % per) return 1;
  for (uint64_t i = 0; i < d->count; ++i)
    if (d->indices[i] < (d->raster_vertices ? -1 : 0)) return 1;
  g_u = d->uniforms;
  memset(g_count, 0, sizeof(g_count));
  g_prim = 0;
  if (d->threads > 0) omp_set_num_threads(d->threads);

  swr::Rasterizer r;
  r.setRasterMode(d->raster_mode == 0 ? swr::RasterMode::Span
                  : d->raster_mode == 1 ? swr::RasterMode::Block
                                        : swr::RasterMode::Adaptive);
  r.setScissorRect(d->scissor[0], d->scissor[1], d->scissor[2], d->scissor[3]);
  switch (d->ps_id) {
    case SWR_PS_TEX_NEAREST: set_ps<PsTexNearest>(r); break;
    case SWR_PS_LAMBERT: set_ps<PsLambert>(r); break;
    case SWR_PS_VCOLOR: set_ps<PsVColor>(r); break;
    case SWR_PS_VCOLOR_AFFINE: set_ps<PsVColorAffine>(r); break;
    case SWR_PS_LAMBERT_TEX: set_ps<PsLambertTex>(r); break;
    case SWR_PS_DIFF: set_ps<PsDiff>(r); break;
    // equations are set only for triangles (points and lines would dereference null)
    case SWR_PS_TEX_MIP:
      if (d->draw_mode != 2 || !make_reference_texture(*d->uniforms)) return 1;
      r.setPixelShader<RefTexMipPS>();
      break;
    case SWR_PS_PERSP_DERIV: if (d->draw_mode != 2) return 1; set_ps<PsPerspDeriv>(r); break;
    default: return 2;
  }
  NumberingRasterizer nr(&r);
  // The reference flushes a batch every 1024 primitives plus once at the end
  // (VertexProcessor.cpp:110-119); counted here for comparison with the port.
  const uint64_t batches = d->raster_vertices ? 0 : d->count / per / 1024 + 1;
  if (d->raster_vertices) {
    int maxi = -1;
    for (uint64_t i = 0; i < d->count; ++i) maxi = d->indices[i] > maxi ? d->indices[i] : maxi;
    std::vector<swr::RasterizerVertex> v((size_t)(maxi + 1));
    if (maxi >= 0) memcpy(v.data(), d->raster_vertices, v.size() * sizeof(swr::RasterizerVertex));
    if (d->draw_mode == 0) nr.drawPointList(v.data(), d->indices, d->count);
    else if (d->draw_mode == 1) nr.drawLineList(v.data(), d->indices, d->count);
    else nr.drawTriangleList(v.data(), d->indices, d->count);
  } else {
    swr::VertexProcessor vp(&nr);
    vp.setViewport(d->viewport[0], d->viewport[1], d->viewport[2], d->viewport[3]);
    vp.setDepthRange(d->depth_range[0], d->depth_range[1]);
    vp.setCullMode(d->cull_mode == 0 ? swr::CullMode::None
                   : d->cull_mode == 1 ? swr::CullMode::CCW
                                       : swr::CullMode::CW);
    switch (d->vs_id) {
      case SWR_VS_POS_UV: set_vs<VsPosUV>(vp); break;
      case SWR_VS_POS_NRM_UV: set_vs<VsPosNrmUV>(vp); break;
      case SWR_VS_POS_RGB: set_vs<VsPosRGB>(vp); break;
      case SWR_VS_POS_RGB_AFFINE: set_vs<VsPosRGBAffine>(vp); break;
      case SWR_VS_POS_RGB_UV: set_vs<VsPosRGBUV>(vp); break;
      default: return 2;
    }
    for (int a = 0; a < 8; ++a)
      if (d->attrib[a]) vp.setVertexAttribPointer(a, d->attrib_stride[a], d->attrib[a]);
    vp.drawElements(swr::DrawMode(d->draw_mode == 0 ? swr::DrawMode::Point
                                  : d->draw_mode == 1 ? swr::DrawMode::Line
                                                      : swr::DrawMode::Triangle),
                    (size_t)d->count, const_cast<int*>(d->indices));
  }
  if (st) {
    st->fragments = st->outside = 0;
    for (const Counters& c : g_count) {
      st->fragments += c.frags;
      st->outside += c.outside;
    }
    st->primitives = nr.prims;
    st->batches = batches;
  }
  return 0;
}

extern "C" float oracle_fold(float v, float a, int k) { return swr_fold(v, a, k); }

// The reference examples' Random (src/examples/Random.cpp, the generator Benchmark.cpp
// draws its vertices from): n values of NextDouble() for `seed`.
#include "Random.h"
extern "C" void oracle_ref_random(int seed, uint64_t n, double* out) {
  Random r(seed);
  for (uint64_t i = 0; i < n; ++i) out[i] = r.NextDouble();
}

// The examples' OBJ loader (src/examples/ObjData.cpp): loadFromFile + toVertexArray.
// Returns the vertex and index counts; copies at most the given capacities.
#include "ObjData.h"
extern "C" int oracle_ref_obj(const char* path, float* vdata, uint64_t vcap, int32_t* idata, uint64_t icap,
                              uint64_t* nverts, uint64_t* nidx) {
  std::vector<ObjData::VertexArrayData> vd;
  std::vector<int> id;
  ObjData::loadFromFile(path).toVertexArray(vd, id);
  static_assert(sizeof(ObjData::VertexArrayData) == 32, "8 floats per vertex");
  *nverts = vd.size();
  *nidx = id.size();
  if (vdata) memcpy(vdata, vd.data(), 32 * (vd.size() < vcap ? vd.size() : vcap));
  for (size_t i = 0; idata && i < id.size() && i < icap; ++i) idata[i] = id[i];
  return 0;
}

// The reference's own sampler (src/examples/Texture.h): Texture::generateMipmaps on the
// level-0 image `base` (w x h, 0x00RRGGBB), then Texture::sample for n records
// {u, v, dudx, dvdx, dudy, dvdy} of q.  `chain` (may be NULL) receives every level of the
// mip chain, level 0 first.  Returns the number of levels.
extern "C" int oracle_ref_tex_sample(const uint32_t* base, int w, int h, int max_aniso, const float* q, uint32_t* out,
                                     uint64_t n, uint32_t* chain) {
  SwrUniforms u;
  memset(&u, 0, sizeof(u));
  u.tex = base;
  u.tex_w = w;
  u.tex_h = h;
  u.max_aniso = max_aniso;
  if (!make_reference_texture(u)) return -1;
  for (uint64_t i = 0; i < n; ++i) {
    const float* r = q + 6 * i;
    Uint32 c = 0;
    g_texture->sample(r[0], r[1], r[2], r[3], r[4], r[5], c);
    out[i] = c;
  }
  // The chain Texture::generateMipmaps built (Texture.h:220-293), level 0 first, read
  // through a view of Texture's two data members (its mip vector is private).
  int levels = 0;
  if (chain) {
    struct View {
      std::vector<SDL_Surface*> mips;
      int max_aniso;
    };
    static_assert(sizeof(swr::Texture) == sizeof(View), "Texture holds a vector<SDL_Surface*> and an int");
    const View* v = reinterpret_cast<const View*>(g_texture.get());
    size_t off = 0;
    for (SDL_Surface* m : v->mips) {
      memcpy(chain + off, m->pixels, (size_t)m->w * (size_t)m->h * 4);
      off += (size_t)m->w * (size_t)m->h;
      ++levels;
    }
  }
  return levels;
}
