// Allocation-free triangle-list draw.
//
// swr_draw_list (the IRasterizer::drawTriangleList path) keeps its scratch -- converted
// vertices, the compacted primitive list, setup records, bin pairs and their sort
// buffers, per-tile bin offsets and the status words -- in device buffers that a
// swr_context allocates with cudaMalloc and grows on demand.  Some callers cannot do
// that: an application whose device memory is owned by another allocator or capped at
// start-up, a real-time frame loop that must not stall in the driver's allocator, or a
// host plugin that is handed a stream and target buffers but no permission to allocate.
// swr_draw_triangle_list_noalloc serves them: it runs the same kernels with all scratch
// placed in one file-scope __device__ array of fixed size, so it never calls cudaMalloc,
// cudaFree or any allocating library routine.
//
// Limits (calls beyond them return SWR_EINVAL before any work is queued):
//   triangles <= 4096, vertices <= 12288, target <= 16384 tiles of 16 x 16 px (for
//   example 2048 x 2048), bin entries <= 262144 (checked on the device: the draw is then
//   skipped and SWR_EOVERFLOW returned).  The array is 8 MiB and every GPU that loads
//   the library holds it until the process exits.
//
// Set-up: the first call on a device (with that device current) looks up the array's
// device address with cudaGetSymbolAddress and caches it together with the id of the
// current CUDA context; make that first call before any stream capture.  With lazy module
// loading (the CUDA default) that first call is also when the library's device code and
// the 8 MiB array are loaded onto the device, so it is the one call that can allocate:
// a caller whose device memory is capped makes it once at start-up.  After the
// application re-creates the device's context (cudaDeviceReset), the next call sees a new
// context id and repeats the set-up.  Every call shares the one array and leaves its
// contents behind; the entry point clears what must start at zero itself.  Calls whose
// work overlaps on the GPU (different streams, or different host threads) race on the
// array: serialise them.
#include <cuda.h>  // CUcontext and CUresult only: the two driver calls are resolved at run time
#include <mutex>
#include <string.h>
#include "../../include/swr_gb300.h"
#include "swr_core.h"
#include "swr_ops.h"

namespace {

using namespace swr;

constexpr uint32_t kMaxTris = 4096;
constexpr uint32_t kMaxVerts = 12288;
constexpr uint32_t kMaxTiles = 16384;
constexpr uint32_t kMaxPairs = 1u << 18;
constexpr int kTile = 16;
constexpr int kMaxS = 16;  // post-transform vertex stride (floats) of every built-in pixel shader
constexpr int kMaxR = 64;  // setup record words
constexpr size_t kBytes = 8u << 20;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kBytes];

struct Layout {
  size_t status, draw, target, zeros, ptv, keep, pos, tris, recs, tile_count, pair_off;
  size_t keys0, vals0, keys1, vals1, tile_start, scan_scr, sort_scr, end;
};

constexpr size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

Layout make_layout() {
  Layout L;
  size_t o = 0;
  auto take = [&](size_t bytes) { const size_t at = o; o = align256(o + bytes); return at; };
  L.status = take(16 * 4);
  L.draw = take(sizeof(SwrDrawDesc));
  L.target = take(sizeof(SwrTargetDesc));
  L.zeros = take(64);
  L.ptv = take((size_t)kMaxVerts * kMaxS * 4);
  L.keep = take((size_t)kMaxTris * 4);
  L.pos = take((size_t)kMaxTris * 4);
  L.tris = take((size_t)kMaxTris * 16);
  L.recs = take((size_t)kMaxTris * kMaxR * 4);
  L.tile_count = take((size_t)kMaxTris * 4);
  L.pair_off = take((size_t)kMaxTris * 4);
  L.keys0 = take((size_t)kMaxPairs * 4);
  L.vals0 = take((size_t)kMaxPairs * 4);
  L.keys1 = take((size_t)kMaxPairs * 4);
  L.vals1 = take((size_t)kMaxPairs * 4);
  L.tile_start = take((size_t)(kMaxTiles + 1) * 4);
  L.scan_scr = take(scan_scratch_words(kMaxTris) * 4 + 128);
  L.sort_scr = take(sort_scratch_words(kMaxPairs) * 4);
  L.end = o;
  return L;
}

constexpr int kMaxDevices = 64;
std::mutex g_mutex;

// Per device: the scratch array's address and the id of the context it was looked up in.
struct DeviceSlot {
  unsigned long long ctx_id;
  unsigned char* base;
};
DeviceSlot g_slot[kMaxDevices] = {};

typedef CUresult (*CtxGetCurrentFn)(CUcontext*);
typedef CUresult (*CtxGetIdFn)(CUcontext, unsigned long long*);
CtxGetCurrentFn g_ctx_get_current = nullptr;
CtxGetIdFn g_ctx_get_id = nullptr;

// Id of the calling thread's current context (unique for the life of the process; 0 when
// no context is current yet).  Caller holds g_mutex.
int current_context_id(unsigned long long* id) {
  *id = 0;
  if (!g_ctx_get_current || !g_ctx_get_id) {
    void* f = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !f)
      return SWR_ECUDA;
    g_ctx_get_current = (CtxGetCurrentFn)f;
    f = nullptr;
    if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &f, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !f)
      return SWR_ECUDA;
    g_ctx_get_id = (CtxGetIdFn)f;
  }
  CUcontext ctx = nullptr;
  if (g_ctx_get_current(&ctx) != CUDA_SUCCESS) return SWR_ECUDA;
  if (ctx && g_ctx_get_id(ctx, id) != CUDA_SUCCESS) return SWR_ECUDA;
  return SWR_OK;
}

// Device address of the scratch array on the current device: looked up once per device
// and again whenever the current context is not the one it was looked up in.
int scratch_base(unsigned char** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    return SWR_ECUDA;
  }
  std::lock_guard<std::mutex> lock(g_mutex);
  unsigned long long id = 0;
  if (current_context_id(&id)) {
    cudaGetLastError();
    return SWR_ECUDA;
  }
  DeviceSlot& slot = g_slot[dev];
  if (!slot.base || !id || id != slot.ctx_id) {
    void* p = nullptr;
    // makes the device's primary context current when no context was yet
    if (cudaGetSymbolAddress(&p, g_noalloc_scratch) != cudaSuccess || !p) {
      cudaGetLastError();
      return SWR_ECUDA;
    }
    if (current_context_id(&id) || !id) {
      cudaGetLastError();
      return SWR_ECUDA;
    }
    slot.base = (unsigned char*)p;
    slot.ctx_id = id;
  }
  *out = slot.base;
  return SWR_OK;
}

}  // namespace

extern "C" int swr_draw_triangle_list_noalloc(const struct SwrUniforms* u, int ps_id, int raster_mode,
                                              int sc_x, int sc_y, int sc_w, int sc_h,
                                              const float* vertices, uint64_t nverts,
                                              const int32_t* indices, uint64_t count, void* stream,
                                              uint64_t* fragments) {
  const PsOps* ps = ps_ops(ps_id);
  if (!u || !ps || raster_mode < 0 || raster_mode > 2 || u->width <= 0 || u->height <= 0 || !u->color)
    return SWR_EINVAL;
  if (count % 3 || count / 3 > kMaxTris || nverts > kMaxVerts) return SWR_EINVAL;
  if ((count && !indices) || (nverts && !vertices)) return SWR_EINVAL;
  if (ps->S > kMaxS || ps->R > kMaxR) return SWR_EINVAL;
  const int tiles_x = (u->width + kTile - 1) / kTile, tiles_y = (u->height + kTile - 1) / kTile;
  if ((uint64_t)tiles_x * (uint64_t)tiles_y > kMaxTiles) return SWR_EINVAL;
  const Layout L = make_layout();
  if (L.end > kBytes) return SWR_EINVAL;
  unsigned char* base = nullptr;
  int rc = scratch_base(&base);
  if (rc) return rc;
  cudaStream_t s = (cudaStream_t)stream;
  const uint32_t nsub = (uint32_t)(count / 3);
  const uint32_t ntiles = (uint32_t)(tiles_x * tiles_y);

  SwrDrawDesc D;
  memset(&D, 0, sizeof(D));
  D.direct = 1;
  D.draw_mode = SWR_DRAW_TRIANGLE;
  D.raster_mode = raster_mode;
  D.sc_minx = sc_x;
  D.sc_miny = sc_y;
  D.sc_maxx = sc_x + sc_w;
  D.sc_maxy = sc_y + sc_h;
  D.nprims = nsub;
  D.nverts = (uint32_t)nverts;
  D.u = *u;
  SwrTargetDesc T;
  memset(&T, 0, sizeof(T));
  T.width = u->width;
  T.height = u->height;
  T.tiles_x = tiles_x;
  T.tiles_y = tiles_y;

  uint32_t* st = (uint32_t*)(base + L.status);
  SwrDrawDesc* dd = (SwrDrawDesc*)(base + L.draw);
  SwrTargetDesc* dt = (SwrTargetDesc*)(base + L.target);
  uint32_t* zeros = (uint32_t*)(base + L.zeros);
  float* ptv = (float*)(base + L.ptv);
  uint32_t* keep = (uint32_t*)(base + L.keep);
  uint32_t* pos = (uint32_t*)(base + L.pos);
  uint4* tris = (uint4*)(base + L.tris);
  float* recs = (float*)(base + L.recs);
  uint32_t* tile_count = (uint32_t*)(base + L.tile_count);
  uint32_t* pair_off = (uint32_t*)(base + L.pair_off);
  uint32_t* k0 = (uint32_t*)(base + L.keys0);
  uint32_t* v0 = (uint32_t*)(base + L.vals0);
  uint32_t* k1 = (uint32_t*)(base + L.keys1);
  uint32_t* v1 = (uint32_t*)(base + L.vals1);
  uint32_t* tile_start = (uint32_t*)(base + L.tile_start);
  uint32_t* scan_scr = (uint32_t*)(base + L.scan_scr);
  uint32_t* sort_scr = (uint32_t*)(base + L.sort_scr);

  // The previous call's contents stay in the array: reset the status words, the primitive
  // count and the per-target lookup words before any kernel reads them.
  cudaMemsetAsync(st, 0, 16 * 4, s);
  cudaMemsetAsync(zeros, 0, 64, s);
  cudaMemcpyAsync(dd, &D, sizeof(D), cudaMemcpyHostToDevice, s);
  cudaMemcpyAsync(dt, &T, sizeof(T), cudaMemcpyHostToDevice, s);
  if ((rc = (cudaGetLastError() == cudaSuccess ? SWR_OK : SWR_ECUDA))) return rc;

  ps->direct_vertices(vertices, (uint32_t)nverts, ptv, s);
  if (nsub) {
    const int grid = (int)((nsub + 255) / 256);
    k_direct_flags<<<grid, 256, 0, s>>>(indices, nsub, 3, keep);
    scan_exclusive(keep, pos, nullptr, nsub, st + SWR_ST_PRIMS, scan_scr, s);
    k_direct_emit<<<grid, 256, 0, s>>>(indices, nsub, 3, (uint32_t)nverts, keep, pos, tris, st);
  }
  SetupArgs sa;
  memset(&sa, 0, sizeof(sa));  // no cell counting: this path bins with the radix sort
  sa.tris = tris;
  sa.status = st;
  sa.cap_prims = kMaxTris;
  sa.ptv = ptv;
  sa.clipv = ptv;  // no clipping on the direct path
  sa.S = ps->S;
  sa.off_a = 8;
  sa.off_p = 8 + ps->A;
  sa.vs_a = ps->A;
  sa.vs_p = ps->P;
  sa.draws = dd;
  sa.targets = dt;
  sa.recs = recs;
  sa.tile_count = tile_count;
  sa.tile = kTile;
  ps->setup(sa, s);
  scan_exclusive(tile_count, pair_off, st + SWR_ST_PRIMS, kMaxTris, st + SWR_ST_PAIRS, scan_scr, s);
  ps->emit_pairs(st, kMaxTris, recs, tile_count, pair_off, st + SWR_ST_PAIRS, kMaxPairs, dd, dt, kTile, k0, v0,
                 st, s);
  int bits = 0;
  while (bits < 32 && (1ull << bits) < (uint64_t)ntiles) ++bits;
  const int which = radix_sort_pairs(k0, v0, k1, v1, st + SWR_ST_PAIRS, kMaxPairs, bits, sort_scr, s);
  uint32_t* keys = which ? k1 : k0;
  uint32_t* vals = which ? v1 : v0;
  segment_starts(keys, st + SWR_ST_PAIRS, kMaxPairs, ntiles, tile_start, s);
  RasterArgs ra;
  ra.status = st;
  ra.tile_start = tile_start;
  ra.tile_stride = 1;
  ra.bin = vals;
  ra.bin_raw = nullptr;  // the radix sort already ordered every tile
  ra.recs = recs;
  ra.draws = dd;
  ra.targets = dt;
  ra.target_tile_base = zeros;
  ra.ntargets = 1;
  ra.draw_prim_base = nullptr;
  ra.status_w = st;
  ra.ntiles = ntiles;
  ra.has_span = raster_mode != SWR_RASTER_BLOCK;
  ra.slices = 1;  // no slice buffer without allocation
  ra.slice_state = nullptr;
  ra.quad_flag = nullptr;  // no heavy-tile quadrant CTAs: every tile is one CTA
  ra.quad_tiles = nullptr;
  ra.quad_count = nullptr;
  ra.quad_cap = 0;
  ra.quad_all = 0;
  ra.dslice = 0;  // no heavy-tile runs: they need the runs' State buffer
  ra.dslice_state = nullptr;
  ra.dslice_done = nullptr;
  ps->raster(ra, ntiles, kTile, s);
  if (cudaGetLastError() != cudaSuccess) return SWR_ECUDA;  // a launch failed: the status words are stale
  uint32_t h[16];
  if (cudaMemcpyAsync(h, st, sizeof(h), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
      cudaStreamSynchronize(s) != cudaSuccess) {
    cudaGetLastError();
    return SWR_ECUDA;
  }
  if (fragments) *fragments = (uint64_t)h[SWR_ST_SHADED_LO] | ((uint64_t)h[SWR_ST_SHADED_HI] << 32);
  if (h[SWR_ST_FLAGS] & SWR_F_ANY_OVERFLOW) return SWR_EOVERFLOW;
  if (h[SWR_ST_FLAGS] & SWR_F_BAD_INDEX) return SWR_EINDEX;
  return SWR_OK;
}
