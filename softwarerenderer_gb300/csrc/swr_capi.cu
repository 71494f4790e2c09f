// C ABI and draw orchestration: the host side of VertexProcessor::drawElements and
// Rasterizer::draw*List for the GPU pipeline.  One draw is a fixed sequence of kernels on
// one stream whose variable sizes (clip output, primitives, bin pairs) stay on the
// device; overflow of a scratch queue is detected on the device, skips the raster stage
// and is reported by swr_finish, which grows the queue for the next attempt.
#include <algorithm>
#include <stdio.h>
#include <string.h>
#include <vector>
#include "../../include/swr_gb300.h"
#include "swr_context.h"
#include "swr_core.h"
#include "swr_ops.h"

namespace swr {

// Status buffer: words [0, SWR_ST_WORDS) as in swr_device.cuh; words 9..13 hold the
// largest per-draw requests (words 1..5) seen since the last finish; words 14-15 count
// colour writes.
constexpr int kStatusWords = 16;
constexpr int kSingleSlots = 8;            // pinned descriptor slots of single draws
constexpr int kBatchSlots = 2;             // pinned descriptor slots (and cached graphs) of batches
constexpr size_t kSingleSlotBytes = 1024;  // >= sizeof(SwrDrawDesc) + sizeof(SwrTargetDesc)
constexpr size_t kBigSortSmem = 128 * 1024;  // shared memory of a k_sort_big CTA (bounds one warp's bitmap)
constexpr int kBigSortWarps = 1216;          // warps of k_sort_big (8 per SM)
constexpr int kStickyBase = SWR_ST_STICKY;
constexpr uint32_t kQuadMin = 3 * SWR_CHUNK;  // bin entries above which a 16-px tile is split into quadrant CTAs

// Tiles k_sort_cells may list for quadrant CTAs: enough to cover the slow tail of a frame
// whose heavy tiles are few; every listed tile adds three CTAs.
uint32_t quad_cap(uint32_t ntiles) {
  uint32_t cap = ntiles / 8;
  cap = cap < 152 ? 152 : (cap > 1024 ? 1024 : cap);
  return cap < ntiles ? cap : ntiles;
}

// Tiles k_sort_cells may list for heavy-tile runs (depth-min shaders): every slot adds
// SWR_DSLICES CTAs at the front of the raster grid, used or not.  On the dense 1080p mesh
// (about 350 tiles of more than one chunk) 512 slots measured 0.9 % faster than 1020 and
// 304 slots 7 % slower (heavy tiles left whole).
uint32_t slice_cap(uint32_t ntiles) {
  const uint32_t cap = quad_cap(ntiles);
  return cap < 512 ? cap : 512;
}

// Descriptor upload from pinned host staging (device-accessible under unified addressing)
// by a kernel rather than cudaMemcpyAsync: a copy-engine transfer would queue behind any
// large host<->device copy the application runs on another stream, delaying the draw.
// The same kernel zeroes the draw's small per-draw words (counters, single-draw bases, the
// heavy-tile list's length), which as separate memsets would each be one more operation (a
// graph node, and a break in the kernels' programmatic dependent launches) ahead of the draw.
struct StageCopy {
  void* dst[6];
  const void* src[6];
  uint32_t words[6];
  int n = 0;
  uint32_t* zero[6];
  uint32_t zero_words[6];
  int nz = 0;
  void add(void* d, const void* s, size_t bytes) {
    dst[n] = d;
    src[n] = s;
    words[n] = (uint32_t)(bytes / 4);
    ++n;
  }
  void clear(void* d, size_t bytes) {
    zero[nz] = (uint32_t*)d;
    zero_words[nz] = (uint32_t)(bytes / 4);
    ++nz;
  }
};
constexpr int kStageCopyBlocks = 8;
static_assert(sizeof(SwrDrawDesc) % 4 == 0 && sizeof(SwrTargetDesc) % 4 == 0, "descriptors copy as words");

__global__ void k_stage_copy(const StageCopy sc) {
  swr_pdl_entry();
  if (blockIdx.x == 0)
    for (int k = 0; k < sc.nz; ++k)
      for (uint32_t i = threadIdx.x; i < sc.zero_words[k]; i += blockDim.x) sc.zero[k][i] = 0u;
  for (int k = 0; k < sc.n; ++k) {
    const uint32_t* s = (const uint32_t*)sc.src[k];
    uint32_t* d = (uint32_t*)sc.dst[k];
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < sc.words[k]; i += gridDim.x * blockDim.x) d[i] = s[i];
  }
}

__global__ void k_close_draw(uint32_t* st) {
  swr_pdl_entry();
  swr_close_status(st);
}

// Device bytes a context holds, and the cap swr_set_memory_limit puts on them (0: none).
struct MemBudget {
  size_t used = 0;
  size_t limit = 0;
};

struct Buffer {
  void* p = nullptr;
  size_t bytes = 0;
  MemBudget* budget = nullptr;
  ~Buffer() {
    if (p) cudaFree(p);
  }
  bool ensure(size_t n) {
    if (n <= bytes) return true;
    size_t want = n + n / 4;
    // over the context's budget: fail like an allocation failure, keeping the old buffer
    if (budget && budget->limit && budget->used - bytes + want > budget->limit) return false;
    if (p) cudaFree(p);
    if (budget) budget->used -= bytes;
    p = nullptr;
    bytes = 0;
    if (cudaMalloc(&p, want) != cudaSuccess) {
      cudaGetLastError();
      return false;
    }
    bytes = want;
    if (budget) budget->used += want;
    return true;
  }
  template <class T>
  T* as() const {
    return (T*)p;
  }
};

struct Attrib {
  const void* ptr = nullptr;
  int stride = 0;
  uint64_t bytes = 0;
};

}  // namespace swr

struct swr_context {
  // VertexProcessor state
  int vp_x = 0, vp_y = 0, vp_w = 0, vp_h = 0;
  float dn = 0.0f, df = 1.0f;
  int cull = SWR_CULL_CW;
  int vs_id = 0;
  const swr::VsOps* vs_cur = nullptr;  // set by swr_set_vertex_shader or swr_set_vertex_program
  swr::Attrib attribs[8];
  // Rasterizer state
  int raster_mode = SWR_RASTER_SPAN;
  int sc_x = 0, sc_y = 0, sc_w = 0, sc_h = 0;
  int ps_id = 0;
  const swr::PsOps* ps_cur = nullptr;  // set by swr_set_pixel_shader or swr_set_pixel_program
  SwrUniforms u;
  bool have_u = false;
  int tile = 16;
  // capacities of the device-sized queues
  uint32_t cap_prims = 0, cap_clip_slots = 0, cap_clip_verts = 0, cap_pairs = 0;
  // device buffers
  swr::Buffer draws, targets, draw_vbase, draw_bbase, target_tile_base;
  swr::Buffer ptv, clipv, clip_table, clip_slot, tri_flags, batch_counts, batch_base;
  swr::Buffer tris, recs, tile_count, pair_off, keys0, vals0, keys1, vals1, tile_start;
  swr::Buffer scratch, status, direct_keep, direct_pos, lp_refs, cell_count, cell_start, draw_pbase;
  swr::Buffer big_cells;  // k_sort_cells -> k_sort_big: [count, cell ids...]
  swr::Buffer quad_flag, quad_tiles, quad_count;  // heavy 16-px tiles rasterized as four quadrant CTAs
  int quad_mode = 0;  // 0: off, 1: heavy tiles (more than kQuadMin entries), 2: every tile (8-px raster tiles)
  bool persistent_geometry = false;  // swr_set_persistent_geometry
  bool geo_stall = false;             // swr_test_stall_geometry_barrier
  swr::Buffer geo_bar;                // its grid barrier's two words
  swr::Buffer slice_state;  // overwrite shaders: per (tile, slice, pixel) State of sliced tiles
  int slices = 1;           // slices the buffer holds for the current tile count
  // depth-min shaders: heavy tiles rasterized in SWR_DSLICES runs (swr_set_tile_slicing)
  swr::Buffer dslice_state, dslice_done;
  int dslice_chunks = -1;  // tiles of more than this many raster chunks (-1: the shader's default)
  bool dslice_ok = false;  // the buffers hold the current tile count's runs
  bool use_draw_pbase = false;  // set while queuing drawElements / batch draws
  int32_t* prim_src = nullptr;  // swr_set_primitive_source
  uint64_t prim_src_cap = 0;
  uint32_t* status_host = nullptr;
  uint32_t last_ntiles = 0;
  // swr_set_queue_capacity: queues sized by the caller are not grown ahead of a draw (only
  // after a draw overflowed them); swr_set_memory_limit caps the device bytes held
  bool fixed_prims = false, fixed_pairs = false;
  swr::MemBudget budget;
  // tracing: CUDA events at the stage boundaries of every draw since the last
  // swr_stage_times call (swr_set_profiling); sextuples reused from a pool
  bool profiling = false;
  std::vector<cudaEvent_t> ev_pool;
  size_t ev_used = 0;  // events recorded (multiple of 6 after a complete draw)
  uint64_t launches = 0;  // kernels launched since the last swr_finish
  // batched submissions: pinned staging of the descriptor arrays, and the CUDA graph of
  // the last batch layout
  unsigned char* stage = nullptr;
  size_t stage_bytes = 0;
  unsigned char* single_stage = nullptr;  // pinned ring of single-draw descriptor slots
  cudaEvent_t single_ev[swr::kSingleSlots] = {};
  bool single_pending[swr::kSingleSlots] = {};
  int single_next = 0;
  int single_cur = -1;               // the slot of the single draw being queued
  // batch descriptors: kBatchSlots pinned staging slots used in turn, each with the event
  // recorded after the last draw that read it and the CUDA graph captured over it
  int stage_next = 0;
  cudaEvent_t stage_ev[swr::kBatchSlots] = {};
  bool stage_pending[swr::kBatchSlots] = {};
  bool graph_mode = false;
  bool capturing = false;
  cudaGraphExec_t gexec[swr::kBatchSlots] = {};
  cudaStream_t cap_stream = nullptr;  // graphs are recorded here, then launched on the caller's stream
  uint64_t gsig[swr::kBatchSlots] = {};
  uint64_t glaunches[swr::kBatchSlots] = {};  // kernels per replay of each cached graph

  void attach_budget() {
    swr::Buffer* all[] = {&draws, &targets, &draw_vbase, &draw_bbase, &target_tile_base, &ptv, &clipv,
                          &clip_table, &clip_slot, &tri_flags, &batch_counts, &batch_base, &tris, &recs,
                          &tile_count, &pair_off, &keys0, &vals0, &keys1, &vals1, &tile_start, &scratch,
                          &status, &direct_keep, &direct_pos, &lp_refs, &cell_count, &cell_start, &draw_pbase,
                          &big_cells, &slice_state, &quad_flag, &quad_tiles, &quad_count, &geo_bar,
                          &dslice_state, &dslice_done};
    for (swr::Buffer* b : all) b->budget = &budget;
  }
};

namespace {

using namespace swr;

int cuda_err_at(cudaError_t e, int line) {
  if (e == cudaSuccess) return SWR_OK;
  fprintf(stderr, "swr_gb300: CUDA error %s (swr_capi.cu:%d)\n", cudaGetErrorString(e), line);
  return e == cudaErrorMemoryAllocation ? SWR_ENOMEM : SWR_ECUDA;
}
#define cuda_err(e) cuda_err_at((e), __LINE__)

void mark(swr_context* c, int i, cudaStream_t s) {
  if (!c->profiling || c->capturing) return;
  if (i == 0) c->ev_used = (c->ev_used + 5) / 6 * 6;  // start a new sextuple
  const size_t k = c->ev_used;
  if (k >= c->ev_pool.size()) {
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) { c->profiling = false; return; }
    c->ev_pool.push_back(e);
  }
  cudaEventRecord(c->ev_pool[k], s);
  c->ev_used = k + 1;
}

int bits_for(uint32_t n) {
  int b = 0;
  while (b < 32 && (1ull << b) < (uint64_t)n) ++b;
  return b;
}

bool grow_u32(uint32_t& cap, uint64_t need) {
  if (need <= cap) return true;
  uint64_t c = need + need / 4 + 1024;
  if (c > 0xffffffffull) return false;
  cap = (uint32_t)c;
  return true;
}

// Allocates every queue a draw with the given host-known sizes needs.
int ensure_capacity(swr_context* c, uint32_t nverts_ptv, int S, uint32_t nsub, uint32_t nbatches,
                    uint32_t ntiles, int R, const PsOps* ps) {
  if (!c->fixed_prims) grow_u32(c->cap_prims, (uint64_t)nsub + 1024);
  grow_u32(c->cap_clip_slots, (uint64_t)nsub / 16 + 1024);
  grow_u32(c->cap_clip_verts, (uint64_t)c->cap_clip_slots * 4);
  if (!c->fixed_pairs) grow_u32(c->cap_pairs, (uint64_t)c->cap_prims * 2 + 65536);
  bool ok = true;
  ok &= c->ptv.ensure((size_t)nverts_ptv * S * 4 + 16);
  ok &= c->clipv.ensure((size_t)c->cap_clip_verts * S * 4 + 16);
  ok &= c->clip_table.ensure((size_t)c->cap_clip_slots * sizeof(SwrClipEntry) + 16);
  ok &= c->clip_slot.ensure((size_t)nsub * 4 + 16);
  ok &= c->tri_flags.ensure((size_t)nsub + 16);
  ok &= c->lp_refs.ensure((size_t)nsub * 8 + 16);
  ok &= c->batch_counts.ensure((size_t)nbatches * 16 + 16);  // per half batch (points/lines: per batch)
  ok &= c->batch_base.ensure((size_t)nbatches * 4 + 16);
  ok &= c->tris.ensure((size_t)c->cap_prims * 16 + 16);
  ok &= c->recs.ensure((size_t)c->cap_prims * R * 4 + 16);
  ok &= c->tile_count.ensure((size_t)c->cap_prims * 4 + 16);
  ok &= c->pair_off.ensure((size_t)c->cap_prims * 4 + 16);
  ok &= c->keys0.ensure((size_t)c->cap_pairs * 4 + 16);
  ok &= c->vals0.ensure((size_t)c->cap_pairs * 4 + 16);
  ok &= c->keys1.ensure((size_t)c->cap_pairs * 4 + 16);
  ok &= c->vals1.ensure((size_t)c->cap_pairs * 4 + 16);
  ok &= c->tile_start.ensure((size_t)(ntiles + 1) * 4 + 16);
  if (c->cell_count.bytes < (size_t)ntiles * SWR_SEGS * 4 + 16) {
    // the per-cell counters start at zero and every draw leaves them at zero (k_fill_bins)
    ok &= c->cell_count.ensure((size_t)ntiles * SWR_SEGS * 4 + 16);
    ok &= c->cell_count.p && cudaMemset(c->cell_count.p, 0, c->cell_count.bytes) == cudaSuccess;
  }
  ok &= c->cell_start.ensure(((size_t)ntiles * SWR_SEGS + 1) * 4 + 16);
  ok &= c->quad_flag.ensure((size_t)ntiles + 16);
  ok &= c->quad_tiles.ensure((size_t)quad_cap(ntiles) * 4 + 16);
  ok &= c->quad_count.ensure(16);
  ok &= c->geo_bar.ensure(16);
  if (c->big_cells.bytes < ((size_t)ntiles * SWR_SEGS + 2) * 4) {
    ok &= c->big_cells.ensure(((size_t)ntiles * SWR_SEGS + 2) * 4 + 16);
    // the list length and completion counter start at zero (k_sort_big resets them)
    ok &= c->big_cells.p && cudaMemset(c->big_cells.p, 0, 8) == cudaSuccess;
  }
  // Overwrite shaders: tiles of many layers are rasterized in up to SWR_SLICES_MAX slices
  // (the buffer is kept under 512 MiB by using fewer slices on large targets).
  c->slices = 1;
  if (ps && ps->overwrite) {
    const size_t per_slice = (size_t)ntiles * c->tile * c->tile * (size_t)ps->state_bytes;
    int k = SWR_SLICES_MAX;
    while (k > 1 && per_slice * (size_t)k > ((size_t)512 << 20)) --k;
    if (k > 1 && c->slice_state.ensure(per_slice * (size_t)k)) c->slices = k;
  }
  // Depth-min shaders: the listed heavy tiles' runs (optional, like the slices above; the
  // per-slot completion counters start at zero and every merge leaves its own at zero)
  c->dslice_ok = false;
  if (ps && ps->depth_min && (c->dslice_chunks < 0 ? ps->slice_chunks : c->dslice_chunks) > 0) {
    const size_t slots = slice_cap(ntiles);
    bool d = c->dslice_state.ensure(slots * SWR_DSLICES * c->tile * c->tile * (size_t)ps->state_bytes + 16);
    if (d && c->dslice_done.bytes < slots * 4 + 16)
      d = c->dslice_done.ensure(slots * 4 + 16) && cudaMemset(c->dslice_done.p, 0, c->dslice_done.bytes) == cudaSuccess;
    c->dslice_ok = d;
  }
  const size_t sw = sort_scratch_words(c->cap_pairs) + scan_scratch_words(c->cap_prims) + 64 + 2 * scan_scratch_words(ntiles * SWR_SEGS);
  ok &= c->scratch.ensure(sw * 4);
  ok &= c->draws.ensure(sizeof(SwrDrawDesc));
  ok &= c->targets.ensure(sizeof(SwrTargetDesc));
  ok &= c->draw_vbase.ensure(64);
  ok &= c->draw_bbase.ensure(64);
  ok &= c->target_tile_base.ensure(64);
  return ok ? SWR_OK : SWR_ENOMEM;
}

void fill_draw(const swr_context* c, SwrDrawDesc& D, int mode) {
  memset(&D, 0, sizeof(D));
  for (int a = 0; a < 8; ++a) {
    D.attrib[a] = c->attribs[a].ptr;
    D.attrib_stride[a] = c->attribs[a].stride;
  }
  D.draw_mode = mode;
  D.cull = c->cull;
  D.raster_mode = c->raster_mode;
  D.vp_px = (float)c->vp_w / 2.0f;  // VertexProcessor::setViewport
  D.vp_py = (float)c->vp_h / 2.0f;
  D.vp_ox = (float)c->vp_x + D.vp_px;
  D.vp_oy = (float)c->vp_y + D.vp_py;
  D.dn = c->dn;
  D.df = c->df;
  D.sc_minx = c->sc_x;
  D.sc_miny = c->sc_y;
  D.sc_maxx = c->sc_x + c->sc_w;
  D.sc_maxy = c->sc_y + c->sc_h;
  if (mode == SWR_DRAW_TRIANGLE && c->prim_src) {
    D.prim_src = c->prim_src;
    D.prim_src_cap = c->prim_src_cap < 0xffffffffull ? (uint32_t)c->prim_src_cap : 0xffffffffu;
  }
  D.u = c->u;
}

// The persistent geometry front end (swr_set_persistent_geometry): vertex shading, assembly
// count and emit as one cooperative launch.  False when it could not be launched; the
// caller then launches the three kernels.
bool geometry_front(swr_context* c, const VsOps* vs, const SwrDrawDesc* draws, int ndraws, const uint32_t* vbase,
                    uint32_t nverts, const AssembleArgs& aa, uint32_t nbatches, cudaStream_t s) {
  if (!vs->geometry) return false;
  // (the test hook starts the arrival count where no arrival can complete the barrier)
  if (cudaMemsetAsync(c->geo_bar.p, c->geo_stall ? 0x40 : 0, 4, s) != cudaSuccess ||
      cudaMemsetAsync(c->geo_bar.as<uint32_t>() + 1, 0, 4, s) != cudaSuccess ||
      vs->geometry(draws, ndraws, vbase, nverts, c->ptv.as<float>(), aa, nbatches, c->geo_bar.as<uint32_t>(), s) !=
          cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  c->launches -= nverts ? 2 : 1;  // one launch for the (up to) three counted kernels
  return true;
}

// Setup, binning and tile raster for the primitives in c->tris (count on the device).
// Binning: setup counts (tile, primitive segment) cells, a scan turns the counts into
// offsets, k_fill_bins scatters primitive ids into their cells, k_sort_cells restores the
// primitive order inside each cell; a tile's bin is then its cells' contiguous range.
int raster_stage(swr_context* c, const PsOps* ps, int S, int off_a, int off_p, int vs_a, int vs_p,
                 uint32_t ntiles, cudaStream_t s, int ntargets, bool has_span) {
  uint32_t* st = c->status.as<uint32_t>();
  const uint32_t ncells = ntiles * SWR_SEGS;
  int seg_shift = 0;
  while (((uint64_t)(c->cap_prims > 0 ? c->cap_prims - 1 : 0) >> seg_shift) >= SWR_SEGS) ++seg_shift;
  SetupArgs sa;
  memset(&sa, 0, sizeof(sa));
  sa.tris = c->tris.as<uint4>();
  sa.status = st;
  sa.cap_prims = c->cap_prims;
  sa.ptv = c->ptv.as<float>();
  sa.clipv = c->clipv.as<float>();
  sa.S = S;
  sa.off_a = off_a;
  sa.off_p = off_p;
  sa.vs_a = vs_a;
  sa.vs_p = vs_p;
  sa.draws = c->draws.as<SwrDrawDesc>();
  sa.targets = c->targets.as<SwrTargetDesc>();
  sa.recs = c->recs.as<float>();
  sa.tile_count = c->tile_count.as<uint32_t>();
  sa.tile = c->tile;
  sa.cell_count = c->cell_count.as<uint32_t>();
  sa.seg_shift = seg_shift;
  ps->setup(sa, s);
  mark(c, 3, s);
  uint32_t* scr = c->scratch.as<uint32_t>();
  uint32_t* cstart = c->cell_start.as<uint32_t>();
  scan_exclusive(c->cell_count.as<uint32_t>(), cstart, nullptr, ncells, cstart + ncells, scr, s);
  ps->fill_bins(st, c->cap_prims, c->recs.as<float>(), c->cell_count.as<uint32_t>(),
                cstart, ncells, seg_shift, c->cap_pairs, c->draws.as<SwrDrawDesc>(), c->targets.as<SwrTargetDesc>(),
                c->tile, c->keys0.as<uint32_t>(), st, s);
  const uint32_t warps_per_block = 8;
  // cells above 64 entries are sorted by k_sort_big, one warp per cell, with a bitmap of
  // the segment's id range in shared memory, while that range fits in kBigSortSmem
  const size_t bm_bytes = ((size_t)1 << seg_shift) / 8;  // one warp's bitmap
  const int big_warps = (int)std::min<size_t>(8, std::max<size_t>(1, kBigSortSmem / std::max<size_t>(bm_bytes, 1)));
  // (buffer: [list length, blocks done, cell ids...]; both words are zeroed when the buffer
  // is allocated and reset by k_sort_big's last block, which also closes the draw)
  const bool use_big = bm_bytes <= kBigSortSmem && c->big_cells.bytes >= (size_t)(ncells + 2) * 4;
  uint32_t* big = use_big ? c->big_cells.as<uint32_t>() : nullptr;
  // heavy tiles listed by k_sort_cells: rasterized in runs of chunks (depth-min shaders,
  // tiles of more than slice_chunks raster chunks), or else as quadrant CTAs (16-px tiles,
  // shaders other than the overwrite ones; 8-px raster tiles split every tile)
  const int slice_chunks = c->dslice_chunks < 0 ? ps->slice_chunks : c->dslice_chunks;
  const bool dsl = ps->depth_min && slice_chunks > 0 && c->dslice_ok && c->quad_mode != 2;
  const bool quads = !dsl && c->tile == 16 && !ps->overwrite && c->quad_mode != 0;
  const bool quad_list = quads && c->quad_mode == 1;
  const bool listed = dsl || quad_list;
  const uint32_t qcap = dsl ? slice_cap(ntiles) : quad_cap(ntiles);
  // (quad_count was zeroed by the draw's k_stage_copy)
  swr::launch(k_sort_cells, (ntiles + warps_per_block - 1) / warps_per_block, 256, 0, s, st, cstart, ntiles, c->cap_pairs, c->keys0.as<uint32_t>(), c->vals0.as<uint32_t>(), use_big ? big + 2 : nullptr,
      big, (uint32_t)SWR_RASTER_SORT,
      listed ? c->quad_flag.as<uint8_t>() : nullptr, c->quad_tiles.as<uint32_t>(), c->quad_count.as<uint32_t>(), qcap,
      dsl ? (uint32_t)(slice_chunks * ps->chunk) : kQuadMin);
  if (use_big) {
    swr::launch(k_sort_big, kBigSortWarps / big_warps, 32 * big_warps, bm_bytes * big_warps, s, st, cstart, ncells, c->cap_pairs, seg_shift, c->keys0.as<uint32_t>(), c->vals0.as<uint32_t>(), big + 2, big);
    c->launches += 1;
  }
  mark(c, 4, s);
  RasterArgs ra;
  ra.status = st;
  ra.tile_start = cstart;
  ra.tile_stride = SWR_SEGS;
  ra.bin = c->vals0.as<uint32_t>();
  ra.bin_raw = c->keys0.as<uint32_t>();  // tiles of <= SWR_RASTER_SORT entries are ordered in k_raster
  ra.recs = c->recs.as<float>();
  ra.draws = c->draws.as<SwrDrawDesc>();
  ra.targets = c->targets.as<SwrTargetDesc>();
  ra.target_tile_base = c->target_tile_base.as<uint32_t>();
  ra.ntargets = ntargets;
  ra.draw_prim_base = c->use_draw_pbase ? c->draw_pbase.as<uint32_t>() : nullptr;
  ra.status_w = st;
  ra.ntiles = ntiles;
  ra.has_span = has_span ? 1 : 0;
  ra.slices = ps->overwrite ? c->slices : 1;
  ra.slice_state = c->slice_state.p;
  ra.quad_flag = listed ? c->quad_flag.as<uint8_t>() : nullptr;
  ra.quad_tiles = c->quad_tiles.as<uint32_t>();
  ra.quad_count = c->quad_count.as<uint32_t>();
  ra.quad_cap = qcap;
  ra.quad_all = quads && c->quad_mode == 2;
  ra.dslice = dsl ? 1 : 0;
  ra.dslice_state = c->dslice_state.p;
  ra.dslice_done = c->dslice_done.as<uint32_t>();
  ps->raster(ra, ntiles, c->tile, s);
  if (ra.slices > 1) c->launches += 1;  // k_merge_slices
  mark(c, 5, s);
  if (!use_big) {
    swr::launch(k_close_draw, 1, 1, 0, s, st);
    c->launches += 1;
  }
  c->launches += 1 + 2 + 1 + 1 + (ntiles ? 1 : 0);
  return cuda_err(cudaGetLastError());
}

// Points and lines: per-primitive DDA setup, one fragment per step, stable sort by pixel,
// per-pixel ordered shading.  Fragment buffers reuse the bin-pair queues.
int lp_stage(swr_context* c, const PsOps* ps, int S, int off_a, int off_p, int vs_a, int vs_p,
             const SwrTargetDesc& T, cudaStream_t s) {
  uint32_t* st = c->status.as<uint32_t>();
  SetupArgs sa;
  memset(&sa, 0, sizeof(sa));
  sa.tris = c->tris.as<uint4>();
  sa.status = st;
  sa.cap_prims = c->cap_prims;
  sa.ptv = c->ptv.as<float>();
  sa.clipv = c->clipv.as<float>();
  sa.S = S;
  sa.off_a = off_a;
  sa.off_p = off_p;
  sa.vs_a = vs_a;
  sa.vs_p = vs_p;
  sa.draws = c->draws.as<SwrDrawDesc>();
  sa.targets = c->targets.as<SwrTargetDesc>();
  sa.recs = c->recs.as<float>();
  sa.tile_count = c->tile_count.as<uint32_t>();
  sa.tile = c->tile;
  ps->lp_setup(sa, s);
  mark(c, 3, s);
  uint32_t* scr = c->scratch.as<uint32_t>();
  uint32_t* sort_scr = scr + scan_scratch_words(c->cap_prims) + 32;
  scan_exclusive(c->tile_count.as<uint32_t>(), c->pair_off.as<uint32_t>(), st + SWR_ST_PRIMS, c->cap_prims,
                 st + SWR_ST_PAIRS, scr, s);
  const uint32_t invalid = (uint32_t)T.width * (uint32_t)T.height;
  LpFragArgs fa;
  fa.status = st;
  fa.cap_prims = c->cap_prims;
  fa.recs = c->recs.as<float>();
  fa.frag_off = c->pair_off.as<uint32_t>();
  fa.nfrags = st + SWR_ST_PAIRS;
  fa.cap_frags = c->cap_pairs;
  fa.draws = c->draws.as<SwrDrawDesc>();
  fa.targets = c->targets.as<SwrTargetDesc>();
  fa.keys = c->keys0.as<uint32_t>();
  fa.vals = c->vals0.as<uint32_t>();
  fa.status_w = st;
  fa.invalid = invalid;
  ps->lp_frags(fa, s);
  const int bits = bits_for(invalid + 1);
  const int which = radix_sort_pairs(c->keys0.as<uint32_t>(), c->vals0.as<uint32_t>(), c->keys1.as<uint32_t>(),
                                     c->vals1.as<uint32_t>(), st + SWR_ST_PAIRS, c->cap_pairs, bits, sort_scr, s);
  mark(c, 4, s);
  LpShadeArgs sh;
  sh.status = st;
  sh.cap_prims = c->cap_prims;
  sh.recs = c->recs.as<float>();
  sh.frag_off = c->pair_off.as<uint32_t>();
  sh.nfrags = st + SWR_ST_PAIRS;
  sh.cap_frags = c->cap_pairs;
  sh.keys = which ? c->keys1.as<uint32_t>() : c->keys0.as<uint32_t>();
  sh.vals = which ? c->vals1.as<uint32_t>() : c->vals0.as<uint32_t>();
  sh.draws = c->draws.as<SwrDrawDesc>();
  sh.targets = c->targets.as<SwrTargetDesc>();
  sh.target_pixel_base = c->target_tile_base.as<uint32_t>();
  sh.ntargets = 1;
  sh.invalid = invalid;
  sh.status_w = st;
  ps->lp_shade(sh, s);
  mark(c, 5, s);
  swr::launch(k_close_draw, 1, 1, 0, s, st);
  c->launches += 1 + 2 + 1 + 3 * ((bits + 7) / 8) + 1 + 1;
  return cuda_err(cudaGetLastError());
}

// Descriptors of a single draw are staged in a ring of pinned slots (a copy from pageable
// memory may block the host until the stream drains); a slot is rewritten only after the
// draw that read it has run, so the host can queue kSingleSlots draws ahead of the GPU.
// The slot's event is recorded after the draw's last kernel (end_single): an event between
// two kernels of the draw would hold back the second one's programmatic early launch.
static_assert(sizeof(SwrDrawDesc) + sizeof(SwrTargetDesc) <= kSingleSlotBytes, "descriptor slot size");

int upload_single(swr_context* c, const SwrDrawDesc& D, const SwrTargetDesc& T, cudaStream_t s) {
  int rc;
  if (!c->single_stage) {
    if ((rc = cuda_err(cudaMallocHost((void**)&c->single_stage, kSingleSlots * kSingleSlotBytes)))) return rc;
    for (int i = 0; i < kSingleSlots; ++i)
      if ((rc = cuda_err(cudaEventCreateWithFlags(&c->single_ev[i], cudaEventDisableTiming)))) return rc;
  }
  const int slot = c->single_next;
  c->single_next = (slot + 1) % kSingleSlots;
  if (c->single_pending[slot] && (rc = cuda_err(cudaEventSynchronize(c->single_ev[slot])))) return rc;
  unsigned char* h = c->single_stage + (size_t)slot * kSingleSlotBytes;
  memcpy(h, &D, sizeof(D));
  memcpy(h + sizeof(D), &T, sizeof(T));
  StageCopy sc;
  sc.add(c->draws.p, h, sizeof(D));
  sc.add(c->targets.p, h + sizeof(D), sizeof(T));
  // a single draw's vertex, batch and tile bases are 0; the per-draw working counters and
  // the heavy-tile list restart (flags and fragment totals are sticky)
  sc.clear(c->draw_vbase.p, 4);
  sc.clear(c->draw_bbase.p, 4);
  sc.clear(c->target_tile_base.p, 4);
  sc.clear(c->status.as<uint32_t>() + SWR_ST_CLIP_SLOTS, 5 * 4);
  sc.clear(c->quad_count.p, 4);
  swr::launch(k_stage_copy, 1, 256, 0, s, sc);
  c->launches += 1;
  c->single_cur = slot;
  return cuda_err(cudaGetLastError());
}

// A batch's staging slot is free again once the draw (or graph replay) that read it has run:
// its event is recorded after the whole draw, outside any captured graph (an event node
// inside the graph would hold back the programmatic early launch of the kernel after it).
int end_batch(swr_context* c, int slot, cudaStream_t s, int rc) {
  cudaEventRecord(c->stage_ev[slot], s);
  c->stage_pending[slot] = true;
  return rc;
}

int end_single(swr_context* c, cudaStream_t s, int rc) {
  if (c->single_cur >= 0) {
    cudaEventRecord(c->single_ev[c->single_cur], s);
    c->single_pending[c->single_cur] = true;
    c->single_cur = -1;
  }
  return rc;
}

SwrTargetDesc make_target(const swr_context* c) {
  SwrTargetDesc T;
  memset(&T, 0, sizeof(T));
  T.width = c->u.width;
  T.height = c->u.height;
  T.tiles_x = (T.width + c->tile - 1) / c->tile;
  T.tiles_y = (T.height + c->tile - 1) / c->tile;
  T.tile_base = 0;
  T.first_draw = 0;
  return T;
}

}  // namespace

extern "C" {

int swr_create(swr_context** out) {
  if (!out) return SWR_EINVAL;
  swr_context* c = new swr_context();
  memset(&c->u, 0, sizeof(c->u));
  c->attach_budget();
  // the segment bitmaps of k_sort_big may exceed the default 48 KB of dynamic shared memory
  cudaFuncSetAttribute(k_sort_big, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kBigSortSmem);
  cudaGetLastError();
  if (!c->status.ensure(kStatusWords * 4)) {
    delete c;
    return SWR_ENOMEM;
  }
  if (cudaMemset(c->status.p, 0, kStatusWords * 4) != cudaSuccess ||
      cudaMallocHost((void**)&c->status_host, kStatusWords * 4) != cudaSuccess) {
    delete c;
    return SWR_ECUDA;
  }
  *out = c;
  return SWR_OK;
}

int swr_destroy(swr_context* c) {
  if (!c) return SWR_EINVAL;
  if (c->status_host) cudaFreeHost(c->status_host);
  for (cudaEvent_t e : c->ev_pool) cudaEventDestroy(e);
  for (int i = 0; i < kBatchSlots; ++i) {
    if (c->gexec[i]) cudaGraphExecDestroy(c->gexec[i]);
    if (c->stage_ev[i]) cudaEventDestroy(c->stage_ev[i]);
  }
  if (c->cap_stream) cudaStreamDestroy(c->cap_stream);
  if (c->single_stage) cudaFreeHost(c->single_stage);
  for (int i = 0; i < kSingleSlots; ++i)
    if (c->single_ev[i]) cudaEventDestroy(c->single_ev[i]);
  if (c->stage) cudaFreeHost(c->stage);
  delete c;
  return SWR_OK;
}

int swr_set_viewport(swr_context* c, int x, int y, int w, int h) {
  if (!c) return SWR_EINVAL;
  c->vp_x = x; c->vp_y = y; c->vp_w = w; c->vp_h = h;
  return SWR_OK;
}

int swr_set_depth_range(swr_context* c, float n, float f) {
  if (!c) return SWR_EINVAL;
  c->dn = n; c->df = f;
  return SWR_OK;
}

int swr_set_cull_mode(swr_context* c, int mode) {
  if (!c || mode < 0 || mode > 2) return SWR_EINVAL;
  c->cull = mode;
  return SWR_OK;
}

int swr_set_vertex_shader(swr_context* c, int id) {
  if (!c || !vs_ops(id)) return SWR_EINVAL;
  c->vs_id = id;
  c->vs_cur = vs_ops(id);
  return SWR_OK;
}

static bool program_ok(const swr_program* p, uint32_t kind) {
  if (!p || p->magic != SWR_PROGRAM_MAGIC || p->abi != SWR_PROGRAM_ABI || p->kind != kind) return false;
  uint32_t mine[10];
  swr_program_layout(mine);
  for (int i = 0; i < 10; ++i)
    if (p->sizes[i] != mine[i]) return false;
  return kind == SWR_PROGRAM_VERTEX ? p->vs != nullptr : p->ps != nullptr;
}

int swr_set_vertex_program(swr_context* c, const swr_program* p) {
  if (!c || !program_ok(p, SWR_PROGRAM_VERTEX)) return SWR_EINVAL;
  const VsOps* o = p->vs;
  if (o->attribs < 0 || o->attribs > 8 || o->A < 0 || o->A > 16 || o->P < 0 || o->P > 16) return SWR_EINVAL;
  c->vs_id = 0;
  c->vs_cur = o;
  return SWR_OK;
}

int swr_set_pixel_program(swr_context* c, const swr_program* p) {
  if (!c || !program_ok(p, SWR_PROGRAM_PIXEL)) return SWR_EINVAL;
  const PsOps* o = p->ps;
  if (o->A < 0 || o->A > 16 || o->P < 0 || o->P > 16) return SWR_EINVAL;
  c->ps_id = 0;
  c->ps_cur = o;
  return SWR_OK;
}

int swr_set_vertex_attrib_pointer(swr_context* c, int index, int stride, const void* buffer, uint64_t bytes) {
  if (!c || index < 0 || index >= 8 || stride < 0) return SWR_EINVAL;  // VertexProcessor.cpp:69
  c->attribs[index].ptr = buffer;
  c->attribs[index].stride = stride;
  c->attribs[index].bytes = bytes;
  return SWR_OK;
}

int swr_set_raster_mode(swr_context* c, int mode) {
  if (!c || mode < 0 || mode > 2) return SWR_EINVAL;
  c->raster_mode = mode;
  return SWR_OK;
}

int swr_set_scissor_rect(swr_context* c, int x, int y, int w, int h) {
  if (!c) return SWR_EINVAL;
  c->sc_x = x; c->sc_y = y; c->sc_w = w; c->sc_h = h;
  return SWR_OK;
}

int swr_set_pixel_shader(swr_context* c, int id) {
  if (!c || !ps_ops(id)) return SWR_EINVAL;
  c->ps_id = id;
  c->ps_cur = ps_ops(id);
  return SWR_OK;
}

int swr_set_uniforms(swr_context* c, const SwrUniforms* u) {
  if (!c || !u || u->width <= 0 || u->height <= 0 || !u->color) return SWR_EINVAL;
  c->u = *u;
  c->have_u = true;
  return SWR_OK;
}

int swr_set_primitive_source(swr_context* c, int32_t* out, uint64_t capacity) {
  if (!c || (out && !capacity)) return SWR_EINVAL;
  c->prim_src = out;
  c->prim_src_cap = out ? capacity : 0;
  return SWR_OK;
}

int swr_set_queue_capacity(swr_context* c, uint64_t primitives, uint64_t bin_entries) {
  if (!c || primitives > 0xffffffffull || bin_entries > 0xffffffffull) return SWR_EINVAL;
  c->fixed_prims = primitives != 0;
  c->fixed_pairs = bin_entries != 0;
  if (primitives) c->cap_prims = (uint32_t)primitives;
  if (bin_entries) c->cap_pairs = (uint32_t)bin_entries;
  return SWR_OK;
}

int swr_get_queue_capacity(swr_context* c, uint64_t* primitives, uint64_t* bin_entries) {
  if (!c) return SWR_EINVAL;
  if (primitives) *primitives = c->cap_prims;
  if (bin_entries) *bin_entries = c->cap_pairs;
  return SWR_OK;
}

int swr_set_memory_limit(swr_context* c, uint64_t bytes) {
  if (!c) return SWR_EINVAL;
  c->budget.limit = (size_t)bytes;
  return SWR_OK;
}

int swr_memory_used(swr_context* c, uint64_t* bytes) {
  if (!c || !bytes) return SWR_EINVAL;
  *bytes = c->budget.used;
  return SWR_OK;
}

int swr_set_tile_size(swr_context* c, int tile) {
  if (!c || (tile != 8 && tile != 16 && tile != 32)) return SWR_EINVAL;
  c->tile = tile == 32 ? 32 : 16;  // 8: 16-px bins, every tile rasterized as four 8 x 8 CTAs
  c->quad_mode = tile == 8 ? 2 : 0;
  return SWR_OK;
}

int swr_set_persistent_geometry(swr_context* c, int on) {
  if (!c) return SWR_EINVAL;
  c->persistent_geometry = on != 0;
  return SWR_OK;
}

int swr_test_stall_geometry_barrier(swr_context* c, int on) {
  if (!c) return SWR_EINVAL;
  c->geo_stall = on != 0;
  return SWR_OK;
}

int swr_set_tile_split(swr_context* c, int on) {
  if (!c) return SWR_EINVAL;
  if (c->quad_mode != 2) c->quad_mode = on ? 1 : 0;
  return SWR_OK;
}

int swr_set_tile_slicing(swr_context* c, int chunks) {
  if (!c || chunks < -1) return SWR_EINVAL;
  c->dslice_chunks = chunks;
  return SWR_OK;
}

int swr_draw_elements(swr_context* c, int mode, uint64_t count, const uint32_t* indices, void* stream) {
  if (!c || !c->have_u) return SWR_EINVAL;
  const VsOps* vs = c->vs_cur;
  const PsOps* ps = c->ps_cur;
  if (!vs || !ps) return SWR_EINVAL;
  if (mode < SWR_DRAW_POINT || mode > SWR_DRAW_TRIANGLE) return SWR_EINVAL;
  if (ps->needs_eq && mode != SWR_DRAW_TRIANGLE) return SWR_EINVAL;  // PixelData::equations is null
  if (c->graph_mode && !c->profiling && mode == SWR_DRAW_TRIANGLE) {
    // graph mode: the draw is a one-item batch, captured once per layout and replayed
    swr_draw_item it;
    memset(&it, 0, sizeof(it));
    it.vs_id = 0;  // the context's current programs
    it.ps_id = 0;
    it.cull_mode = c->cull;
    it.raster_mode = c->raster_mode;
    it.viewport[0] = c->vp_x; it.viewport[1] = c->vp_y; it.viewport[2] = c->vp_w; it.viewport[3] = c->vp_h;
    it.depth_range[0] = c->dn;
    it.depth_range[1] = c->df;
    it.scissor[0] = c->sc_x; it.scissor[1] = c->sc_y; it.scissor[2] = c->sc_w; it.scissor[3] = c->sc_h;
    for (int a = 0; a < 8; ++a) {
      it.attrib[a] = c->attribs[a].ptr;
      it.attrib_stride[a] = c->attribs[a].stride;
      it.attrib_bytes[a] = c->attribs[a].bytes;
    }
    it.indices = indices;
    it.count = count;
    it.uniforms = &c->u;
    it.prim_src = c->prim_src;
    it.prim_src_capacity = c->prim_src_cap;
    return swr_draw_batch(c, &it, 1, stream);
  }
  const uint64_t per = mode == SWR_DRAW_POINT ? 1 : (mode == SWR_DRAW_LINE ? 2 : 3);
  if (count % per || count / per >= 0x7fffffffull || (count && !indices)) return SWR_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  uint64_t nverts = ~0ull;
  for (int a = 0; a < vs->attribs; ++a) {
    const Attrib& at = c->attribs[a];
    if (!at.ptr || at.stride <= 0 || at.bytes == 0) return SWR_EINVAL;
    uint64_t elem = (uint64_t)vs->elem_bytes[a < 2 ? a : 1];
    if (!elem) elem = (uint64_t)at.stride;
    // element i occupies [i * stride, i * stride + elem): the last one must fit
    const uint64_t n = at.bytes >= elem ? (at.bytes - elem) / (uint64_t)at.stride + 1 : 0;
    nverts = n < nverts ? n : nverts;
  }
  if (vs->attribs == 0) nverts = 0;
  if (nverts >= 0x7fffffffull) return SWR_EINVAL;
  const uint32_t nsub = (uint32_t)(count / per);
  const uint32_t nbatches = (nsub + SWR_BATCH_PRIMS - 1) / SWR_BATCH_PRIMS;
  const SwrTargetDesc T = make_target(c);
  const uint32_t ntiles = (uint32_t)T.tiles_x * (uint32_t)T.tiles_y;
  int rc = ensure_capacity(c, (uint32_t)nverts, vs->S, nsub, nbatches, ntiles, ps->R > ps->lp_R ? ps->R : ps->lp_R, ps);
  if (rc) return rc;
  SwrDrawDesc D;
  fill_draw(c, D, mode);
  D.indices = indices;
  D.nidx = (uint32_t)count;
  D.nverts = (uint32_t)nverts;
  D.nprims = nsub;
  if ((rc = upload_single(c, D, T, s))) return rc;
  uint32_t* st = c->status.as<uint32_t>();
  mark(c, 0, s);
  // triangles with the persistent geometry front end: vertex shading and assembly in one launch
  const bool geo = mode == SWR_DRAW_TRIANGLE && c->persistent_geometry && nbatches;
  if (!geo) vs->vertex(c->draws.as<SwrDrawDesc>(), 1, c->draw_vbase.as<uint32_t>(), (uint32_t)nverts, c->ptv.as<float>(), s);
  mark(c, 1, s);
  c->launches += (nverts ? 1 : 0) + (nbatches ? 2 : 0) + (mode == SWR_DRAW_TRIANGLE ? 0 : 1);
  AssembleArgs aa;
  aa.draws = c->draws.as<SwrDrawDesc>();
  aa.ndraws = 1;
  aa.draw_bbase = c->draw_bbase.as<uint32_t>();
  aa.ptv = c->ptv.as<float>();
  aa.clipv = c->clipv.as<float>();
  aa.clip_table = c->clip_table.as<SwrClipEntry>();
  aa.clip_slot = c->clip_slot.as<uint32_t>();
  aa.tri_flags = c->tri_flags.as<uint8_t>();
  aa.batch_counts = c->batch_counts.as<uint2>();
  aa.batch_base = c->batch_base.as<uint32_t>();
  aa.tris = c->tris.as<uint4>();
  aa.lp_refs = c->lp_refs.as<uint2>();
  aa.draw_prim_base = nullptr;  // a single draw numbers its primitives from 0
  aa.status = st;
  aa.cap_clip_slots = c->cap_clip_slots;
  aa.cap_clip_verts = c->cap_clip_verts;
  aa.cap_prims = c->cap_prims;
  c->use_draw_pbase = false;
  if (mode == SWR_DRAW_TRIANGLE) {
    if (!(geo && geometry_front(c, vs, c->draws.as<SwrDrawDesc>(), 1, c->draw_vbase.as<uint32_t>(),
                                (uint32_t)nverts, aa, nbatches, s))) {
      if (geo) vs->vertex(c->draws.as<SwrDrawDesc>(), 1, c->draw_vbase.as<uint32_t>(), (uint32_t)nverts,
                          c->ptv.as<float>(), s);
      vs->assemble_count(aa, nbatches, s);
      vs->assemble_emit(aa, nbatches, s);  // derives batch bases and the primitive count itself
    }
  } else {
    vs->assemble_lp_count(aa, nbatches, s);
    swr::launch(k_batch_scan, 1, 1024, 0, s, c->batch_counts.as<uint2>(), nbatches, c->batch_base.as<uint32_t>(), st,
                                    c->cap_prims);
    vs->assemble_lp_emit(aa, nbatches, s);
  }
  mark(c, 2, s);
  c->last_ntiles = ntiles;
  if (mode != SWR_DRAW_TRIANGLE) return end_single(c, s, lp_stage(c, ps, vs->S, 8, 8 + vs->A, vs->A, vs->P, T, s));
  return end_single(c, s, raster_stage(c, ps, vs->S, 8, 8 + vs->A, vs->A, vs->P, ntiles, s, 1,
                                       c->raster_mode != SWR_RASTER_BLOCK));
}

int swr_draw_list(swr_context* c, int mode, const float* vertices, uint64_t nverts, const int32_t* indices,
                  uint64_t count, void* stream) {
  if (!c || !c->have_u) return SWR_EINVAL;
  const PsOps* ps = c->ps_cur;
  if (!ps) return SWR_EINVAL;
  if (mode < SWR_DRAW_POINT || mode > SWR_DRAW_TRIANGLE) return SWR_EINVAL;
  if (ps->needs_eq && mode != SWR_DRAW_TRIANGLE) return SWR_EINVAL;  // PixelData::equations is null
  const int per = mode == SWR_DRAW_POINT ? 1 : (mode == SWR_DRAW_LINE ? 2 : 3);
  if (count % per || count / per >= 0x7fffffffull || nverts >= 0x7fffffffull) return SWR_EINVAL;
  if ((count && !indices) || (nverts && !vertices)) return SWR_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  const uint32_t nsub = (uint32_t)(count / per);
  const SwrTargetDesc T = make_target(c);
  const uint32_t ntiles = (uint32_t)T.tiles_x * (uint32_t)T.tiles_y;
  int rc = ensure_capacity(c, (uint32_t)nverts, ps->S, nsub, 1, ntiles, ps->R > ps->lp_R ? ps->R : ps->lp_R, ps);
  if (rc) return rc;
  if (!c->direct_keep.ensure((size_t)nsub * 4 + 16) || !c->direct_pos.ensure((size_t)nsub * 4 + 16))
    return SWR_ENOMEM;
  SwrDrawDesc D;
  fill_draw(c, D, mode);
  D.direct = 1;
  D.nprims = nsub;
  D.nverts = (uint32_t)nverts;
  if ((rc = upload_single(c, D, T, s))) return rc;
  uint32_t* st = c->status.as<uint32_t>();
  mark(c, 0, s);
  ps->direct_vertices(vertices, (uint32_t)nverts, c->ptv.as<float>(), s);
  mark(c, 1, s);
  c->launches += (nverts ? 1 : 0) + (nsub ? 4 : 0);
  if (nsub) {
    const int grid = (int)((nsub + 255) / 256 < 1216 ? (nsub + 255) / 256 : 1216);
    swr::launch(k_direct_flags, grid, 256, 0, s, indices, nsub, per, c->direct_keep.as<uint32_t>());
    scan_exclusive(c->direct_keep.as<uint32_t>(), c->direct_pos.as<uint32_t>(), nullptr, nsub,
                   st + SWR_ST_PRIMS, c->scratch.as<uint32_t>(), s);
    swr::launch(k_direct_emit, grid, 256, 0, s, indices, nsub, per, (uint32_t)nverts, c->direct_keep.as<uint32_t>(),
                                       c->direct_pos.as<uint32_t>(), c->tris.as<uint4>(), st);
  }
  mark(c, 2, s);
  c->last_ntiles = ntiles;
  if (mode != SWR_DRAW_TRIANGLE) return end_single(c, s, lp_stage(c, ps, ps->S, 8, 8 + ps->A, ps->A, ps->P, T, s));
  return end_single(c, s, raster_stage(c, ps, ps->S, 8, 8 + ps->A, ps->A, ps->P, ntiles, s, 1,
                                       c->raster_mode != SWR_RASTER_BLOCK));
}

int swr_set_graph_mode(swr_context* c, int on) {
  if (!c) return SWR_EINVAL;
  c->graph_mode = on != 0;
  return SWR_OK;
}

int swr_draw_batch(swr_context* c, const swr_draw_item* items, int n, void* stream) {
  if (!c || !items || n <= 0) return SWR_EINVAL;
  // id 0: the context's current program (a built-in one or a caller's swr_program)
  const VsOps* vs = items[0].vs_id ? vs_ops(items[0].vs_id) : c->vs_cur;
  const PsOps* ps = items[0].ps_id ? ps_ops(items[0].ps_id) : c->ps_cur;
  if (!vs || !ps) return SWR_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  std::vector<SwrDrawDesc> D(n);
  bool any_span = false;  // some item rasterizes in Span or Adaptive mode
  std::vector<SwrTargetDesc> T;
  std::vector<const void*> tcolor;
  std::vector<uint32_t> vbase(n), bbase(n), tbase;
  uint64_t V = 0, P = 0, B = 0, NT = 0, PIX = 0;
  uint64_t sig = 1469598103934665603ull;
  auto mix = [&](uint64_t x) { sig = (sig ^ x) * 1099511628211ull; };
  for (int i = 0; i < n; ++i) {
    const swr_draw_item& it = items[i];
    if (it.vs_id != items[0].vs_id || it.ps_id != items[0].ps_id || !it.uniforms) return SWR_EINVAL;
    if (it.cull_mode < 0 || it.cull_mode > 2 || it.raster_mode < 0 || it.raster_mode > 2) return SWR_EINVAL;
    if (it.count % 3 || (it.count && !it.indices)) return SWR_EINVAL;
    const SwrUniforms& u = *it.uniforms;
    if (u.width <= 0 || u.height <= 0 || !u.color) return SWR_EINVAL;
    uint64_t nv = ~0ull;
    for (int a = 0; a < vs->attribs; ++a) {
      if (!it.attrib[a] || it.attrib_stride[a] <= 0 || it.attrib_bytes[a] == 0) return SWR_EINVAL;
      uint64_t elem = (uint64_t)vs->elem_bytes[a < 2 ? a : 1];
      if (!elem) elem = (uint64_t)it.attrib_stride[a];
      const uint64_t k = it.attrib_bytes[a] >= elem ? (it.attrib_bytes[a] - elem) / (uint64_t)it.attrib_stride[a] + 1 : 0;
      nv = k < nv ? k : nv;
    }
    if (vs->attribs == 0) nv = 0;
    // target: shared with an earlier item drawing into the same colour buffer
    int t = -1;
    for (size_t j = 0; j < tcolor.size(); ++j)
      if (tcolor[j] == u.color) t = (int)j;
    if (t >= 0 && (T[t].width != u.width || T[t].height != u.height)) return SWR_EINVAL;
    if (t < 0) {
      SwrTargetDesc td;
      memset(&td, 0, sizeof(td));
      td.width = u.width;
      td.height = u.height;
      td.tiles_x = (u.width + c->tile - 1) / c->tile;
      td.tiles_y = (u.height + c->tile - 1) / c->tile;
      td.tile_base = (uint32_t)NT;
      td.pixel_base = (uint32_t)PIX;
      td.first_draw = i;
      NT += (uint64_t)td.tiles_x * (uint64_t)td.tiles_y;
      PIX += (uint64_t)u.width * (uint64_t)u.height;
      t = (int)T.size();
      T.push_back(td);
      tcolor.push_back(u.color);
      tbase.push_back(td.tile_base);
    }
    SwrDrawDesc& d = D[i];
    memset(&d, 0, sizeof(d));
    for (int a = 0; a < 8; ++a) {
      d.attrib[a] = it.attrib[a];
      d.attrib_stride[a] = it.attrib_stride[a];
    }
    d.indices = it.indices;
    d.nidx = (uint32_t)it.count;
    d.nverts = (uint32_t)nv;
    d.nprims = (uint32_t)(it.count / 3);
    d.vbase = (uint32_t)V;
    d.pbase = (uint32_t)P;
    d.bbase = (uint32_t)B;
    d.target = t;
    d.draw_mode = SWR_DRAW_TRIANGLE;
    d.cull = it.cull_mode;
    d.raster_mode = it.raster_mode;
    any_span |= it.raster_mode != SWR_RASTER_BLOCK;
    d.vp_px = (float)it.viewport[2] / 2.0f;
    d.vp_py = (float)it.viewport[3] / 2.0f;
    d.vp_ox = (float)it.viewport[0] + d.vp_px;
    d.vp_oy = (float)it.viewport[1] + d.vp_py;
    d.dn = it.depth_range[0];
    d.df = it.depth_range[1];
    d.sc_minx = it.scissor[0];
    d.sc_miny = it.scissor[1];
    d.sc_maxx = it.scissor[0] + it.scissor[2];
    d.sc_maxy = it.scissor[1] + it.scissor[3];
    d.u = u;
    if (it.prim_src) {
      if (!it.prim_src_capacity) return SWR_EINVAL;
      d.prim_src = it.prim_src;
      d.prim_src_cap = it.prim_src_capacity < 0xffffffffull ? (uint32_t)it.prim_src_capacity : 0xffffffffu;
    }
    vbase[i] = (uint32_t)V;
    bbase[i] = (uint32_t)B;
    V += nv;
    P += d.nprims;
    B += (d.nprims + SWR_BATCH_PRIMS - 1) / SWR_BATCH_PRIMS;
    mix(nv); mix(d.nprims); mix((uint64_t)t); mix((uint64_t)u.width << 32 | (uint32_t)u.height);
    mix((uint64_t)it.raster_mode << 8 | (uint64_t)it.cull_mode);
  }
  if (V >= 0x7fffffffull || P >= 0x7fffffffull || NT >= 0x7fffffffull / SWR_SEGS || PIX >= 0xffffffffull)
    return SWR_EINVAL;
  const int ntg = (int)T.size();
  int rc = ensure_capacity(c, (uint32_t)V, vs->S, (uint32_t)P, (uint32_t)B, (uint32_t)NT,
                           ps->R > ps->lp_R ? ps->R : ps->lp_R, ps);
  if (rc) return rc;
  bool ok = c->draws.ensure(sizeof(SwrDrawDesc) * n) && c->targets.ensure(sizeof(SwrTargetDesc) * ntg) &&
            c->draw_vbase.ensure(4 * n + 16) && c->draw_bbase.ensure(4 * n + 16) && c->draw_pbase.ensure(4 * n + 16) &&
            c->target_tile_base.ensure(4 * ntg + 16);
  if (!ok) return SWR_ENOMEM;
  // pinned staging, kBatchSlots slots used in turn; wait until the last draw that read this
  // slot has run (the draw kBatchSlots calls back, normally long finished)
  const size_t bytes = sizeof(SwrDrawDesc) * n + sizeof(SwrTargetDesc) * ntg + 4 * (2 * n + ntg) + 64;
  const int slot = c->stage_next;
  c->stage_next = (slot + 1) % kBatchSlots;
  if (c->stage_pending[slot]) {
    if ((rc = cuda_err(cudaEventSynchronize(c->stage_ev[slot])))) return rc;
    c->stage_pending[slot] = false;
  }
  if (bytes > c->stage_bytes / kBatchSlots) {
    for (int k = 0; k < kBatchSlots; ++k)  // the other slots' draws may still read them
      if (c->stage_pending[k]) {
        if ((rc = cuda_err(cudaEventSynchronize(c->stage_ev[k])))) return rc;
        c->stage_pending[k] = false;
      }
    if (c->stage) cudaFreeHost(c->stage);
    c->stage = nullptr;
    c->stage_bytes = 0;
    if ((rc = cuda_err(cudaMallocHost((void**)&c->stage, bytes * 2 * kBatchSlots)))) return rc;
    c->stage_bytes = bytes * 2 * kBatchSlots;
  }
  for (int k = 0; k < kBatchSlots; ++k)
    if (!c->stage_ev[k] && (rc = cuda_err(cudaEventCreateWithFlags(&c->stage_ev[k], cudaEventDisableTiming))))
      return rc;
  unsigned char* h = c->stage + (size_t)slot * (c->stage_bytes / kBatchSlots);
  const size_t o_d = 0, o_t = o_d + sizeof(SwrDrawDesc) * n, o_vb = o_t + sizeof(SwrTargetDesc) * ntg;
  const size_t o_bb = o_vb + 4 * n, o_tb = o_bb + 4 * n;
  memcpy(h + o_d, D.data(), sizeof(SwrDrawDesc) * n);
  memcpy(h + o_t, T.data(), sizeof(SwrTargetDesc) * ntg);
  memcpy(h + o_vb, vbase.data(), 4 * n);
  memcpy(h + o_bb, bbase.data(), 4 * n);
  memcpy(h + o_tb, tbase.data(), 4 * ntg);
  mix((uint64_t)(uintptr_t)vs); mix((uint64_t)(uintptr_t)ps);  // the programs (their kernels)
  mix((uint64_t)c->quad_mode);
  mix((uint64_t)c->persistent_geometry);
  mix((uint64_t)vs->S); mix((uint64_t)ps->R); mix((uint64_t)c->tile); mix((uint64_t)n);
  mix(c->cap_prims); mix(c->cap_pairs); mix(c->cap_clip_slots); mix(c->cap_clip_verts);
  const void* bufs[] = {c->ptv.p, c->clipv.p, c->clip_table.p, c->clip_slot.p, c->tri_flags.p, c->batch_counts.p,
                        c->tris.p, c->recs.p, c->tile_count.p, c->keys0.p, c->vals0.p, c->cell_count.p,
                        c->cell_start.p, c->scratch.p, c->draws.p, c->targets.p, c->draw_vbase.p,
                        c->draw_bbase.p, c->target_tile_base.p, c->draw_pbase.p, c->big_cells.p, h,
                        c->slice_state.p, (const void*)(uintptr_t)c->slices, c->quad_flag.p, c->quad_tiles.p,
                        c->quad_count.p, c->geo_bar.p, c->dslice_state.p, c->dslice_done.p,
                        (const void*)(uintptr_t)c->dslice_ok, (const void*)(intptr_t)c->dslice_chunks};
  for (const void* b : bufs) mix((uint64_t)(uintptr_t)b);
  if (c->graph_mode && c->gexec[slot] && sig == c->gsig[slot]) {
    if ((rc = cuda_err(cudaGraphLaunch(c->gexec[slot], s)))) return rc;
    c->launches += c->glaunches[slot];
    return end_batch(c, slot, s, SWR_OK);
  }
  cudaGraph_t graph = nullptr;
  const uint64_t launches0 = c->launches;
  cudaStream_t launch_stream = s;
  if (c->graph_mode) {
    // the caller's stream may be the legacy default stream, which cannot be captured
    if (!c->cap_stream && (rc = cuda_err(cudaStreamCreateWithFlags(&c->cap_stream, cudaStreamNonBlocking))))
      return rc;
    s = c->cap_stream;
    if ((rc = cuda_err(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal)))) return rc;
    c->capturing = true;
  }
  int q = SWR_OK;
  {
    StageCopy sc;
    sc.add(c->draws.p, h + o_d, sizeof(SwrDrawDesc) * n);
    sc.add(c->targets.p, h + o_t, sizeof(SwrTargetDesc) * ntg);
    sc.add(c->draw_vbase.p, h + o_vb, 4 * n);
    sc.add(c->draw_bbase.p, h + o_bb, 4 * n);
    sc.add(c->target_tile_base.p, h + o_tb, 4 * ntg);
    // the per-draw working counters and the heavy-tile list restart (flags and fragment
    // totals are sticky)
    sc.clear(c->status.as<uint32_t>() + SWR_ST_CLIP_SLOTS, 5 * 4);
    sc.clear(c->quad_count.p, 4);
    swr::launch(k_stage_copy, kStageCopyBlocks, 256, 0, s, sc);
    c->launches += 1;
    q = cuda_err(cudaGetLastError());
  }
  q = q ? q : cuda_err(cudaGetLastError());
  uint32_t* st = c->status.as<uint32_t>();
  mark(c, 0, s);
  const bool geo = c->persistent_geometry && B;
  if (!geo) vs->vertex(c->draws.as<SwrDrawDesc>(), n, c->draw_vbase.as<uint32_t>(), (uint32_t)V, c->ptv.as<float>(), s);
  mark(c, 1, s);
  AssembleArgs aa;
  memset(&aa, 0, sizeof(aa));
  aa.draws = c->draws.as<SwrDrawDesc>();
  aa.ndraws = n;
  aa.draw_bbase = c->draw_bbase.as<uint32_t>();
  aa.ptv = c->ptv.as<float>();
  aa.clipv = c->clipv.as<float>();
  aa.clip_table = c->clip_table.as<SwrClipEntry>();
  aa.clip_slot = c->clip_slot.as<uint32_t>();
  aa.tri_flags = c->tri_flags.as<uint8_t>();
  aa.batch_counts = c->batch_counts.as<uint2>();
  aa.batch_base = c->batch_base.as<uint32_t>();
  aa.tris = c->tris.as<uint4>();
  aa.lp_refs = c->lp_refs.as<uint2>();
  aa.draw_prim_base = c->draw_pbase.as<uint32_t>();
  aa.status = st;
  aa.cap_clip_slots = c->cap_clip_slots;
  aa.cap_clip_verts = c->cap_clip_verts;
  aa.cap_prims = c->cap_prims;
  c->use_draw_pbase = true;
  if (!(geo && geometry_front(c, vs, c->draws.as<SwrDrawDesc>(), n, c->draw_vbase.as<uint32_t>(), (uint32_t)V, aa,
                              (uint32_t)B, s))) {
    if (geo) vs->vertex(c->draws.as<SwrDrawDesc>(), n, c->draw_vbase.as<uint32_t>(), (uint32_t)V, c->ptv.as<float>(), s);
    vs->assemble_count(aa, (uint32_t)B, s);
    vs->assemble_emit(aa, (uint32_t)B, s);
  }
  mark(c, 2, s);
  c->launches += (V ? 1 : 0) + (B ? 2 : 0);
  if (!q) q = cuda_err(cudaGetLastError());
  rc = raster_stage(c, ps, vs->S, 8, 8 + vs->A, vs->A, vs->P, (uint32_t)NT, s, ntg, any_span);
  if (q) rc = q;
  c->use_draw_pbase = false;
  if (c->graph_mode) {
    c->capturing = false;
    const int rc2 = cuda_err(cudaStreamEndCapture(s, &graph));
    if (rc || rc2) {
      if (graph) cudaGraphDestroy(graph);
      return rc ? rc : rc2;
    }
    if (c->gexec[slot]) cudaGraphExecDestroy(c->gexec[slot]);
    c->gexec[slot] = nullptr;
    rc = cuda_err(cudaGraphInstantiate(&c->gexec[slot], graph, 0));
    cudaGraphDestroy(graph);
    if (rc) return rc;
    c->gsig[slot] = sig;
    c->glaunches[slot] = c->launches - launches0;
    if ((rc = cuda_err(cudaGraphLaunch(c->gexec[slot], launch_stream)))) return rc;
  }
  return end_batch(c, slot, launch_stream, rc);
}

int swr_finish(swr_context* c, void* stream, swr_stats* stats) {
  if (!c) return SWR_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  int rc = cuda_err(cudaMemcpyAsync(c->status_host, c->status.p, kStatusWords * 4, cudaMemcpyDeviceToHost, s));
  if (rc) return rc;
  if ((rc = cuda_err(cudaStreamSynchronize(s)))) return rc;
  const uint32_t* h = c->status_host;
  if (stats) {
    stats->fragments = (uint64_t)h[SWR_ST_SHADED_LO] | ((uint64_t)h[SWR_ST_SHADED_HI] << 32);
    stats->primitives = h[SWR_ST_PRIMS];
    stats->bin_pairs = h[SWR_ST_PAIRS];
    stats->clip_polygons = h[SWR_ST_CLIP_SLOTS];
    stats->flags = h[SWR_ST_FLAGS];
    stats->launches = c->launches;
    stats->passes = (uint64_t)h[SWR_ST_PASSES_LO] | ((uint64_t)h[SWR_ST_PASSES_HI] << 32);
  }
  c->launches = 0;
  const uint32_t flags = h[SWR_ST_FLAGS];
  if (flags & SWR_F_ANY_OVERFLOW) {
    grow_u32(c->cap_clip_slots, h[kStickyBase + SWR_ST_CLIP_SLOTS]);
    grow_u32(c->cap_clip_verts, h[kStickyBase + SWR_ST_CLIP_VERTS]);
    grow_u32(c->cap_prims, h[kStickyBase + SWR_ST_PRIMS]);
    grow_u32(c->cap_pairs, h[kStickyBase + SWR_ST_PAIRS]);
  }
  cudaMemsetAsync(c->status.p, 0, kStatusWords * 4, s);
  if ((rc = cuda_err(cudaStreamSynchronize(s)))) return rc;
  if (flags & SWR_F_ANY_OVERFLOW) return SWR_EOVERFLOW;
  if (flags & SWR_F_BARRIER_TIMEOUT) return SWR_ECUDA;
  if (flags & (SWR_F_BAD_INDEX | SWR_F_BAD_GRAD_INPUT)) return SWR_EINDEX;
  if (flags & SWR_F_SRC_OVERFLOW) return SWR_EINVAL;
  return SWR_OK;
}

int swr_set_profiling(swr_context* c, int on) {
  if (!c) return SWR_EINVAL;
  c->profiling = on != 0;
  c->ev_used = 0;
  return SWR_OK;
}

int swr_stage_times(swr_context* c, float* ms) {
  if (!c || !ms) return SWR_EINVAL;
  for (int i = 0; i < 5; ++i) ms[i] = 0.0f;
  const size_t draws = c->ev_used / 6;
  int rc = SWR_OK;
  if (draws) rc = cuda_err(cudaEventSynchronize(c->ev_pool[6 * draws - 1]));
  for (size_t d = 0; d < draws && !rc; ++d)
    for (int i = 0; i < 5; ++i) {
      float t = 0.0f;
      if ((rc = cuda_err(cudaEventElapsedTime(&t, c->ev_pool[6 * d + i], c->ev_pool[6 * d + i + 1])))) break;
      ms[i] += t;
    }
  c->ev_used = 0;
  return rc;
}

const char* swr_status_string(int st) {
  switch (st) {
    case SWR_OK: return "ok";
    case SWR_EINVAL: return "invalid argument";
    case SWR_ENOMEM: return "out of device memory";
    case SWR_EOVERFLOW: return "scratch queue overflow (queue grown; issue the draw again)";
    case SWR_ECUDA: return "CUDA error";
    case SWR_EINDEX: return "index beyond the bound vertex buffers";
    default: return "unknown status";
  }
}

}  // extern "C"
namespace swr {
uint32_t* context_status(swr_context* c) { return c->status.as<uint32_t>(); }
void context_add_launches(swr_context* c, uint64_t n) { c->launches += n; }
}  // namespace swr
