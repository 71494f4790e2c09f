// Generic device primitives with device-resident lengths, so a whole draw can be queued
// (and captured in a CUDA graph) without reading counts back to the host:
//   * exclusive scan (reduce / scan-of-partials / downsweep over fixed chunks),
//   * stable LSD radix sort of (key, value) pairs, 8 bits per pass.  Stability is what
//     keeps every tile's primitive list in submission order after binning,
//   * segment starts of a sorted key array (the per-tile bin offsets).
#include "swr_core.h"

namespace swr {
namespace {

constexpr int kThreads = 256;
constexpr int kTile = 1024;  // items per block iteration (4 per thread)
constexpr int kSortBlocks = 304;  // radix-sort blocks (2 per SM)

__device__ __forceinline__ uint32_t load_n(const uint32_t* n_dev, uint32_t n_max) {
  if (!n_dev) return n_max;
  const uint32_t n = *n_dev;
  return n < n_max ? n : n_max;
}

__device__ __forceinline__ void chunk_range(uint32_t n, uint32_t chunk, uint32_t& b, uint32_t& e) {
  b = blockIdx.x * chunk;
  e = b + chunk;
  if (b > n) b = n;
  if (e > n) e = n;
}

__global__ void __launch_bounds__(kThreads) k_scan_reduce(const uint32_t* in, const uint32_t* n_dev,
                                                          uint32_t n_max, uint32_t chunk,
                                                          uint32_t* partials) {
  swr_pdl_entry();
  __shared__ uint32_t tmp[32];
  const uint32_t n = load_n(n_dev, n_max);
  uint32_t b, e;
  chunk_range(n, chunk, b, e);
  uint32_t s = 0;
  for (uint32_t i = b + threadIdx.x; i < e; i += kThreads) s += in[i];
  uint32_t tot;
  swr_block_exscan(s, tmp, &tot);
  if (threadIdx.x == 0) partials[blockIdx.x] = tot;
}

__global__ void __launch_bounds__(kThreads) k_scan_down(const uint32_t* in, uint32_t* out,
                                                        const uint32_t* n_dev, uint32_t n_max,
                                                        uint32_t chunk, const uint32_t* partials,
                                                        uint32_t* total) {
  swr_pdl_entry();
  __shared__ uint32_t tmp[32];
  const uint32_t n = load_n(n_dev, n_max);
  uint32_t b, e;
  chunk_range(n, chunk, b, e);
  // prefix of the partial sums of the blocks before this one (and the grand total)
  __shared__ uint32_t pref[2];
  {
    uint32_t mine = 0, all = 0;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += kThreads) {
      const uint32_t v = partials[i];
      all += v;
      if (i < (int)blockIdx.x) mine += v;
    }
    uint32_t t0, t1;
    swr_block_exscan(mine, tmp, &t0);
    swr_block_exscan(all, tmp, &t1);
    if (threadIdx.x == 0) { pref[0] = t0; pref[1] = t1; }
    __syncthreads();
  }
  if (blockIdx.x == 0 && threadIdx.x == 0 && total) *total = pref[1];
  uint32_t run = pref[0];
  for (uint32_t base = b; base < e; base += kTile) {
    uint32_t v[4], s = 0;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const uint32_t i = base + threadIdx.x * 4 + j;
      v[j] = i < e ? in[i] : 0u;
      s += v[j];
    }
    uint32_t tot;
    uint32_t ex = swr_block_exscan(s, tmp, &tot) + run;
#pragma unroll
    for (int j = 0; j < 4; ++j) {
      const uint32_t i = base + threadIdx.x * 4 + j;
      if (i < e) out[i] = ex;
      ex += v[j];
    }
    run += tot;
  }
}

uint32_t chunk_for(uint32_t n_max, int blocks) {
  uint32_t c = (n_max + blocks - 1) / blocks;
  c = (c + kTile - 1) / kTile * kTile;
  return c ? c : kTile;
}

// --- radix sort --------------------------------------------------------------------

constexpr int kWarps = kThreads / 32;

__global__ void __launch_bounds__(kThreads) k_radix_hist(const uint32_t* keys, const uint32_t* n_dev,
                                                         uint32_t n_max, uint32_t chunk, int shift,
                                                         uint32_t* hist, int nblocks) {
  swr_pdl_entry();
  __shared__ uint32_t cnt[256];
  cnt[threadIdx.x] = 0;
  __syncthreads();
  const uint32_t n = load_n(n_dev, n_max);
  uint32_t b, e;
  chunk_range(n, chunk, b, e);
  for (uint32_t i = b + threadIdx.x; i < e; i += kThreads) atomicAdd(&cnt[(keys[i] >> shift) & 255u], 1u);
  __syncthreads();
  hist[blockIdx.x * 256 + threadIdx.x] = cnt[threadIdx.x];  // [block][digit]
}

// Per-digit exclusive prefix over the block histograms, one warp per digit:
// off[b][d] = digit-d keys in blocks before b; tot[d] = all digit-d keys.
__global__ void __launch_bounds__(256) k_radix_offsets(const uint32_t* hist, uint32_t* off, uint32_t* tot,
                                                       int nblocks) {
  swr_pdl_entry();
  const int d = blockIdx.x * 8 + (threadIdx.x >> 5), lane = threadIdx.x & 31;
  uint32_t run = 0;
  for (int b0 = 0; b0 < nblocks; b0 += 32) {
    const int b = b0 + lane;
    const uint32_t v = b < nblocks ? hist[b * 256 + d] : 0u;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (b < nblocks) off[b * 256 + d] = run + x - v;
    run += __shfl_sync(0xffffffffu, x, 31);
  }
  if (lane == 0) tot[d] = run;
}

// Stable scatter: the block walks its chunk in 1024-item tiles; warp w ranks items
// [w*128, w*128+128) of the tile in 4 rounds of 32 with match_any, warps are combined
// by a per-digit prefix over warps, and the running per-digit base keeps chunk order.
__global__ void __launch_bounds__(kThreads) k_radix_scatter(const uint32_t* kin, const uint32_t* vin,
                                                            uint32_t* kout, uint32_t* vout,
                                                            const uint32_t* n_dev, uint32_t n_max,
                                                            uint32_t chunk, int shift,
                                                            const uint32_t* off, const uint32_t* tot) {
  swr_pdl_entry();
  __shared__ uint32_t wcnt[kWarps][256];
  __shared__ uint32_t base[256];
  __shared__ uint32_t tile_tot[256];
  __shared__ uint32_t tmp[32];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  for (int w = 0; w < kWarps; ++w) wcnt[w][threadIdx.x] = 0;
  {
    // digit d starts at (keys with a smaller digit) + (digit-d keys in earlier blocks)
    const uint32_t dbase = swr_block_exscan(tot[threadIdx.x], tmp, nullptr);
    base[threadIdx.x] = dbase + off[blockIdx.x * 256 + threadIdx.x];
  }
  __syncthreads();
  const uint32_t n = load_n(n_dev, n_max);
  uint32_t b, e;
  chunk_range(n, chunk, b, e);
  const uint32_t lt = (1u << lane) - 1u;
  for (uint32_t t0 = b; t0 < e; t0 += kTile) {
    uint32_t key[4], val[4], dig[4], rank[4];
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const uint32_t i = t0 + warp * 128 + r * 32 + lane;
      const bool ok = i < e;
      key[r] = ok ? kin[i] : 0u;
      val[r] = ok ? vin[i] : 0u;
      dig[r] = ok ? ((key[r] >> shift) & 255u) : 0xffffffffu;
      const uint32_t peers = __match_any_sync(0xffffffffu, dig[r]);
      const uint32_t before = ok ? wcnt[warp][dig[r]] : 0u;
      rank[r] = before + __popc(peers & lt);
      __syncwarp();
      if (ok && (peers & lt) == 0u) wcnt[warp][dig[r]] = before + __popc(peers);
      __syncwarp();
    }
    __syncthreads();
    {
      uint32_t run = 0;
      for (int w = 0; w < kWarps; ++w) {
        const uint32_t c = wcnt[w][threadIdx.x];
        wcnt[w][threadIdx.x] = run;
        run += c;
      }
      tile_tot[threadIdx.x] = run;
    }
    __syncthreads();
#pragma unroll
    for (int r = 0; r < 4; ++r) {
      const uint32_t i = t0 + warp * 128 + r * 32 + lane;
      if (i < e) {
        const uint32_t d = dig[r];
        const uint32_t dst = base[d] + wcnt[warp][d] + rank[r];
        kout[dst] = key[r];
        vout[dst] = val[r];
      }
    }
    __syncthreads();
    base[threadIdx.x] += tile_tot[threadIdx.x];
    for (int w = 0; w < kWarps; ++w) wcnt[w][threadIdx.x] = 0;
    __syncthreads();
  }
}

__global__ void k_segment_starts(const uint32_t* keys, const uint32_t* n_dev, uint32_t n_max,
                                 uint32_t ntiles, uint32_t* start) {
  swr_pdl_entry();
  const uint32_t n = load_n(n_dev, n_max);
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i <= n; i += gridDim.x * blockDim.x) {
    const uint32_t kc = i < n ? keys[i] : ntiles;
    const int64_t kp = i == 0 ? -1 : (int64_t)keys[i - 1];
    for (int64_t t = kp + 1; t <= (int64_t)kc && t <= (int64_t)ntiles; ++t) start[t] = i;
  }
}

}  // namespace

size_t scan_scratch_words(uint32_t) { return kScanBlocks; }

void scan_exclusive(const uint32_t* in, uint32_t* out, const uint32_t* n_dev, uint32_t n_max,
                    uint32_t* total, uint32_t* scratch, cudaStream_t s) {
  const uint32_t chunk = chunk_for(n_max, kScanBlocks);
  swr::launch(k_scan_reduce, kScanBlocks, kThreads, 0, s, in, n_dev, n_max, chunk, scratch);
  swr::launch(k_scan_down, kScanBlocks, kThreads, 0, s, in, out, n_dev, n_max, chunk, scratch, total);
}

size_t sort_scratch_words(uint32_t) { return 2 * 256 * kSortBlocks + 256; }

int radix_sort_pairs(uint32_t* k0, uint32_t* v0, uint32_t* k1, uint32_t* v1, const uint32_t* n_dev,
                     uint32_t n_max, int bits, uint32_t* scratch, cudaStream_t s) {
  const uint32_t chunk = chunk_for(n_max, kSortBlocks);
  uint32_t* hist = scratch;
  uint32_t* off = scratch + 256 * kSortBlocks;
  uint32_t* tot = scratch + 2 * 256 * kSortBlocks;
  int cur = 0;
  for (int shift = 0; shift < bits; shift += 8) {
    uint32_t* ki = cur ? k1 : k0;
    uint32_t* vi = cur ? v1 : v0;
    uint32_t* ko = cur ? k0 : k1;
    uint32_t* vo = cur ? v0 : v1;
    swr::launch(k_radix_hist, kSortBlocks, kThreads, 0, s, ki, n_dev, n_max, chunk, shift, hist, kSortBlocks);
    swr::launch(k_radix_offsets, 32, 256, 0, s, hist, off, tot, kSortBlocks);
    swr::launch(k_radix_scatter, kSortBlocks, kThreads, 0, s, ki, vi, ko, vo, n_dev, n_max, chunk, shift, off, tot);
    cur ^= 1;
  }
  return cur;
}

void segment_starts(const uint32_t* keys, const uint32_t* n_dev, uint32_t n_max, uint32_t ntiles,
                    uint32_t* start, cudaStream_t s) {
  const uint32_t want = (n_max + 1 + 255) / 256;
  const int grid = (int)(want < 8192u ? want : 8192u);
  swr::launch(k_segment_starts, grid, 256, 0, s, keys, n_dev, n_max, ntiles, start);
}

}  // namespace swr
