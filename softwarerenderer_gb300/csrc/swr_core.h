// Host launchers of the generic device primitives (swr_core.cu) and of the pipeline
// stages (swr_stages.cuh, instantiated per shader program).
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>
#include "swr_device.cuh"

namespace swr {

// Blocks used by the fixed-grid scan / sort kernels (each owns a contiguous chunk).
constexpr int kScanBlocks = 304;  // 2 x 152 SMs

// Exclusive prefix sum of in[0..n) into out, where n = min(*n_dev, n_max) when n_dev is
// given (device-resident length) else n_max.  total (device) receives the sum.
// scratch needs scan_scratch_words(n_max) words.  Two kernels: block partial sums, then
// each block prefixes the partials before it and scans its chunk.
size_t scan_scratch_words(uint32_t n_max);
void scan_exclusive(const uint32_t* in, uint32_t* out, const uint32_t* n_dev, uint32_t n_max,
                    uint32_t* total, uint32_t* scratch, cudaStream_t s);

// Stable LSD radix sort of (key, value) pairs by the low `bits` bits of key; three kernels
// per 8-bit pass (block histograms, per-digit offsets, stable scatter).
// n = min(*n_dev, n_max).  Ping-pongs between (k0,v0) and (k1,v1); returns 0 when the
// result ends in (k0, v0), 1 when it ends in (k1, v1).  scratch: sort_scratch_words(n_max).
size_t sort_scratch_words(uint32_t n_max);
int radix_sort_pairs(uint32_t* k0, uint32_t* v0, uint32_t* k1, uint32_t* v1,
                     const uint32_t* n_dev, uint32_t n_max, int bits, uint32_t* scratch,
                     cudaStream_t s);

// start[t] = first index i of sorted keys[0..n) with keys[i] >= t, for t in [0, ntiles].
void segment_starts(const uint32_t* keys, const uint32_t* n_dev, uint32_t n_max,
                    uint32_t ntiles, uint32_t* start, cudaStream_t s);

}  // namespace swr
