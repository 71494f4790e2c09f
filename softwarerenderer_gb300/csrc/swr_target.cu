// Render-target clear: colour (4 or 16 bytes per pixel), depth and the optional per-pixel
// records (drawPixel count, winning primitive) of one target in a single launch with
// 16-byte stores.  The reference leaves clearing to the application (e.g. Box.cpp's
// SDL_FillRect each frame); doing it here saves one fill pass per buffer.
#include <string.h>

#include "../../include/swr_gb300.h"
#include "swr_device.cuh"

namespace {

struct ClearArgs {
  void* buf[4];         // colour, depth, frag_count, winner (null: absent)
  uint32_t bytes_px[4]; // bytes per pixel of each buffer (4 or 16)
  uint4 value[4];       // 16-byte clear pattern of each buffer
  uint64_t npx;
};

__global__ void k_clear_target(const ClearArgs a) {
  const uint64_t stride = (uint64_t)gridDim.x * blockDim.x;
  const uint64_t t0 = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x;
#pragma unroll
  for (int k = 0; k < 4; ++k) {
    if (!a.buf[k]) continue;
    const uint64_t bytes = a.npx * a.bytes_px[k];
    const uint64_t vec = bytes / 16;
    uint4* v = (uint4*)a.buf[k];
    for (uint64_t i = t0; i < vec; i += stride) v[i] = a.value[k];
    // a 4-byte buffer whose pixel count is not a multiple of 4 leaves up to 3 words
    uint32_t* w = (uint32_t*)a.buf[k];
    for (uint64_t i = vec * 4 + t0; i < bytes / 4; i += stride) w[i] = a.value[k].x;
  }
}

uint4 splat(uint32_t v) { return make_uint4(v, v, v, v); }

}  // namespace

extern "C" int swr_clear_target(const struct SwrUniforms* u, int color_bytes, const void* clear_color,
                                float clear_depth, void* stream) {
  if (!u || !u->color || u->width <= 0 || u->height <= 0 || (color_bytes != 4 && color_bytes != 16) ||
      !clear_color)
    return SWR_EINVAL;
  if (((uintptr_t)u->color | (uintptr_t)u->depth | (uintptr_t)u->frag_count | (uintptr_t)u->winner) & 15u)
    return SWR_EINVAL;  // 16-byte stores
  ClearArgs a;
  memset(&a, 0, sizeof(a));
  a.npx = (uint64_t)u->width * (uint64_t)u->height;
  a.buf[0] = u->color;
  a.bytes_px[0] = (uint32_t)color_bytes;
  uint32_t cv[4];
  if (color_bytes == 4) {
    memcpy(&cv[0], clear_color, 4);
    cv[1] = cv[2] = cv[3] = cv[0];
  } else {
    memcpy(cv, clear_color, 16);
  }
  a.value[0] = make_uint4(cv[0], cv[1], cv[2], cv[3]);
  uint32_t dbits;
  memcpy(&dbits, &clear_depth, 4);
  a.buf[1] = u->depth;
  a.bytes_px[1] = 4;
  a.value[1] = splat(dbits);
  a.buf[2] = u->frag_count;
  a.bytes_px[2] = 4;
  a.value[2] = splat(0u);
  a.buf[3] = u->winner;
  a.bytes_px[3] = 4;
  a.value[3] = splat(0xffffffffu);
  const uint64_t work = a.npx * (uint64_t)color_bytes / 16 + 1;
  const int grid = (int)(work / 256 + 1 < 4096 ? work / 256 + 1 : 4096);
  k_clear_target<<<grid, 256, 0, (cudaStream_t)stream>>>(a);
  return cudaGetLastError() == cudaSuccess ? SWR_OK : SWR_ECUDA;
}
