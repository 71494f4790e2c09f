// Mip chain of a 0x00RRGGBB texture for the mip-mapped sampler (PsTexMip): level 0 with
// the alpha byte cleared, then each level box-filtered from the one before
// (Texture::generateMipmaps, Texture.h:220-293): texel (x, y) of a max(1, w/2) x
// max(1, h/2) level is the per-channel (p00 + p10 + p01 + p11) >> 2 of the 2 x 2 source
// texels at (2x, 2y), where a neighbour past an odd edge is replaced by p00.  Integer
// work; one launch per level, one thread per output texel.
#include "../../include/swr_gb300.h"
#include "swr_device.cuh"

namespace {

__global__ void k_mip_base(const uint32_t* __restrict__ src, uint32_t* __restrict__ dst, uint64_t n) {
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x)
    dst[i] = src[i] & 0x00ffffffu;
}

__global__ void k_mip_level(const uint32_t* __restrict__ src, int sw, int sh, uint32_t* __restrict__ dst, int dw,
                            int dh) {
  const uint64_t n = (uint64_t)dw * (uint64_t)dh;
  for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n; i += (uint64_t)gridDim.x * blockDim.x) {
    const int x = (int)(i % (uint64_t)dw), y = (int)(i / (uint64_t)dw);
    const int x0 = 2 * x, y0 = 2 * y;  // < sw, sh: dw = max(1, sw / 2)
    const bool rx = x0 + 1 < sw, ry = y0 + 1 < sh;
    const size_t w = (size_t)sw;
    const uint32_t p00 = src[(size_t)y0 * w + x0];
    const uint32_t p10 = rx ? src[(size_t)y0 * w + x0 + 1] : p00;
    const uint32_t p01 = ry ? src[(size_t)(y0 + 1) * w + x0] : p00;
    const uint32_t p11 = (rx && ry) ? src[(size_t)(y0 + 1) * w + x0 + 1] : p00;
    uint32_t out = 0;
#pragma unroll
    for (int s = 16; s >= 0; s -= 8) {
      const uint32_t c = ((p00 >> s) & 255u) + ((p10 >> s) & 255u) + ((p01 >> s) & 255u) + ((p11 >> s) & 255u);
      out |= (c >> 2) << s;
    }
    dst[i] = out;
  }
}

int grid_for(uint64_t n) {
  const uint64_t g = (n + 255) / 256;
  return (int)(g < 4096 ? (g ? g : 1) : 4096);
}

}  // namespace

extern "C" int swr_mip_chain_size(int width, int height, int* levels, uint64_t* texels) {
  if (width <= 0 || height <= 0) return SWR_EINVAL;
  int w = width, h = height, n = 1;
  uint64_t t = (uint64_t)w * (uint64_t)h;
  while (w > 1 || h > 1) {
    w = w / 2 > 1 ? w / 2 : 1;
    h = h / 2 > 1 ? h / 2 : 1;
    t += (uint64_t)w * (uint64_t)h;
    ++n;
  }
  if (levels) *levels = n;
  if (texels) *texels = t;
  return SWR_OK;
}

extern "C" int swr_build_mip_chain(const uint32_t* base, int width, int height, uint32_t* chain, void* stream) {
  if (!base || !chain || width <= 0 || height <= 0) return SWR_EINVAL;
  if ((uint64_t)width * (uint64_t)height >= (1ull << 40)) return SWR_EINVAL;
  cudaStream_t s = (cudaStream_t)stream;
  const uint64_t n0 = (uint64_t)width * (uint64_t)height;
  k_mip_base<<<grid_for(n0), 256, 0, s>>>(base, chain, n0);
  const uint32_t* src = chain;
  uint32_t* dst = chain + n0;
  int w = width, h = height;
  while (w > 1 || h > 1) {
    const int nw = w / 2 > 1 ? w / 2 : 1, nh = h / 2 > 1 ? h / 2 : 1;
    const uint64_t n = (uint64_t)nw * (uint64_t)nh;
    k_mip_level<<<grid_for(n), 256, 0, s>>>(src, w, h, dst, nw, nh);
    src = dst;
    dst += n;
    w = nw;
    h = nh;
  }
  return cudaGetLastError() == cudaSuccess ? SWR_OK : SWR_ECUDA;
}
