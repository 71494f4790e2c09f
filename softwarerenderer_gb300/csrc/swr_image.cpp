// Headless presentation: the render target written to an image file.  The reference's
// examples present through an SDL window surface (Box.cpp:170-171, 315); here a target in
// device (or host) memory is written as binary PPM (P6) or PNG, 8 bits per channel RGB.
// The PNG encoder stores the scanlines in uncompressed deflate blocks (RFC 1951, BTYPE 00)
// inside a zlib stream (RFC 1950, Adler-32) with CRC-32 chunk checksums (PNG spec,
// ISO/IEC 15948), so it needs no compression library.
#include <stdio.h>
#include <string.h>

#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "../../include/swr_gb300.h"

namespace {

struct Crc32Table {
  uint32_t t[256];
  Crc32Table() {
    for (uint32_t i = 0; i < 256; ++i) {
      uint32_t c = i;
      for (int k = 0; k < 8; ++k) c = (c & 1) ? 0xedb88320u ^ (c >> 1) : c >> 1;
      t[i] = c;
    }
  }
};

uint32_t crc32_update(uint32_t crc, const unsigned char* p, size_t n) {
  static const Crc32Table tab;  // initialised once, thread-safe (C++11 function-local static)
  const uint32_t* table = tab.t;
  crc = ~crc;
  for (size_t i = 0; i < n; ++i) crc = table[(crc ^ p[i]) & 0xff] ^ (crc >> 8);
  return ~crc;
}

void put32(std::string& s, uint32_t v) {
  s.push_back((char)(v >> 24));
  s.push_back((char)(v >> 16));
  s.push_back((char)(v >> 8));
  s.push_back((char)v);
}

void chunk(std::string& out, const char* type, const std::string& data) {
  put32(out, (uint32_t)data.size());
  std::string td(type, 4);
  td += data;
  out += td;
  put32(out, crc32_update(0, (const unsigned char*)td.data(), td.size()));
}

std::string png(const std::vector<unsigned char>& rgb, int w, int h) {
  std::string raw;  // filter byte 0 + RGB scanline per row
  raw.reserve((size_t)h * (1 + 3 * (size_t)w));
  for (int y = 0; y < h; ++y) {
    raw.push_back(0);
    raw.append((const char*)&rgb[(size_t)y * 3 * w], 3 * (size_t)w);
  }
  std::string z;
  z.push_back((char)0x78);
  z.push_back((char)0x01);
  uint32_t a = 1, b = 0;
  for (unsigned char c : raw) {
    a = (a + c) % 65521u;
    b = (b + a) % 65521u;
  }
  size_t off = 0;
  do {
    const size_t n = raw.size() - off < 65535 ? raw.size() - off : 65535;
    z.push_back(off + n == raw.size() ? 1 : 0);  // BFINAL, BTYPE 00
    z.push_back((char)(n & 0xff));
    z.push_back((char)(n >> 8));
    z.push_back((char)(~n & 0xff));
    z.push_back((char)((~n >> 8) & 0xff));
    z.append(raw, off, n);
    off += n;
  } while (off < raw.size());
  put32(z, (b << 16) | a);
  std::string out("\x89PNG\r\n\x1a\n", 8);
  std::string ihdr;
  put32(ihdr, (uint32_t)w);
  put32(ihdr, (uint32_t)h);
  ihdr += std::string("\x08\x02\x00\x00\x00", 5);  // 8-bit RGB, deflate, filter 0, no interlace
  chunk(out, "IHDR", ihdr);
  chunk(out, "IDAT", z);
  chunk(out, "IEND", std::string());
  return out;
}

unsigned char to8(float v) {
  if (!(v > 0.0f)) return 0;
  if (v >= 1.0f) return 255;
  return (unsigned char)(v * 255.0f + 0.5f);
}

}  // namespace

extern "C" int swr_write_image(const char* path, const void* pixels, int width, int height, int format) {
  if (!path || !pixels || width <= 0 || height <= 0 || (uint64_t)width * (uint64_t)height > (1ull << 31))
    return SWR_EINVAL;
  if (format != SWR_PIXELS_RGBA8 && format != SWR_PIXELS_XRGB8 && format != SWR_PIXELS_RGBA32F) return SWR_EINVAL;
  const std::string p(path);
  const bool is_png = p.size() >= 4 && (p.compare(p.size() - 4, 4, ".png") == 0 || p.compare(p.size() - 4, 4, ".PNG") == 0);
  const bool is_ppm = p.size() >= 4 && (p.compare(p.size() - 4, 4, ".ppm") == 0 || p.compare(p.size() - 4, 4, ".PPM") == 0);
  if (!is_png && !is_ppm) return SWR_EINVAL;
  const size_t n = (size_t)width * (size_t)height;
  const size_t bytes = n * (format == SWR_PIXELS_RGBA32F ? 16 : 4);
  // device or host source: cudaMemcpyDefault needs unified addressing, which a plain host
  // pointer also satisfies; without a GPU fall back to reading host memory directly
  std::vector<unsigned char> src(bytes);
  cudaPointerAttributes at;
  const bool dev = cudaPointerGetAttributes(&at, pixels) == cudaSuccess && at.type == cudaMemoryTypeDevice;
  if (!dev) cudaGetLastError();
  if (dev) {
    if (cudaMemcpy(src.data(), pixels, bytes, cudaMemcpyDeviceToHost) != cudaSuccess) {
      cudaGetLastError();
      return SWR_ECUDA;
    }
  } else {
    memcpy(src.data(), pixels, bytes);
  }
  std::vector<unsigned char> rgb(3 * n);
  for (size_t i = 0; i < n; ++i) {
    if (format == SWR_PIXELS_RGBA32F) {
      float c[4];
      memcpy(c, &src[16 * i], 16);
      for (int k = 0; k < 3; ++k) rgb[3 * i + k] = to8(c[k]);
    } else {
      uint32_t c;
      memcpy(&c, &src[4 * i], 4);
      const int sr = format == SWR_PIXELS_RGBA8 ? 0 : 16, sb = format == SWR_PIXELS_RGBA8 ? 16 : 0;
      rgb[3 * i + 0] = (unsigned char)(c >> sr);
      rgb[3 * i + 1] = (unsigned char)(c >> 8);
      rgb[3 * i + 2] = (unsigned char)(c >> sb);
    }
  }
  std::string out;
  if (is_png) {
    out = png(rgb, width, height);
  } else {
    out = "P6\n" + std::to_string(width) + " " + std::to_string(height) + "\n255\n";
    out.append((const char*)rgb.data(), rgb.size());
  }
  FILE* f = fopen(path, "wb");
  if (!f) return SWR_EINVAL;
  const bool ok = fwrite(out.data(), 1, out.size(), f) == out.size();
  return (fclose(f) == 0 && ok) ? SWR_OK : SWR_EINVAL;
}
