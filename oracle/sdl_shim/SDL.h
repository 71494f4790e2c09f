// Test infrastructure only: the memory-surface part of SDL2's API that the reference's
// example texture (src/examples/Texture.h) uses, so that the reference's own sampler and
// mip-chain code compile into the oracle harness (oracle/ref_harness.cpp).  A surface is a
// plain host image; there is no video subsystem, window, renderer or pixel-format
// conversion here, and no SDL library is linked.  Surfaces hold 32-bit pixels; a blit
// copies between surfaces of the same size and channel masks (the only blit Texture.h
// makes: its base-level copy) and fails otherwise.
#pragma once
#include <algorithm>  // std::clamp, which Texture.h uses without including it
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

typedef uint8_t Uint8;
typedef uint32_t Uint32;

struct SDL_Rect;

typedef struct SDL_Surface {
  Uint32 flags;
  int w, h;
  int pitch;     // bytes per row
  void* pixels;
  Uint32 Rmask, Gmask, Bmask, Amask;
} SDL_Surface;

inline SDL_Surface* SDL_CreateRGBSurface(Uint32 flags, int width, int height, int depth, Uint32 Rmask, Uint32 Gmask,
                                         Uint32 Bmask, Uint32 Amask) {
  if (depth != 32 || width <= 0 || height <= 0) return nullptr;
  SDL_Surface* s = (SDL_Surface*)calloc(1, sizeof(SDL_Surface));
  if (!s) return nullptr;
  s->flags = flags;
  s->w = width;
  s->h = height;
  s->pitch = width * 4;
  s->pixels = calloc((size_t)width * (size_t)height, 4);
  s->Rmask = Rmask;
  s->Gmask = Gmask;
  s->Bmask = Bmask;
  s->Amask = Amask;
  if (!s->pixels) {
    free(s);
    return nullptr;
  }
  return s;
}

inline void SDL_FreeSurface(SDL_Surface* s) {
  if (!s) return;
  free(s->pixels);
  free(s);
}

inline int SDL_LockSurface(SDL_Surface* s) { return s ? 0 : -1; }
inline void SDL_UnlockSurface(SDL_Surface*) {}

// Whole-surface copy between surfaces of equal size and masks (both rectangles NULL).
inline int SDL_BlitSurface(SDL_Surface* src, const SDL_Rect* srcrect, SDL_Surface* dst, SDL_Rect* dstrect) {
  if (!src || !dst || srcrect || dstrect || src->w != dst->w || src->h != dst->h || src->Rmask != dst->Rmask ||
      src->Gmask != dst->Gmask || src->Bmask != dst->Bmask)
    return -1;
  for (int y = 0; y < src->h; ++y)
    memcpy((char*)dst->pixels + (size_t)y * dst->pitch, (const char*)src->pixels + (size_t)y * src->pitch,
           (size_t)src->w * 4);
  return 0;
}

inline const char* SDL_GetError() { return "memory surface error"; }
