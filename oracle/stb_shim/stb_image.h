// Stand-in for stb_image.h (the single-header image library the reference's
// src/photon/pbrt/image_loader.cpp includes; it is not part of the reference
// checkout).  TEST INFRASTRUCTURE ONLY: it lets image_loader.cpp compile
// unmodified into oracle/_ref, so the reference's own PFM reader
// (image_loader.cpp:20-74) runs; every stb format (PNG, JPEG, TGA, BMP, HDR,
// PNM) reports "cannot load", as the product's reader does.
#pragma once

// the real header brings these in for its float conversions
#include <cmath>
#include <cstdlib>
#include <cstring>

static inline float *stbi_loadf(char const *, int *x, int *y, int *comp, int)
{
  *x = *y = *comp = 0;
  return nullptr;
}

static inline void stbi_image_free(void *) {}
