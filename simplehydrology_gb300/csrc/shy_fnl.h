// shy_fnl.h -- the reference's own terrain: quad::map::init's height noise.
//
// quad::map::init (source/cellpool.h:323-411) sums eight layers of
// FastNoiseLite noise (the single-header library the reference vendors as
// source/include/FastNoiseLite.h), OpenSimplex2 in 3D with FBm fractals,
// and min-max normalises the sum.  Layer o samples the noise at frequency
// 2^o and weighs it by 0.6^(o+1); the world seed enters only as the third
// coordinate, SEED % 10000, while the library's own noise seed keeps its
// default 1337.  The library's settings at that point are its defaults:
// three FBm octaves, lacunarity 2, gain 0.5, weighted strength 0, fractal
// bounding 1 / 1.75, and the OpenSimplex2 3D rotation.
//
// These functions restate that computation step for step in float, in the
// library's operation order, so that with multiply-add contraction off
// (the whole library builds with --fmad=false and the host with
// -ffp-contract=off) the device gives the reference's bits.  Integer hashes
// use unsigned 32-bit arithmetic, which wraps exactly as the library's
// signed arithmetic does on every target.
//
// shy_fnl_os2 follows FastNoiseLite's SingleOpenSimplex2 (3D) closely, as
// bit parity with the reference's terrain requires, so this file is a
// derivative of that library and carries its licence:
//
//   MIT License
//
//   Copyright(c) 2020 Jordan Peck (jordan.me2@gmail.com)
//   Copyright(c) 2020 Contributors
//
//   Permission is hereby granted, free of charge, to any person obtaining a
//   copy of this software and associated documentation files(the
//   "Software"), to deal in the Software without restriction, including
//   without limitation the rights to use, copy, modify, merge, publish,
//   distribute, sublicense, and / or sell copies of the Software, and to
//   permit persons to whom the Software is furnished to do so, subject to
//   the following conditions :
//
//   The above copyright notice and this permission notice shall be included
//   in all copies or substantial portions of the Software.
//
//   THE SOFTWARE IS PROVIDED "AS IS", WITHOUT WARRANTY OF ANY KIND, EXPRESS
//   OR IMPLIED, INCLUDING BUT NOT LIMITED TO THE WARRANTIES OF
//   MERCHANTABILITY, FITNESS FOR A PARTICULAR PURPOSE AND NONINFRINGEMENT.
//   IN NO EVENT SHALL THE AUTHORS OR COPYRIGHT HOLDERS BE LIABLE FOR ANY
//   CLAIM, DAMAGES OR OTHER LIABILITY, WHETHER IN AN ACTION OF CONTRACT,
//   TORT OR OTHERWISE, ARISING FROM, OUT OF OR IN CONNECTION WITH THE
//   SOFTWARE OR THE USE OR OTHER DEALINGS IN THE SOFTWARE.
#pragma once

#include <stdint.h>

#include "shy_math.h"

// The library's coordinate-hash primes and multiplier.
#define SHY_FNL_PRIME_X 501125321u
#define SHY_FNL_PRIME_Y 1136930381u
#define SHY_FNL_PRIME_Z 1720413743u
#define SHY_FNL_HASH_MUL 0x27d4eb2du

// Gradient g (0..63) of 3D OpenSimplex2: the twelve cube-edge directions, in
// the library's order, five times over, then four of them again (directions
// 8, 1, 9, 3).  Direction e has a zero in component e / 4 and signs
// (-1)^(e & 1), (-1)^((e >> 1) & 1) on the other two, in order.
SHY_HD void shy_fnl_grad(int g, float* gx, float* gy, float* gz) {
  int e = g < 60 ? g % 12 : (g == 60 ? 8 : (g == 61 ? 1 : (g == 62 ? 9 : 3)));
  const float a = (e & 1) ? -1.0f : 1.0f, b = (e & 2) ? -1.0f : 1.0f;
  const int zero = e >> 2;
  *gx = zero == 0 ? 0.0f : a;
  *gy = zero == 0 ? a : (zero == 1 ? 0.0f : b);
  *gz = zero == 2 ? 0.0f : b;
}

// Gradient dot product at a primed lattice point.
SHY_HD float shy_fnl_grad_coord(uint32_t seed, uint32_t xp, uint32_t yp, uint32_t zp, float xd, float yd,
                                float zd) {
  uint32_t h = (seed ^ xp ^ yp ^ zp) * SHY_FNL_HASH_MUL;
  h ^= h >> 15;  // the bits kept below do not depend on the shift's sign fill
  const int g = (int)((h & 252u) >> 2);
  float gx, gy, gz;
  shy_fnl_grad(g, &gx, &gy, &gz);
  return xd * gx + yd * gy + zd * gz;
}

// The library's rounding of a coordinate to the nearest lattice point.
SHY_HD int shy_fnl_round(float f) { return f >= 0 ? (int)(f + 0.5f) : (int)(f - 0.5f); }

// One octave of 3D OpenSimplex2 at rotated coordinates: two offset cube
// lattices, each contributing its nearest vertex and the next one along the
// coordinate of largest distance.
SHY_HD float shy_fnl_os2(uint32_t seed, float x, float y, float z) {
  int ri = shy_fnl_round(x), rj = shy_fnl_round(y), rk = shy_fnl_round(z);
  float x0 = x - (float)ri, y0 = y - (float)rj, z0 = z - (float)rk;
  int sx = (int)(-1.0f - x0) | 1, sy = (int)(-1.0f - y0) | 1, sz = (int)(-1.0f - z0) | 1;
  float ax0 = (float)sx * -x0, ay0 = (float)sy * -y0, az0 = (float)sz * -z0;
  uint32_t i = (uint32_t)ri * SHY_FNL_PRIME_X, j = (uint32_t)rj * SHY_FNL_PRIME_Y, k = (uint32_t)rk * SHY_FNL_PRIME_Z;
  float value = 0.0f;
  float a = (0.6f - x0 * x0) - (y0 * y0 + z0 * z0);
  for (int l = 0; l < 2; ++l) {
    if (a > 0) value += (a * a) * (a * a) * shy_fnl_grad_coord(seed, i, j, k, x0, y0, z0);
    float b = a + 1;
    uint32_t i1 = i, j1 = j, k1 = k;
    float x1 = x0, y1 = y0, z1 = z0;
    if (ax0 >= ay0 && ax0 >= az0) {
      x1 += (float)sx;
      b -= (float)(sx * 2) * x1;
      i1 -= (uint32_t)sx * SHY_FNL_PRIME_X;
    } else if (ay0 > ax0 && ay0 >= az0) {
      y1 += (float)sy;
      b -= (float)(sy * 2) * y1;
      j1 -= (uint32_t)sy * SHY_FNL_PRIME_Y;
    } else {
      z1 += (float)sz;
      b -= (float)(sz * 2) * z1;
      k1 -= (uint32_t)sz * SHY_FNL_PRIME_Z;
    }
    if (b > 0) value += (b * b) * (b * b) * shy_fnl_grad_coord(seed, i1, j1, k1, x1, y1, z1);
    if (l == 1) break;
    // the second lattice, offset by half a cell
    ax0 = 0.5f - ax0;
    ay0 = 0.5f - ay0;
    az0 = 0.5f - az0;
    x0 = (float)sx * ax0;
    y0 = (float)sy * ay0;
    z0 = (float)sz * az0;
    a += (0.75f - ax0) - (ay0 + az0);
    i += sx < 0 ? SHY_FNL_PRIME_X : 0u;
    j += sy < 0 ? SHY_FNL_PRIME_Y : 0u;
    k += sz < 0 ? SHY_FNL_PRIME_Z : 0u;
    sx = -sx;
    sy = -sy;
    sz = -sz;
    seed = ~seed;
  }
  return value * 32.69428253173828125f;
}

// FastNoiseLite GetNoise(x, y, z) with the settings init uses: frequency
// `freq`, the OpenSimplex2 3D rotation, three FBm octaves from noise seed
// 1337 (lacunarity 2, gain 0.5, weighted strength 0, so an octave's weight
// only halves), summed with the fractal bounding 1 / 1.75.
SHY_HD float shy_fnl_noise(float x, float y, float z, float freq) {
  x *= freq;
  y *= freq;
  z *= freq;
  const float r3 = (float)(2.0 / 3.0);
  const float r = (x + y + z) * r3;
  x = r - x;
  y = r - y;
  z = r - z;
  float sum = 0.0f, amp = 1.0f / 1.75f;
  uint32_t seed = 1337u;
  for (int o = 0; o < 3; ++o) {
    const float n = shy_fnl_os2(seed++, x, y, z);
    sum += n * amp;
    x *= 2.0f;
    y *= 2.0f;
    z *= 2.0f;
    amp *= 0.5f;
  }
  return sum;
}

// The unnormalised height init gives cell (x, y) of an nx x ny map
// (source/cellpool.h:354-375): layer o at frequency 2^o weighs
// scale[o] (0.6, then each times 0.6 in double, rounded to float).
SHY_HD float shy_fnl_height(int x, int y, int nx, int ny, float zc, const float* scale) {
  const float px = (float)x / (float)nx, py = (float)y / (float)ny;
  float h = 0.0f, freq = 1.0f;
  for (int o = 0; o < 8; ++o) {
    h += scale[o] * shy_fnl_noise(px, py, zc, freq);
    freq *= 2.0f;
  }
  return h;
}

// The eight layer weights: 0.6f, then scale *= 0.6 with the double 0.6.
SHY_HD void shy_fnl_scales(float* scale) {
  float s = 0.6f;
  for (int o = 0; o < 8; ++o) {
    scale[o] = s;
    s = (float)((double)s * 0.6);
  }
}

// The world seed's noise coordinate: (float)(SEED % 10000), C remainder.
SHY_HD float shy_fnl_zcoord(int32_t seed) { return (float)(seed % 10000); }
