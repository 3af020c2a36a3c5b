// shy_math.h -- arithmetic shared by the host side and the CUDA kernels.
//
// Everything here is evaluated with IEEE additions and multiplications in a
// fixed order (on the device through the _rn intrinsics, which are never
// contracted into FMAs; on the host the library is built with
// -ffp-contract=off), so the host and the GPU produce the same bits.
#pragma once

#include <stdint.h>

#if defined(__CUDACC__)
#define SHY_HD __host__ __device__ __forceinline__
#define SHY_ERF_TABLE_QUAL static __device__ __constant__ const
#else
#define SHY_HD static inline
#define SHY_ERF_TABLE_QUAL static const
#endif

#if defined(__CUDACC__)
// Host copies of the tables, for the host-side callers of shy_erf_d.
namespace shy_host_tables {
#undef SHY_ERF_TABLE_QUAL
#define SHY_ERF_TABLE_QUAL static const
#include "shy_erf_table.h"
}  // namespace shy_host_tables
#undef SHY_ERF_TABLE_QUAL
#define SHY_ERF_TABLE_QUAL static __device__ __constant__ const
namespace shy_dev_tables {
#include "shy_erf_table.h"
}  // namespace shy_dev_tables
#else
#include "shy_erf_table.h"
#endif

SHY_HD double shy_dmul(double a, double b) {
#if defined(__CUDA_ARCH__)
  return __dmul_rn(a, b);
#else
  return a * b;
#endif
}
SHY_HD double shy_dadd(double a, double b) {
#if defined(__CUDA_ARCH__)
  return __dadd_rn(a, b);
#else
  return a + b;
#endif
}

// erf in double for the arguments the erosion model uses, accurate to about
// one double ulp (the coefficient generator documents the method).  NaN in,
// NaN out.
SHY_HD double shy_erf_d(double x) {
#if defined(__CUDA_ARCH__)
  using namespace shy_dev_tables;
#elif defined(__CUDACC__)
  using namespace shy_host_tables;
#endif
  if (!(x == x)) return x;
  const double ax = x < 0.0 ? -x : x;
  double r;
  if (ax < 0.5) {
    const double u = shy_dmul(ax, ax);
    double p = shy_erf_small[SHY_ERF_SMALL_TERMS - 1];
    for (int i = SHY_ERF_SMALL_TERMS - 2; i >= 0; --i) p = shy_dadd(shy_dmul(p, u), shy_erf_small[i]);
    r = shy_dmul(ax, p);
  } else if (ax < 4.0) {
    const int s = (int)((ax - 0.5) * 4.0);  // exact: ax - 0.5 and *4 are exact
    const double u = shy_dadd(ax, -(0.625 + 0.25 * s));
    const double* c = shy_erf_seg[s];
    double p = c[SHY_ERF_SEG_DEGREE];
    for (int k = SHY_ERF_SEG_DEGREE - 1; k >= 0; --k) p = shy_dadd(shy_dmul(p, u), c[k]);
    r = p;
  } else {
    r = 1.0;
  }
  return x < 0.0 ? -r : r;
}

// erf rounded to float (almost always the correctly rounded erff).
SHY_HD float shy_erff(float x) { return (float)shy_erf_d((double)x); }

// SplitMix64 finaliser (Steele, Lea, Flood 2014).
SHY_HD uint64_t shy_splitmix64(uint64_t z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// Spawn position of drop `k` of batched cycle `cycle` on an nx-by-ny map:
// x from the low and y from the high half of one SplitMix64 draw.
SHY_HD void shy_spawn_xy(uint64_t seed, uint64_t cycle, uint32_t k, int nx, int ny,
                         int* x, int* y) {
  const uint64_t key = shy_splitmix64(seed) ^ shy_splitmix64((cycle << 32) | (uint64_t)k);
  const uint64_t r = shy_splitmix64(key);
  *x = (int)((uint32_t)r % (uint32_t)nx);
  *y = (int)((uint32_t)(r >> 32) % (uint32_t)ny);
}

// Counter-based uniform in [0, 1) with 24 bits, for the per-cell vegetation
// draws: stream `what` of cell `cell` in step `step`.
SHY_HD float shy_uniform24(uint64_t seed, uint64_t step, uint64_t cell, uint32_t what) {
  const uint64_t r = shy_splitmix64(shy_splitmix64(seed ^ 0x5851F42D4C957F2Dull) ^
                                    shy_splitmix64((step << 36) ^ (cell << 4) ^ what));
  return (float)(uint32_t)(r >> 40) * (1.0f / 16777216.0f);
}

// ---- seeded fractal value noise (the terrain recipe of the workloads) ----
// lowbias32 integer hash (C. Wellons).
SHY_HD uint32_t shy_hash32(uint32_t x) {
  x ^= x >> 16;
  x *= 0x7FEB352Du;
  x ^= x >> 15;
  x *= 0x846CA68Bu;
  x ^= x >> 16;
  return x;
}

SHY_HD double shy_lattice(uint64_t seed, uint32_t octave, int ix, int iy) {
  uint32_t k = shy_hash32((uint32_t)seed ^ shy_hash32((uint32_t)(seed >> 32) + octave * 0x9E3779B9u));
  k = shy_hash32(k ^ (uint32_t)ix);
  k = shy_hash32(k + (uint32_t)iy * 0x85EBCA77u);
  return (double)(k >> 8) * (1.0 / 16777216.0);
}

// Unnormalised fractal sum at cell (x, y) of a map whose longer side is
// `side`: `octaves` octaves of bilinear value noise with smoothstep weights,
// base frequency 4 lattice cells per side, lacunarity 2, gain 0.5.
SHY_HD double shy_value_noise(uint64_t seed, int x, int y, int side, int octaves) {
  double total = 0.0, amp = 1.0, freq = 4.0;
  for (int o = 0; o < octaves; ++o) {
    const double u = shy_dmul((double)x, freq) / (double)side;
    const double v = shy_dmul((double)y, freq) / (double)side;
    const int iu = (int)u, iv = (int)v;  // u, v >= 0: truncation is floor
    const double fu = shy_dadd(u, -(double)iu), fv = shy_dadd(v, -(double)iv);
    const double su = shy_dmul(shy_dmul(fu, fu), shy_dadd(3.0, -shy_dmul(2.0, fu)));
    const double sv = shy_dmul(shy_dmul(fv, fv), shy_dadd(3.0, -shy_dmul(2.0, fv)));
    const double a = shy_lattice(seed, (uint32_t)o, iu, iv);
    const double b = shy_lattice(seed, (uint32_t)o, iu + 1, iv);
    const double c = shy_lattice(seed, (uint32_t)o, iu, iv + 1);
    const double d = shy_lattice(seed, (uint32_t)o, iu + 1, iv + 1);
    const double top = shy_dadd(a, shy_dmul(shy_dadd(b, -a), su));
    const double bot = shy_dadd(c, shy_dmul(shy_dadd(d, -c), su));
    const double val = shy_dadd(top, shy_dmul(shy_dadd(bot, -top), sv));
    total = shy_dadd(total, shy_dmul(amp, val));
    amp = shy_dmul(amp, 0.5);
    freq = shy_dmul(freq, 2.0);
  }
  return total;
}
