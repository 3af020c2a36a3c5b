// shy_math.h -- arithmetic shared by the host side and the CUDA kernels.
//
// Everything here is evaluated with IEEE additions and multiplications in a
// fixed order (on the device through the _rn intrinsics, which are never
// contracted into FMAs; on the host the library is built with
// -ffp-contract=off), so the host and the GPU produce the same bits.
#pragma once

#include <math.h>
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

// ---- integer restatements of three roundings -----------------------------
// The reference evaluates these in FP64, which the GPU runs far slower than
// FP32 and integer arithmetic.  Each function gives exactly the bits of the
// expression named, with integer arithmetic only; oracle/emulation_check.c
// verifies them over every normal float.  They are the definition the host,
// the oracle and the streaming kernels use.  The lock-step kernel converts
// between 32.32 and float on the hardware int64 <-> float converters instead
// (shy_unq_dev, shy_q32_dev in shy_device.cuh), which give the same bits with
// a shorter latency.

#if defined(__CUDA_ARCH__)
#define SHY_CLZ64(x) __clzll((long long)(x))
#define SHY_MULHI64(a, b) __umul64hi((a), (b))
#define SHY_AS_UINT(f) __float_as_uint(f)
#define SHY_AS_FLOAT(u) __uint_as_float(u)
#else
#include <string.h>
static inline uint32_t shy_as_uint_h(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }
static inline float shy_as_float_h(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
#define SHY_CLZ64(x) __builtin_clzll((unsigned long long)(x))
#define SHY_MULHI64(a, b) ((uint64_t)(((unsigned __int128)(a) * (unsigned __int128)(b)) >> 64))
#define SHY_AS_UINT(f) shy_as_uint_h(f)
#define SHY_AS_FLOAT(u) shy_as_float_h(u)
#endif

// x + y = s + e exactly (Knuth's TwoSum).
SHY_HD void shy_two_sum(float a, float b, float* s, float* e) {
  const float t = a + b;
  const float bb = t - a;
  *e = (a - (t - bb)) + (b - bb);
  *s = t;
}

// shy_erff in float arithmetic.  The polynomial shy_erf_d evaluates is
// evaluated again in float-float arithmetic (TwoSum and the FMA-based exact
// product; coefficients as float pairs), to about 2^-42 relative.  Rounded to
// float, that gives shy_erff's result except within 2^-37 of a rounding
// midpoint, where shy_erf_d itself decides; tiny arguments take shy_erf_d
// too.  Equal to shy_erff for every float (shy_check_conversions compares
// all 2^32 on the device); the GPU's FP64 unit is far slower than this.
SHY_HD float shy_erff_ff(float x) {
#if defined(__CUDA_ARCH__)
  using namespace shy_dev_tables;
#elif defined(__CUDACC__)
  using namespace shy_host_tables;
#endif
  if (!(x == x) || x == 0.0f) return x;
  const float ax = x < 0.0f ? -x : x;
  if (ax >= 4.0f) return x < 0.0f ? -1.0f : 1.0f;
  if (ax < 8.673617379884035e-19f) return shy_erff(x);  // 2^-60
  float uh, ul;
  const float(*c)[2];
  int n;
  if (ax < 0.5f) {  // x * P(x^2)
    uh = ax * ax;
    ul = fmaf(ax, ax, -uh);
    c = shy_erf_small_f;
    n = SHY_ERF_SMALL_TERMS - 1;
  } else {  // P(x - centre) on the segment (the subtraction is exact)
    const int sg = (int)((ax - 0.5f) * 4.0f);
    uh = ax - (0.625f + 0.25f * (float)sg);
    ul = 0.0f;
    c = shy_erf_seg_f[sg];
    n = SHY_ERF_SEG_DEGREE;
  }
  float ph = c[n][0], pl = c[n][1];
  for (int k = n - 1; k >= 0; --k) {  // p = p * u + c[k]
    const float th = ph * uh;
    const float te = fmaf(ph, uh, -th) + (pl * uh + ph * ul);
    float sh, se;
    shy_two_sum(th, c[k][0], &sh, &se);
    se = se + (te + c[k][1]);
    ph = sh + se;
    pl = se - (ph - sh);
  }
  if (ax < 0.5f) {
    const float rh = ph * ax;
    const float re = fmaf(ph, ax, -rh) + pl * ax;
    ph = rh + re;
    pl = re - (ph - rh);
  }
  // r = the float nearest ph + pl; e = the rest, exactly
  float r, e;
  shy_two_sum(ph, pl, &r, &e);
  const uint32_t ru = SHY_AS_UINT(r);
  float half = 0.5f * SHY_AS_FLOAT((ru & 0x7F800000u) - (23u << 23));  // half an ulp of r (r >= 2^-61)
  if (e < 0.0f && (ru & 0x7FFFFFu) == 0u) half *= 0.5f;  // below a power of two the ulp halves
  if ((e < 0.0f ? -e : e) > half * (1.0f - 1.220703125e-4f)) return shy_erff(x);  // within 2^-13 half-ulp
  return x < 0.0f ? -r : r;
}

// Round x (> 0) to nearest-even after dropping its `cut` low bits (cut >= 1);
// `sticky` says whether nonzero bits were already dropped below x.
SHY_HD uint64_t shy_rne_drop(uint64_t x, int cut, int sticky) {
  const uint64_t keep = x >> cut;
  const uint64_t rest = x & ((1ull << cut) - 1ull);
  const uint64_t half = 1ull << (cut - 1);
  const int up = rest > half || (rest == half && (sticky || (keep & 1ull)));
  return (keep + (uint64_t)up) << cut;
}

// llrintf(v * 2^32): v in 32.32 fixed point, round half to even.  |v| < 2^31.
SHY_HD int64_t shy_q32(float v) {
  const uint32_t u = SHY_AS_UINT(v);
  const int ef = (int)((u >> 23) & 0xFFu);
  uint64_t m = u & 0x7FFFFFu;
  int e;  // v = m * 2^e
  if (ef == 0) {
    e = -149;
  } else {
    m |= 0x800000u;
    e = ef - 150;
  }
  const int s = -(e + 32);  // v * 2^32 = m * 2^(e + 32)
  uint64_t r;
  if (s <= 0) {
    r = m << (-s);
  } else if (s > 25) {
    r = 0;  // |v * 2^32| < 1/2
  } else {
    const uint64_t keep = m >> s, rest = m & ((1ull << s) - 1ull), half = 1ull << (s - 1);
    r = keep + (uint64_t)(rest > half || (rest == half && (keep & 1ull)));
  }
  return (u >> 31) ? -(int64_t)r : (int64_t)r;
}

// (float)((double)q * 2^-32): a 32.32 fixed-point value rounded to float.
// |q| < 2^53, where the double product is exact and this is one rounding.
SHY_HD float shy_unq(int64_t q) {
  if (q == 0) return 0.0f;
  const uint32_t sign = q < 0 ? 0x80000000u : 0u;
  uint64_t a = q < 0 ? (uint64_t)(-q) : (uint64_t)q;
  int lead = 63 - SHY_CLZ64(a);
  if (lead > 23) {
    a = shy_rne_drop(a, lead - 23, 0);
    lead = 63 - SHY_CLZ64(a);
  }
  // value = a * 2^-32, leading bit `lead`; biased exponent lead - 32 + 127
  const int be = lead + 95;
  if (be <= 0) {  // subnormal result: |q| * 2^-32 < 2^-126 cannot happen for |q| >= 1
    return 0.0f;
  }
  const uint64_t mant = lead >= 23 ? (a >> (lead - 23)) : (a << (23 - lead));
  return SHY_AS_FLOAT(sign | ((uint32_t)be << 23) | ((uint32_t)mant & 0x7FFFFFu));
}

// (float)((double)s / (1.0 - (double)evap)) of the reference's evaporation
// (source/water.h:135), for the evaporation constant described by `ev`.
typedef struct shy_evap {
  uint64_t nc;    // 1 - evap = nc * 2^-k exactly
  uint64_t inv;   // floor((2^64 - 1) / nc)
  uint64_t d;     // evap = d * 2^-k
  int k;
  int fast;       // 0: use the double expression
  double c;       // 1 - (double)evap
  float ih, il;   // 1 / c as a float pair: ih + il to about 2^-48
  float ch, cl;   // c as a float pair
} shy_evap;

SHY_HD shy_evap shy_evap_make(float evap) {
  shy_evap E;
  E.c = 1.0 - (double)evap;
  const double inv = 1.0 / E.c;
  E.ih = (float)inv;
  E.il = (float)(inv - (double)E.ih);
  E.ch = (float)E.c;
  E.cl = (float)(E.c - (double)E.ch);
  E.fast = 0;
  E.nc = E.inv = E.d = 0;
  E.k = 0;
  const uint32_t u = SHY_AS_UINT(evap);
  const int ef = (int)((u >> 23) & 0xFFu);
  if ((u >> 31) == 0 && ef > 0 && ef < 127) {  // 0 < evap < 1, normal
    const int k = 150 - ef;                     // evap = d * 2^-k
    if (k <= 34) {
      E.k = k;
      E.d = (u & 0x7FFFFFu) | 0x800000u;
      E.nc = (1ull << k) - E.d;
      E.inv = ~0ull / E.nc;
      E.fast = 1;
    }
  }
  return E;
}

SHY_HD float shy_evap_div(float s, const shy_evap* E) {
  const uint32_t u = SHY_AS_UINT(s);
  const int ef = (int)((u >> 23) & 0xFFu);
  if (!E->fast || (u >> 31) || ef == 0 || ef > 252) return (float)((double)s / E->c);
  // s = m * 2^(ef-150); s / c = s + s * d / nc
  const uint64_t m = (u & 0x7FFFFFu) | 0x800000u;
  const uint64_t y = m * E->d;  // < 2^48
  uint64_t qi = SHY_MULHI64(y, E->inv);
  uint64_t r = y - qi * E->nc;
  while (r >= E->nc) { r -= E->nc; ++qi; }
  const uint64_t rs = r << 30;  // r < nc < 2^34
  uint64_t f = SHY_MULHI64(rs, E->inv);
  uint64_t r2 = rs - f * E->nc;
  while (r2 >= E->nc) { r2 -= E->nc; ++f; }
  // exact quotient = ((m + qi) * 2^30 + f + r2 / nc) * 2^(ef - 180)
  uint64_t x = ((m + qi) << 30) | f;
  int lead = 63 - SHY_CLZ64(x);
  x = shy_rne_drop(x, lead - 52, r2 != 0);  // to double: 53 significant bits
  lead = 63 - SHY_CLZ64(x);
  x = shy_rne_drop(x, lead - 23, 0);         // then to float: 24 bits
  lead = 63 - SHY_CLZ64(x);
  const int be = ef + lead - 53;
  const uint64_t mant = x >> (lead - 23);
  return SHY_AS_FLOAT(((uint32_t)be << 23) | ((uint32_t)mant & 0x7FFFFFu));
}

// shy_evap_div in float arithmetic: s times 1 / c held as a float pair,
// accurate to about 2^-46 relative.  Within 2^-37 of a float rounding
// midpoint, and for s outside [2^-100, 2^100], the integer restatement
// decides.  Equal to shy_evap_div: the bound above leaves no other input
// undecided, and shy_check_conversions compares every positive float on the
// device for the default evaporation rate and three others.
SHY_HD float shy_evap_div_ff(float s, const shy_evap* E) {
  if (!(s >= 7.888609052210118e-31f && s <= 1.2676506002282294e30f)) return s == 0.0f ? s : shy_evap_div(s, E);
  const float qh = s * E->ih;
  const float ql = fmaf(s, E->ih, -qh) + s * E->il;
  float r, e;
  shy_two_sum(qh, ql, &r, &e);
  const uint32_t ru = SHY_AS_UINT(r);
  float half = 0.5f * SHY_AS_FLOAT((ru & 0x7F800000u) - (23u << 23));  // half an ulp of r
  if (e < 0.0f && (ru & 0x7FFFFFu) == 0u) half *= 0.5f;  // below a power of two the ulp halves
  if ((e < 0.0f ? -e : e) > half * (1.0f - 1.220703125e-4f)) return shy_evap_div(s, E);
  return r;
}

// (float)((double)v * (1 - (double)evap)) of the reference's volume
// evaporation (source/water.h:136), in float arithmetic: v times c held as a
// float pair, like shy_evap_div_ff, with the double expression near rounding
// midpoints and for v outside [2^-100, 2^100].  Equal to the double
// expression (shy_check_conversions compares every positive float at four
// evaporation rates).
SHY_HD float shy_evap_mul_ff(float v, const shy_evap* E) {
  if (!(v >= 7.888609052210118e-31f && v <= 1.2676506002282294e30f)) return (float)((double)v * E->c);
  const float ph = v * E->ch;
  const float pl = fmaf(v, E->ch, -ph) + v * E->cl;
  float r, e;
  shy_two_sum(ph, pl, &r, &e);
  const uint32_t ru = SHY_AS_UINT(r);
  float half = 0.5f * SHY_AS_FLOAT((ru & 0x7F800000u) - (23u << 23));  // half an ulp of r
  if (e < 0.0f && (ru & 0x7FFFFFu) == 0u) half *= 0.5f;  // below a power of two the ulp halves
  if ((e < 0.0f ? -e : e) > half * (1.0f - 1.220703125e-4f)) return (float)((double)v * E->c);
  return r;
}

// (float)((double)h - 0.002), the height past the map's edge
// (source/water.h:120-124), in float arithmetic: h minus 0.002 held as a
// float pair (0x1.0624dep-9 + -0x1.a1cacp-34, within 2^-59 of the double
// 0.002), by TwoSum, to about 2^-56 absolute.  Within 2^-37 of a float
// rounding midpoint, for results below 2^-12 in magnitude and for |h| above
// 2^100, the double expression decides.  Equal to the double expression for
// every float (shy_check_conversions compares all 2^32 on the device).
SHY_HD float shy_minus_0002(float h) {
  if (!(h >= -1.2676506002282294e30f && h <= 1.2676506002282294e30f)) return (float)((double)h - 0.002);
  float s, e;
  shy_two_sum(h, -0x1.0624dep-9f, &s, &e);
  e = e - -0x1.a1cacp-34f;
  float r, f;
  shy_two_sum(s, e, &r, &f);
  const float ar = r < 0.0f ? -r : r;
  if (!(ar >= 0x1p-12f)) return (float)((double)h - 0.002);
  const uint32_t ru = SHY_AS_UINT(ar);
  float half = 0.5f * SHY_AS_FLOAT((ru & 0x7F800000u) - (23u << 23));  // half an ulp of r
  if ((ru & 0x7FFFFFu) == 0u && ((f < 0.0f) == (r > 0.0f))) half *= 0.5f;  // toward zero past a power of two
  if ((f < 0.0f ? -f : f) > half * (1.0f - 1.220703125e-4f)) return (float)((double)h - 0.002);
  return r;
}

// The C library's rand() as the reference's process draws it (spawn
// positions, source/world.h:69; plant events, source/vegetation.h:67-182):
// the GNU C library's default generator, an additive lagged-Fibonacci
// generator of degree 31 with lags 3 and 31 (its "TYPE_3" random_r).
// srand(seed): r[0] = seed (1 if 0), r[i] = 16807 r[i-1] mod (2^31 - 1) by
// Schrage's method for i = 1..30, then 310 outputs are discarded.  Each
// output adds the word 31 places back into the word 3 places back (32-bit
// wrap-around), stores the sum and returns it shifted right by one bit.
typedef struct shy_crand {
  int32_t r[31];
  int32_t f, b;  // front (r[f] += r[b]) and back indices
} shy_crand;

SHY_HD int shy_crand_next(shy_crand* g) {
  const uint32_t v = (uint32_t)g->r[g->f] + (uint32_t)g->r[g->b];
  g->r[g->f] = (int32_t)v;
  g->f = g->f == 30 ? 0 : g->f + 1;
  g->b = g->b == 30 ? 0 : g->b + 1;
  return (int)(v >> 1);
}

SHY_HD void shy_crand_seed(shy_crand* g, uint32_t seed) {
  if (seed == 0) seed = 1;
  int32_t word = (int32_t)seed;  // the seed as a signed 32-bit word
  g->r[0] = word;
  for (int i = 1; i < 31; ++i) {
    const int64_t hi = word / 127773, lo = word % 127773;
    word = (int32_t)(16807 * lo - 2836 * hi);
    if (word < 0) word += 2147483647;
    g->r[i] = word;
  }
  g->f = 3;
  g->b = 0;
  for (int i = 0; i < 310; ++i) (void)shy_crand_next(g);
}
