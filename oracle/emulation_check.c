/* emulation_check.c -- TEST INFRASTRUCTURE.
 *
 * Verifies the integer-only conversions of shy_math.h, which the batched GPU
 * kernels use in place of FP64 and 64-bit conversion instructions, against
 * the floating-point expressions they stand for:
 *   shy_q32(v)        == llrintf(v * 2^32)                 every float, |v| < 2^31
 *   shy_unq(q)        == (float)((double)q * 2^-32)        structured + random q
 *   shy_evap_div(s)   == (float)((double)s / (1 - evap))  every normal s >= 0
 * Usage: emulation_check [evap [stride]]   (exit status 0 when all agree)
 * stride 1 (the default) checks every float; larger strides check a subset.
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../simplehydrology_gb300/csrc/shy_math.h"

static float f_of(uint32_t u) { float f; memcpy(&f, &u, 4); return f; }
static uint32_t u_of(float f) { uint32_t u; memcpy(&u, &f, 4); return u; }

int main(int argc, char** argv) {
  const float evap = argc > 1 ? (float)atof(argv[1]) : 0.001f;
  const uint64_t stride = argc > 2 ? (uint64_t)atoll(argv[2]) : 1;
  long bad = 0;
  /* q32 over every float with |v| < 2^31 */
  for (uint64_t b = 0; b < 0x100000000ull; b += stride) {
    const float v = f_of((uint32_t)b);
    if (!(fabsf(v) < 2147483648.0f)) continue;
    if (shy_q32(v) != (int64_t)llrintf(v * 4294967296.0f)) {
      if (bad++ < 5) printf("q32 mismatch v=%a\n", v);
    }
  }
  printf("q32 checked, mismatches so far %ld\n", bad);
  /* unq: all q with |q| < 2^26, powers of two and halfway neighbourhoods, random */
  for (int64_t q = -(1 << 26); q <= (1 << 26); ++q)
    if (u_of(shy_unq(q)) != u_of((float)((double)q * (1.0 / 4294967296.0)))) {
      if (bad++ < 10) printf("unq mismatch q=%lld\n", (long long)q);
    }
  uint64_t x = 88172645463325252ull;
  for (long i = 0; i < 200000000 / (long)stride; ++i) {
    x ^= x << 13; x ^= x >> 7; x ^= x << 17;
    int64_t q = (int64_t)(x >> (11 + (i % 40)));
    if (i & 1) q = -q;
    if (u_of(shy_unq(q)) != u_of((float)((double)q * (1.0 / 4294967296.0)))) {
      if (bad++ < 10) printf("unq mismatch q=%lld\n", (long long)q);
    }
  }
  for (int p = 0; p < 53; ++p)
    for (int64_t d = -3; d <= 3; ++d) {
      const int64_t base = (int64_t)1 << p;
      for (int64_t hb = -1; hb <= 1; ++hb) {
        const int64_t q = base + d + (p > 25 ? hb * ((int64_t)1 << (p - 25)) : 0);
        if (q <= 0) continue;
        if (u_of(shy_unq(q)) != u_of((float)((double)q * (1.0 / 4294967296.0)))) {
          if (bad++ < 10) printf("unq mismatch q=%lld\n", (long long)q);
        }
      }
    }
  printf("unq checked, mismatches so far %ld\n", bad);
  /* evap_div over every finite s >= 0 (the fast path covers the normal ones) */
  const shy_evap E = shy_evap_make(evap);
  const double c = 1.0 - (double)evap;
  printf("evap %.9g fast path %d (k=%d)\n", evap, E.fast, E.k);
  for (uint64_t b = 0; b < 0x7F800000u; b += stride) {
    const float s = f_of((uint32_t)b);
    const float want = (float)((double)s / c);
    if (u_of(shy_evap_div(s, &E)) != u_of(want)) {
      if (bad++ < 10) printf("evap_div mismatch s=%a got %a want %a\n", s, shy_evap_div(s, &E), want);
    }
  }
  printf("evap_div checked; total mismatches %ld\n", bad);
  return bad ? 1 : 0;
}
