// shy_device.cuh -- device-side building blocks of the erosion model.
//
// Every floating-point expression here reproduces the reference's evaluation
// order (the library is compiled with --fmad=false, so nothing is fused into
// an FMA, and with IEEE-rounded division and square root), which is what lets
// the exact mode match the reference bit for bit.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "shy_internal.h"
#include "shy_math.h"

namespace shy {

// ---- glm semantics on float2/float3 (component-wise, dot summed left to right)
__device__ __forceinline__ float dot2(float ax, float ay, float bx, float by) { return ax * bx + ay * by; }
__device__ __forceinline__ float len2(float x, float y) { return sqrtf(dot2(x, y, x, y)); }

__device__ __forceinline__ float3 cross_scaled(float3 a, float3 b, float ms) {
  // cross(s * a, s * b) with s = vec3(1, mapscale, 1)  (source/cellpool.h:185-198)
  const float3 sa = make_float3(1.0f * a.x, ms * a.y, 1.0f * a.z);
  const float3 sb = make_float3(1.0f * b.x, ms * b.y, 1.0f * b.z);
  return make_float3(sa.y * sb.z - sb.y * sa.z, sa.z * sb.x - sb.z * sa.x, sa.x * sb.y - sb.x * sa.y);
}

// Fixed-point conversions on the hardware converters, with the bits of the
// integer restatements shy_unq / shy_q32 (shy_math.h).  The converters have
// a low throughput but a short latency, and the lock-step phases are latency
// chains, so the batched kernel uses these; shy_check_conversions compares
// them with the restatements over every float and 2^30 int64 values.
//  * shy_unq_dev: the int64 -> float conversion rounds q once and the scaling
//    by 2^-32 is exact, so for |q| <= 2^53 this is (float)((double)q * 2^-32);
//    larger |q| (heights of 2^21 and more) take the integer restatement.
//  * shy_q32_dev: the scaling by 2^32 is exact and the float -> int64
//    conversion rounds half to even: llrintf(v * 2^32) for |v| < 2^31.
__device__ __forceinline__ float shy_unq_dev(long long q) {
  if (__builtin_expect((unsigned long long)q + (1ull << 53) > (1ull << 54), 0)) return shy_unq(q);
  return __ll2float_rn(q) * 2.3283064365386963e-10f;
}
__device__ __forceinline__ long long shy_q32_dev(float v) { return __float2ll_rn(v * 4294967296.0f); }

__device__ __forceinline__ bool oob(int x, int y, int nx, int ny) {
  return x < 0 || y < 0 || x >= nx || y >= ny;
}

// quad::_normal (source/cellpool.h:182-204) on a height map `h` (terrain
// base already applied), map.height() returning 0 outside the map.
template <class HeightAt>
__device__ __forceinline__ float3 normal_from(HeightAt hat, int px, int py, int nx, int ny, float ms) {
  float3 n = make_float3(0.0f, 0.0f, 0.0f);
  const float hp = hat(px, py);
  auto add = [&](float3 a, float3 b) {
    const float3 c = cross_scaled(a, b, ms);
    n = make_float3(n.x + c.x, n.y + c.y, n.z + c.z);
  };
  if (!oob(px + 1, py + 1, nx, ny))
    add(make_float3(0.0f, hat(px, py + 1) - hp, 1.0f), make_float3(1.0f, hat(px + 1, py) - hp, 0.0f));
  if (!oob(px - 1, py - 1, nx, ny))
    add(make_float3(0.0f, hat(px, py - 1) - hp, -1.0f), make_float3(-1.0f, hat(px - 1, py) - hp, 0.0f));
  if (!oob(px + 1, py - 1, nx, ny))
    add(make_float3(1.0f, hat(px + 1, py) - hp, 0.0f), make_float3(0.0f, hat(px, py - 1) - hp, -1.0f));
  if (!oob(px - 1, py + 1, nx, ny))
    add(make_float3(-1.0f, hat(px - 1, py) - hp, 0.0f), make_float3(0.0f, hat(px, py + 1) - hp, 1.0f));
  const float dd = n.x * n.x + n.y * n.y + n.z * n.z;
  if (sqrtf(dd) > 0.0f) {
    const float r = 1.0f / sqrtf(n.x * n.x + n.y * n.y + n.z * n.z);
    n = make_float3(n.x * r, n.y * r, n.z * r);
  }
  return n;
}

struct PlainHeights {
  const float* h;  // terrain-local
  int nx, ny;
  __device__ __forceinline__ float operator()(int x, int y) const {
    return oob(x, y, nx, ny) ? 0.0f : h[(long long)x * ny + y];
  }
};

// The neighbour order of World::cascade (source/world.h:94-103).
__device__ __forceinline__ int nb_dx(int k) { return k < 3 ? -1 : (k < 5 ? 0 : 1); }
__device__ __forceinline__ int nb_dy(int k) {
  // -1, 0, 1, -1, 1, -1, 0, 1
  return (k == 0 || k == 3 || k == 5) ? -1 : ((k == 1 || k == 6) ? 0 : 1);
}


// ---- exact (sequential, live) model ------------------------------------------

struct DropS {
  int age;
  float px, py, sx, sy, vol, sed;
};

// World::cascade (source/world.h:90-168) on live heights, in place.
__device__ __forceinline__ void cascade_live(float* h, int nx, int ny, float px, float py,
                                             const shy_params& P) {
  int sxs[8], sys_[8];
  float sh[8], sd[8];
  int num = 0;
  const int ix = (int)px, iy = (int)py;
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    const int x = ix + nb_dx(k), y = iy + nb_dy(k);
    if (oob(x, y, nx, ny)) continue;
    const float fx = (float)nb_dx(k), fy = (float)nb_dy(k);
    sxs[num] = x;
    sys_[num] = y;
    sh[num] = h[(long long)x * ny + y];
    sd[num] = len2(fx, fy);
    ++num;
  }
  // stable insertion sort by height (std::sort on <= 16 elements)
  for (int i = 1; i < num; ++i) {
    const int vx = sxs[i], vy = sys_[i];
    const float vh = sh[i], vd = sd[i];
    int j = i;
    while (j > 0 && vh < sh[j - 1]) {
      sxs[j] = sxs[j - 1];
      sys_[j] = sys_[j - 1];
      sh[j] = sh[j - 1];
      sd[j] = sd[j - 1];
      --j;
    }
    sxs[j] = vx;
    sys_[j] = vy;
    sh[j] = vh;
    sd[j] = vd;
  }
  // The centre is never one of its neighbours, so its live height stays in a
  // register through the loop (written back once) instead of a global-memory
  // read after every transfer.
  float* hc = h + (long long)ix * ny + iy;
  float hcv = *hc;
  bool moved = false;
  for (int i = 0; i < num; ++i) {
    const float diff = hcv - sh[i];
    if (diff == 0.0f) continue;
    float excess;
    if (sh[i] >= 0.1f)  // (double)h > 0.1: no float lies between 0.1 and 0.1f
      excess = fabsf(diff) - sd[i] * P.max_diff;
    else
      excess = fabsf(diff);
    if (excess <= 0.0f) continue;
    const float transfer = P.settling * excess / 2.0f;
    float* hn = h + (long long)sxs[i] * ny + sys_[i];
    if (diff > 0.0f) {
      hcv -= transfer;
      *hn += transfer;
    } else {
      hcv += transfer;
      *hn -= transfer;
    }
    moved = true;
  }
  if (moved) *hc = hcv;
}

// Drop::descend (source/water.h:58-156) on live maps.  `rec` holds the
// per-cell {momentumx, momentumy, discharge, 1 + entrainment*erf(0.4 d)}.
__device__ __forceinline__ bool descend_live(float* h, const float4* rec, const float* effd,
                                             float* td, float* tmx, float* tmy, int nx, int ny,
                                             DropS& d, const shy_params& P, double& gain,
                                             double& loss, unsigned long long& steps,
                                             unsigned long long& oobs, const shy_evap& E) {
  const int ix = (int)d.px, iy = (int)d.py;
  if (oob(ix, iy, nx, ny)) return false;
  const long long c = (long long)ix * ny + iy;
  const float3 n = normal_from(PlainHeights{h, nx, ny}, ix, iy, nx, ny, P.map_scale);
  if ((float)d.age > P.max_age) {
    h[c] += d.sed;
    return false;
  }
  if (d.vol < P.min_vol) {
    h[c] += d.sed;
    return false;
  }
  ++steps;
  const float4 r = rec[c];
  const float ed = effd[c];
  d.sx = d.sx + (P.gravity * n.x) / d.vol;
  d.sy = d.sy + (P.gravity * n.z) / d.vol;
  if (len2(r.x, r.y) > 0.0f && len2(d.sx, d.sy) > 0.0f) {
    const float rf = 1.0f / sqrtf(dot2(r.x, r.y, r.x, r.y));
    const float rs = 1.0f / sqrtf(dot2(d.sx, d.sy, d.sx, d.sy));
    const float k = (P.momentum_transfer * dot2(r.x * rf, r.y * rf, d.sx * rs, d.sy * rs)) / (d.vol + r.z);
    d.sx = d.sx + k * r.x;
    d.sy = d.sy + k * r.y;
  }
  if (len2(d.sx, d.sy) > 0.0f) {
    const float root2 = sqrtf(2.0f);
    const float rs = 1.0f / sqrtf(dot2(d.sx, d.sy, d.sx, d.sy));
    const float ux = d.sx * rs, uy = d.sy * rs;
    d.sx = root2 * ux;
    d.sy = root2 * uy;
  }
  d.px = d.px + d.sx;
  d.py = d.py + d.sy;
  td[c] += d.vol;
  tmx[c] += d.vol * d.sx;
  tmy[c] += d.vol * d.sy;
  const int jx = (int)d.px, jy = (int)d.py;
  const bool out = oob(jx, jy, nx, ny);
  float h2;
  if (out)
    h2 = shy_minus_0002(h[c]);  // (float)((double)h - 0.002)
  else
    h2 = h[(long long)jx * ny + jy];
  float ceq = r.w * (h[c] - h2);
  if (ceq < 0.0f) ceq = 0.0f;
  const float cdiff = ceq - d.sed;
  d.sed += ed * cdiff;
  h[c] -= ed * cdiff;
  const float s0 = d.sed;
  // water.h:135-136, the reference's double roundings in float arithmetic
  d.sed = shy_evap_div_ff(d.sed, &E);
  d.vol = shy_evap_mul_ff(d.vol, &E);
  gain += (double)d.sed - (double)s0;
  if (out) {
    d.vol = 0.0f;
    ++oobs;
    loss += (double)d.sed;
    return false;
  }
  cascade_live(h, nx, ny, d.px, d.py, P);
  d.age++;
  return true;
}

}  // namespace shy
