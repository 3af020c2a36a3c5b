// shy_terrain.cu -- terrain generation on the device.
//
// Two generators:
//  * the workloads' heightmaps: seeded fractal value noise normalised to
//    [0, 1] (shy_value_noise in shy_math.h: bilinear value noise with
//    smoothstep weights, 8 octaves, lacunarity 2, gain 0.5), in IEEE double
//    in a fixed order, so the result matches the host restatement bit for
//    bit;
//  * the reference's own terrain, quad::map::init's eight layers of
//    OpenSimplex2 FBm noise (source/cellpool.h:349-409, restated in
//    shy_fnl.h), in float in the reference's operation order, so the result
//    is the reference's bit for bit.
// Both min-max normalise as the reference does (:382-409).
#include "shy_device.cuh"
#include "shy_fnl.h"

namespace shy {

namespace {

// order-preserving map of a double to an unsigned 64-bit key
__device__ __forceinline__ unsigned long long dkey(double v) {
  const unsigned long long b = (unsigned long long)__double_as_longlong(v);
  return (b & 0x8000000000000000ull) ? ~b : (b | 0x8000000000000000ull);
}
__device__ __forceinline__ double dunkey(unsigned long long k) {
  const unsigned long long b = (k & 0x8000000000000000ull) ? (k & 0x7FFFFFFFFFFFFFFFull) : ~k;
  return __longlong_as_double((long long)b);
}

__global__ void noise_kernel(Terrain T, unsigned long long seed, int octaves, double* raw,
                             unsigned long long* minmax) {
  const long long n = (long long)T.nx * T.ny;
  const int side = T.nx > T.ny ? T.nx : T.ny;
  unsigned long long lo = ~0ull, hi = 0ull;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(i / T.ny), y = (int)(i - (long long)x * T.ny);
    const double v = shy_value_noise(seed, x, y, side, octaves);
    raw[i] = v;
    const unsigned long long k = dkey(v);
    lo = k < lo ? k : lo;
    hi = k > hi ? k : hi;
  }
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned long long a = __shfl_down_sync(0xffffffffu, lo, o);
    const unsigned long long b = __shfl_down_sync(0xffffffffu, hi, o);
    lo = a < lo ? a : lo;
    hi = b > hi ? b : hi;
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMin(&minmax[0], lo);
    atomicMax(&minmax[1], hi);
  }
}

__global__ void normalise_kernel(long long n, const double* raw, const unsigned long long* minmax,
                                 float* h) {
  const double lo = dunkey(minmax[0]), hi = dunkey(minmax[1]);
  const double span = hi - lo;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    h[i] = span > 0.0 ? __double2float_rn((raw[i] - lo) / span) : 0.0f;
}

// order-preserving map of a float to an unsigned 32-bit key
__device__ __forceinline__ unsigned fkey(float v) {
  const unsigned b = __float_as_uint(v);
  return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}
__device__ __forceinline__ float funkey(unsigned k) {
  return __uint_as_float((k & 0x80000000u) ? (k & 0x7FFFFFFFu) : ~k);
}

struct FnlScales {
  float s[8];
};

// Unnormalised heights of the reference's init (source/cellpool.h:354-375)
// into h, and their minimum and maximum, both starting at 0 as the
// reference's do (:377-385).
__global__ void fnl_kernel(Terrain T, float zc, FnlScales sc, float* __restrict__ h, unsigned* minmax) {
  const long long n = (long long)T.nx * T.ny;
  unsigned lo = fkey(0.0f), hi = fkey(0.0f);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(i / T.ny), y = (int)(i - (long long)x * T.ny);
    const float v = shy_fnl_height(x, y, T.nx, T.ny, zc, sc.s);
    h[i] = v;
    const unsigned k = fkey(v);
    lo = k < lo ? k : lo;
    hi = k > hi ? k : hi;
  }
  for (int o = 16; o > 0; o >>= 1) {
    const unsigned a = __shfl_down_sync(0xffffffffu, lo, o);
    const unsigned b = __shfl_down_sync(0xffffffffu, hi, o);
    lo = a < lo ? a : lo;
    hi = b > hi ? b : hi;
  }
  if ((threadIdx.x & 31) == 0) {
    atomicMin(&minmax[0], lo);
    atomicMax(&minmax[1], hi);
  }
}

// (height - min) / (max - min), source/cellpool.h:407
__global__ void fnl_normalise_kernel(long long n, const unsigned* minmax, float* __restrict__ h) {
  const float lo = funkey(minmax[0]), hi = funkey(minmax[1]);
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x)
    h[i] = (h[i] - lo) / (hi - lo);
}

}  // namespace

cudaError_t launch_reference_terrain(shy_world* w, int t, int32_t seed, unsigned* minmax) {
  const Terrain& T = w->terrains[t];
  const long long n = (long long)T.nx * T.ny;
  FnlScales sc;
  shy_fnl_scales(sc.s);
  const unsigned init[2] = {0x80000000u, 0x80000000u};  // the keys of 0.0f
  cudaError_t e = cudaMemcpyAsync(minmax, init, sizeof(init), cudaMemcpyHostToDevice, w->stream);
  if (e != cudaSuccess) return e;
  long long blocks = (n + 255) / 256;
  if (blocks > 4096) blocks = 4096;
  fnl_kernel<<<(int)blocks, 256, 0, w->stream>>>(T, shy_fnl_zcoord(seed), sc, w->h + T.cell_base, minmax);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  fnl_normalise_kernel<<<(int)blocks, 256, 0, w->stream>>>(n, minmax, w->h + T.cell_base);
  return cudaGetLastError();
}

cudaError_t launch_value_noise(shy_world* w, int t, unsigned long long seed, int octaves, double* raw,
                               unsigned long long* minmax) {
  const Terrain& T = w->terrains[t];
  const long long n = (long long)T.nx * T.ny;
  const unsigned long long init[2] = {~0ull, 0ull};
  cudaError_t e = cudaMemcpyAsync(minmax, init, sizeof(init), cudaMemcpyHostToDevice, w->stream);
  if (e != cudaSuccess) return e;
  long long blocks = (n + 255) / 256;
  if (blocks > 4096) blocks = 4096;
  noise_kernel<<<(int)blocks, 256, 0, w->stream>>>(T, seed, octaves, raw, minmax);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  normalise_kernel<<<(int)blocks, 256, 0, w->stream>>>(n, raw, minmax, w->h + T.cell_base);
  return cudaGetLastError();
}

}  // namespace shy
