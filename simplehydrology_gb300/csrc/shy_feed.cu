// shy_feed.cu -- the front end's per-frame data as device buffers.
//
// After every erosion frame the reference's front end rebuilds, from the
// maps:
//   the discharge texture  vec4(waterColor, map.discharge(p)), waterColor =
//       (92, 133, 142) / 255 (SimpleHydrology.cpp:341-346, source/model.h:22,
//       map.discharge = erf(0.4 d), source/cellpool.h:242-244)
//   the momentum texture   vec4(0.5 (1 + erf(mx)), 0.5 (1 + erf(my)), 0.5, 1)
//       (SimpleHydrology.cpp:348-354)
//   the terrain mesh       per cell P = (x, mapscale h(x, y), y), the normal
//       quad::_normal, T - P and B - P with T, B the points at x + 1 and y + 1
//       (updatenode, source/cellpool.h:286-317; heights are 0 outside the map)
// and uploads them to OpenGL.  Here they are written into plain buffers (no
// graphics interop): on the device for a caller that keeps them there, or
// copied to the host.  erf is the library's correctly rounded erf, the one
// the rest of the engine uses.
#include "shy_device.cuh"

namespace shy {

namespace {

__global__ void feed_kernel(int kind, const float* __restrict__ h, const float4* __restrict__ rec, int nx,
                            int ny, float* __restrict__ out, float map_scale) {
  const long long n = (long long)nx * ny;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    if (kind == SHY_FEED_DISCHARGE_RGBA) {
      const float4 r = rec[i];
      float4 o;
      o.x = 92.0f / 255.0f;
      o.y = 133.0f / 255.0f;
      o.z = 142.0f / 255.0f;
      o.w = shy_erff_ff(0.4f * r.z);
      reinterpret_cast<float4*>(out)[i] = o;
    } else if (kind == SHY_FEED_MOMENTUM_RGBA) {
      const float4 r = rec[i];
      float4 o;
      o.x = 0.5f * (1.0f + shy_erff_ff(r.x));
      o.y = 0.5f * (1.0f + shy_erff_ff(r.y));
      o.z = 0.5f;
      o.w = 1.0f;
      reinterpret_cast<float4*>(out)[i] = o;
    } else {
      const int x = (int)(i / ny), y = (int)(i - (long long)x * ny);
      const PlainHeights H{h, nx, ny};
      const float px = (float)x, py = (float)y;
      const float hp = map_scale * H(x, y);
      const float3 nrm = normal_from(H, x, y, nx, ny, map_scale);
      float* o = out + 12 * i;
      o[0] = px;
      o[1] = hp;
      o[2] = py;
      o[3] = nrm.x;
      o[4] = nrm.y;
      o[5] = nrm.z;
      o[6] = (float)(x + 1) - px;  // T - P
      o[7] = map_scale * H(x + 1, y) - hp;
      o[8] = py - py;
      o[9] = px - px;  // B - P
      o[10] = map_scale * H(x, y + 1) - hp;
      o[11] = (float)(y + 1) - py;
    }
  }
}

}  // namespace

}  // namespace shy

using namespace shy;

extern "C" int shy_feed(shy_world* w, int terrain, int kind, float* out, size_t count, int out_is_device) {
  if (!w || !out) {
    set_error("shy_feed: null world or output");
    return SHY_ERR_INVALID_ARG;
  }
  if (terrain < 0 || terrain >= (int)w->terrains.size()) {
    set_error("shy_feed: terrain %d out of range", terrain);
    return SHY_ERR_INVALID_ARG;
  }
  if (kind != SHY_FEED_DISCHARGE_RGBA && kind != SHY_FEED_MOMENTUM_RGBA && kind != SHY_FEED_VERTICES) {
    set_error("shy_feed: unknown kind %d", kind);
    return SHY_ERR_INVALID_ARG;
  }
  const Terrain& T = w->terrains[terrain];
  const long long cells = (long long)T.nx * T.ny;
  const size_t per = kind == SHY_FEED_VERTICES ? 12 : 4;
  if (count != (size_t)cells * per) {
    set_error("shy_feed: count %zu, expected %lld (%zu floats per cell)", count, (long long)cells * (long long)per,
              per);
    return SHY_ERR_INVALID_ARG;
  }
  float* dst = out;
  if (!out_is_device) {
    if (w->feed_len < count) {
      if (w->feed) cudaFree(w->feed);
      w->feed = nullptr;
      w->feed_len = 0;
      SHY_CHECK_CUDA(cudaMalloc((void**)&w->feed, sizeof(float) * count), "shy_feed: allocate buffer");
      w->feed_len = count;
    }
    dst = w->feed;
  } else if (((uintptr_t)out & 15) != 0) {
    set_error("shy_feed: device output must be 16-byte aligned");
    return SHY_ERR_INVALID_ARG;
  }
  long long blocks = (cells + 255) / 256;
  if (blocks > 65536) blocks = 65536;
  if (blocks < 1) blocks = 1;
  feed_kernel<<<(int)blocks, 256, 0, w->stream>>>(kind, w->h + T.cell_base, w->rec + T.cell_base, T.nx, T.ny, dst,
                                                  w->P.map_scale);
  SHY_CHECK_CUDA(cudaGetLastError(), "shy_feed: launch");
  if (!out_is_device) {
    SHY_CHECK_CUDA(cudaMemcpyAsync(out, dst, sizeof(float) * count, cudaMemcpyDeviceToHost, w->stream),
                   "shy_feed: copy out");
    SHY_CHECK_CUDA(cudaStreamSynchronize(w->stream), "shy_feed: synchronize");
  }
  return SHY_OK;
}
