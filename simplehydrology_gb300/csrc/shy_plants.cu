// shy_plants.cu -- the reference's frame loop in its own sequence: random
// stream, World::erode spawns and Vegetation::grow's plant agents.
//
// The reference draws every random number of a frame (World::erode's spawn
// positions, source/world.h:69, and the plant events of Vegetation::grow,
// source/vegetation.h:122-188) from the C library's rand().  A world here
// carries that generator on the device (shy_crand, shy_math.h), so that
//   shy_world_srand(w, s); for each frame: shy_erode_rand(w, n);
//   shy_vegetation_grow(w);
// reproduces `srand(s); World::erode(n); Vegetation::grow();` with the
// reference's plant list.  Like the exact erosion mode these are parity
// paths: one device thread runs the sequence in the reference's order.
#include "shy_device.cuh"

namespace shy {

namespace {

__global__ void crand_seed_kernel(shy_crand* g, unsigned seed) {
  if (blockIdx.x == 0 && threadIdx.x == 0) shy_crand_seed(g, seed);
}

// World::erode's spawn draws, source/world.h:64-69: two rand() per drop,
// the argument evaluated first taking the first draw.
__global__ void crand_spawns_kernel(shy_crand* gen, int n, int nx, int ny, int order, int2* out) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  shy_crand g = *gen;
  for (int i = 0; i < n; ++i) {
    const int r1 = shy_crand_next(&g), r2 = shy_crand_next(&g);
    out[i] = make_int2((order == 0 ? r1 : r2) % nx, (order == 0 ? r2 : r1) % ny);
  }
  *gen = g;
}

struct PlantMaps {
  const float* h;
  const float4* rec;
  float* root;
  float* effd;
  CellQ* cq;
  int nx, ny;
};

// quad::map::discharge, source/cellpool.h:439-443
__device__ float map_discharge(const PlantMaps& M, int x, int y) {
  return oob(x, y, M.nx, M.ny) ? 0.0f : shy_erff_ff(0.4f * M.rec[(long long)x * M.ny + y].z);
}

// Plant::root(f), source/vegetation.h:87-118, and the deposition rate of
// every cell it changes (source/water.h:86-87)
__device__ void plant_root(const PlantMaps& M, float px, float py, float f, const shy_params& P) {
  const int ox[9] = {0, 1, -1, 0, 0, -1, 1, -1, 1};
  const int oy[9] = {0, 0, 0, 1, -1, -1, -1, 1, 1};
  const float wgt[9] = {1.0f, 0.6f, 0.6f, 0.6f, 0.6f, 0.4f, 0.4f, 0.4f, 0.4f};
  for (int k = 0; k < 9; ++k) {
    const int x = (int)(px + (float)ox[k]), y = (int)(py + (float)oy[k]);
    if (oob(x, y, M.nx, M.ny)) continue;
    const long long c = (long long)x * M.ny + y;
    const float r = M.root[c] + f * wgt[k];
    M.root[c] = r;
    const float e = P.deposition_rate * (1.0f - r);
    M.effd[c] = e < 0.0f ? 0.0f : e;
    M.cq[c].effd = e < 0.0f ? 0.0f : e;
  }
}

// Vegetation::grow, source/vegetation.h:122-188, on the plant list
// `plants[0 .. *count)` ((x, y, size) each).  *err = 1 if the list would
// outgrow `cap` (the call then stops at that point).
__global__ void plants_grow_kernel(shy_crand* gen, float3* plants, int* count, int cap, int* err, PlantMaps M,
                                   int order, shy_params P) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  shy_crand g = *gen;
  int n = *count;
  const PlainHeights H{M.h, M.nx, M.ny};
  {  // a random position, :126-139
    const int x = shy_crand_next(&g) % M.nx;
    const int y = shy_crand_next(&g) % M.ny;
    // Plant::spawn, :76-85
    if (!(map_discharge(M, x, y) >= P.plant_max_discharge) &&
        !(normal_from(H, x, y, M.nx, M.ny, P.map_scale).y < P.plant_max_steep) &&
        !(H(x, y) >= P.plant_max_height)) {
      if (n >= cap) {
        *err = 1;
        *gen = g;
        *count = n;
        return;
      }
      plants[n++] = make_float3((float)x, (float)y, 0.0f);
      plant_root(M, (float)x, (float)y, 1.0f, P);
    }
  }
  for (int i = 0; i < n; ++i) {  // :143-183 (plants appended here are visited too)
    float3 p = plants[i];
    p.z = p.z + P.plant_grow_rate * (P.plant_max_size - p.z);  // Plant::grow, :63-65
    plants[i] = p;
    const int cx = (int)p.x, cy = (int)p.y;
    // Plant::die, :67-74, with its short-circuit order
    const bool die = map_discharge(M, cx, cy) >= P.plant_max_discharge || H(cx, cy) >= P.plant_max_height ||
                     shy_crand_next(&g) % 1000 == 0;
    if (die) {
      plant_root(M, p.x, p.y, -1.0f, P);
      for (int k = i; k + 1 < n; ++k) plants[k] = plants[k + 1];
      --n;
      --i;
      continue;
    }
    if (shy_crand_next(&g) % 20 != 0) continue;  // :160
    const int r1 = shy_crand_next(&g), r2 = shy_crand_next(&g);
    const int dx = (order == 0 ? r1 : r2) % 9 - 4, dy = (order == 0 ? r2 : r1) % 9 - 4;  // :162
    const float nxp = p.x + (float)dx, nyp = p.y + (float)dy;
    const int ix = (int)nxp, iy = (int)nyp;
    if (oob(ix, iy, M.nx, M.ny)) continue;                              // :165
    if (map_discharge(M, ix, iy) >= P.plant_max_discharge) continue;    // :168
    if ((double)(float)(shy_crand_next(&g) % 1000) / 1000.0 <= (double)M.root[(long long)ix * M.ny + iy])
      continue;                                                          // :171
    if (normal_from(H, ix, iy, M.nx, M.ny, P.map_scale).y <= P.plant_max_steep) continue;  // :174-177
    if (n >= cap) {
      *err = 1;
      break;
    }
    plants[n++] = make_float3(nxp, nyp, 0.0f);
    plant_root(M, nxp, nyp, 1.0f, P);
  }
  *gen = g;
  *count = n;
}

int ensure_crand(shy_world* w) {
  if (w->crand) return SHY_OK;
  SHY_CHECK_CUDA(cudaMalloc((void**)&w->crand, sizeof(shy_crand)), "allocate random stream");
  crand_seed_kernel<<<1, 1, 0, w->stream>>>(w->crand, 1u);  // rand() before any srand() is srand(1)
  SHY_CHECK_CUDA(cudaGetLastError(), "seed random stream");
  return SHY_OK;
}

}  // namespace

}  // namespace shy

using namespace shy;

extern "C" int shy_world_srand(shy_world* w, uint32_t seed) {
  int rc = world_check(w);
  if (rc) return rc;
  if ((rc = ensure_crand(w)) != SHY_OK) return rc;
  crand_seed_kernel<<<1, 1, 0, w->stream>>>(w->crand, seed);
  SHY_CHECK_CUDA(cudaGetLastError(), "shy_world_srand");
  SHY_CHECK_CUDA(cudaStreamSynchronize(w->stream), "synchronize");
  return SHY_OK;
}

extern "C" int shy_world_set_rand_order(shy_world* w, int order) {
  int rc = world_check(w);
  if (rc) return rc;
  if (order != 0 && order != 1) {
    set_error("shy_world_set_rand_order: order must be 0 or 1");
    return SHY_ERR_INVALID_ARG;
  }
  w->rand_order = order;
  return SHY_OK;
}

extern "C" int shy_erode_rand(shy_world* w, int drops) {
  int rc = world_check(w);
  if (rc) return rc;
  if (drops < 0) {
    set_error("shy_erode_rand: negative drop count");
    return SHY_ERR_INVALID_ARG;
  }
  if ((rc = ensure_crand(w)) != SHY_OK) return rc;
  if ((rc = ensure_spawn_capacity(w, drops)) != SHY_OK) return rc;
  const Terrain& T = w->terrains[0];
  crand_spawns_kernel<<<1, 1, 0, w->stream>>>(w->crand, drops, T.nx, T.ny, w->rand_order, w->dspawn);
  SHY_CHECK_CUDA(cudaGetLastError(), "shy_erode_rand: spawns");
  return exact_erode_device_spawns(w, 0, drops);
}

extern "C" int shy_vegetation_grow(shy_world* w) {
  int rc = world_check(w);
  if (rc) return rc;
  if ((rc = ensure_crand(w)) != SHY_OK) return rc;
  // room for every plant to spread once, twice over, before the call
  const long long want = 4ll * ((long long)w->plant_count + 1) + 4096;
  if (want > (1ll << 30)) {
    set_error("shy_vegetation_grow: plant list too long");
    return SHY_ERR_STATE;
  }
  if (w->plant_cap < want) {
    float3* np = nullptr;
    SHY_CHECK_CUDA(cudaMalloc((void**)&np, sizeof(float3) * (size_t)want), "allocate plant list");
    if (w->plants && w->plant_count > 0) {
      cudaError_t e = cudaMemcpyAsync(np, w->plants, sizeof(float3) * (size_t)w->plant_count,
                                      cudaMemcpyDeviceToDevice, w->stream);
      if (e == cudaSuccess) e = cudaStreamSynchronize(w->stream);
      if (e != cudaSuccess) {
        cudaFree(np);
        return cuda_fail(e, "shy_vegetation_grow: grow plant list");
      }
    }
    if (w->plants) cudaFree(w->plants);
    w->plants = np;
    w->plant_cap = (int)want;
  }
  const Terrain& T = w->terrains[0];
  PlantMaps M{w->h, w->rec, w->root, w->effd, w->cq, T.nx, T.ny};
  int host[2] = {w->plant_count, 0};
  SHY_CHECK_CUDA(cudaMemcpyAsync(w->dint, host, sizeof(host), cudaMemcpyHostToDevice, w->stream), "upload count");
  plants_grow_kernel<<<1, 1, 0, w->stream>>>(w->crand, w->plants, w->dint, w->plant_cap, w->dint + 1, M,
                                             w->rand_order, w->P);
  SHY_CHECK_CUDA(cudaGetLastError(), "shy_vegetation_grow: launch");
  SHY_CHECK_CUDA(cudaMemcpyAsync(host, w->dint, sizeof(host), cudaMemcpyDeviceToHost, w->stream), "read count");
  SHY_CHECK_CUDA(cudaStreamSynchronize(w->stream), "synchronize");
  w->plant_count = host[0];
  if (host[1]) {
    set_error("shy_vegetation_grow: plant list capacity exceeded");
    return SHY_ERR_STATE;
  }
  return SHY_OK;
}

extern "C" int shy_plants(shy_world* w, float* out, int max_plants, int* count) {
  int rc = world_check(w);
  if (rc) return rc;
  if (!count || max_plants < 0 || (max_plants > 0 && !out)) {
    set_error("shy_plants: invalid output");
    return SHY_ERR_INVALID_ARG;
  }
  *count = w->plant_count;
  const int n = w->plant_count < max_plants ? w->plant_count : max_plants;
  if (n > 0) {
    SHY_CHECK_CUDA(cudaMemcpyAsync(out, w->plants, sizeof(float3) * (size_t)n, cudaMemcpyDeviceToHost, w->stream),
                   "shy_plants: copy");
    SHY_CHECK_CUDA(cudaStreamSynchronize(w->stream), "synchronize");
  }
  return SHY_OK;
}
