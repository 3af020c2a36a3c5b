// shy_vegetation.cu -- per-cell vegetation, the engine's form of
// Vegetation::grow (source/vegetation.h:122-188).
//
// Every cell holds at most one plant (size > 0).  One step grows every plant
// once, in parallel, against the maps as they were at the start of the step:
// grow (:63-65), die on discharge, height or a 1/1000 draw (:67-74) with
// root(-1), spread with 1/20 to a cell offset by up to 4 (:160-183), and
// spawn on empty cells with plant_spawn_prob where Plant::spawn allows
// (:76-85).  A new plant may spread in the step it appears, as the
// reference's loop visits appended plants in the same call.  root(f) adds f * {1, 0.6, 0.4} over the 3 x 3 block (:87-118)
// as 32.32 fixed-point sums.  A cell that several new plants reach gets one
// (claimed atomically; the outcome does not depend on who wins), and the
// plant map is double-buffered, so the step is deterministic.  After the
// step the deposition records (source/water.h:86-87) follow the new root
// density.  oracle/hydro_oracle.cpp (vegetation_step) restates it.
#include "shy_device.cuh"

namespace shy {

namespace {

__device__ __forceinline__ float veg_weight(int dx, int dy) {
  const int n = (dx != 0) + (dy != 0);
  return n == 0 ? 1.0f : (n == 1 ? 0.6f : 0.4f);
}

__device__ __forceinline__ void add_i64(long long* p, long long v) {
  atomicAdd((unsigned long long*)p, (unsigned long long)v);
}

__device__ __forceinline__ int terrain_of_cell(const Terrain* T, int n, long long i) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (T[mid].cell_base <= i) lo = mid; else hi = mid - 1;
  }
  return lo;
}

__global__ void veg_step_kernel(const Terrain* __restrict__ terrains, int n_terrains, long long cells,
                                const float* __restrict__ h, const float4* __restrict__ rec,
                                const float* __restrict__ root, const float* __restrict__ plant0,
                                float* __restrict__ plant1, long long* __restrict__ rootq,
                                unsigned* __restrict__ claim, unsigned tag, shy_params P,
                                unsigned long long step) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < cells;
       i += (long long)gridDim.x * blockDim.x) {
    const Terrain T = terrains[terrain_of_cell(terrains, n_terrains, i)];
    const long long lc = i - T.cell_base;
    const int x = (int)(lc / T.ny), y = (int)(lc - (long long)x * T.ny);
    const float* hT = h + T.cell_base;
    auto u = [&](long long cell, unsigned what) { return shy_uniform24(T.seed, step, (unsigned long long)cell, what); };
    auto erfd = [&](long long gi) { return shy_erff_ff(0.4f * rec[gi].z); };
    auto root_add = [&](int cx, int cy, float f) {
      for (int dx = -1; dx <= 1; ++dx)
        for (int dy = -1; dy <= 1; ++dy)
          if (!oob(cx + dx, cy + dy, T.nx, T.ny))
            add_i64(&rootq[T.cell_base + (long long)(cx + dx) * T.ny + (cy + dy)], shy_q32(f * veg_weight(dx, dy)));
    };
    // a new plant, at most one per cell (the first claim wins; every claim
    // places the same plant)
    auto claim_cell = [&](int tx, int ty) {
      const long long t = T.cell_base + (long long)tx * T.ny + ty;
      if (atomicExch(&claim[t], tag) == tag) return false;
      plant1[t] = P.plant_grow_rate * (P.plant_max_size - 0.0f);
      root_add(tx, ty, 1.0f);
      return true;
    };
    // the spread rule (:160-183) from (sx, sy) with the draws of local cell
    // `c` (what = w0 .. w0 + 3), on the step's starting maps
    auto spread_target = [&](int sx, int sy, long long c, unsigned w0, int& tx, int& ty) {
      if (!(u(c, w0) < P.plant_spread_prob)) return false;
      tx = sx + (int)(u(c, w0 + 1) * 9.0f) - 4;
      ty = sy + (int)(u(c, w0 + 2) * 9.0f) - 4;
      if (oob(tx, ty, T.nx, T.ny)) return false;
      const long long t = T.cell_base + (long long)tx * T.ny + ty;
      if (erfd(t) >= P.plant_max_discharge) return false;
      if ((float)(int)(u(c, w0 + 3) * 1000.0f) / 1000.0f <= root[t]) return false;
      if (!(normal_from(PlainHeights{hT, T.nx, T.ny}, tx, ty, T.nx, T.ny, P.map_scale).y > P.plant_max_steep))
        return false;
      return !(plant0[t] > 0.0f);
    };
    // The reference visits a plant appended during Vegetation::grow in the
    // same call (:138 re-reads plants.size()), so a new plant may spread at
    // once: the plant a claim places takes one spread attempt in the same
    // step, with draws keyed by its own cell (chains of three or more new
    // plants in one step are cut at two).
    auto place = [&](int tx, int ty) {
      if (!claim_cell(tx, ty)) return;
      int ux, uy;
      if (spread_target(tx, ty, (long long)tx * T.ny + ty, 6, ux, uy)) claim_cell(ux, uy);
    };
    const float s0 = plant0[i];
    if (s0 > 0.0f) {
      const float s = s0 + P.plant_grow_rate * (P.plant_max_size - s0);
      if (erfd(i) >= P.plant_max_discharge || hT[lc] >= P.plant_max_height || u(lc, 0) < P.plant_death_prob) {
        plant1[i] = 0.0f;
        root_add(x, y, -1.0f);
        continue;
      }
      plant1[i] = s;
      int tx, ty;
      if (spread_target(x, y, lc, 1, tx, ty)) place(tx, ty);
    } else {
      if (!(u(lc, 5) < P.plant_spawn_prob)) continue;
      if (erfd(i) >= P.plant_max_discharge) continue;
      if (normal_from(PlainHeights{hT, T.nx, T.ny}, x, y, T.nx, T.ny, P.map_scale).y < P.plant_max_steep) continue;
      if (hT[lc] >= P.plant_max_height) continue;
      place(x, y);
    }
  }
}

// root density += the step's sums; deposition records follow.
__global__ void veg_apply_kernel(long long cells, float* __restrict__ root, long long* __restrict__ rootq,
                                 float* __restrict__ effd, CellQ* __restrict__ cq, shy_params P) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < cells;
       i += (long long)gridDim.x * blockDim.x) {
    const long long q = rootq[i];
    float r = root[i];
    if (q != 0) {
      r = r + shy_unq(q);
      root[i] = r;
      rootq[i] = 0;
    }
    const float e = P.deposition_rate * (1.0f - r);  // source/water.h:86-87
    effd[i] = e < 0.0f ? 0.0f : e;
    cq[i].effd = e < 0.0f ? 0.0f : e;  // the batched mode's copy
  }
}

int grid_for(long long n) {
  long long b = (n + 255) / 256;
  return (int)(b > 65536 ? 65536 : (b < 1 ? 1 : b));
}

}  // namespace

cudaError_t launch_vegetation_step(shy_world* w) {
  cudaError_t e = cudaMemcpyAsync(w->plant_next, w->plant, sizeof(float) * w->cells, cudaMemcpyDeviceToDevice,
                                  w->stream);
  if (e != cudaSuccess) return e;
  const unsigned tag = (unsigned)(w->veg_step & 0x7FFFFFFFull);
  veg_step_kernel<<<grid_for(w->cells), 256, 0, w->stream>>>(w->dterrains, (int)w->terrains.size(), w->cells,
                                                              w->h, w->rec, w->root, w->plant, w->plant_next,
                                                              w->rootq, w->veg_claim, tag, w->P, w->veg_step);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  veg_apply_kernel<<<grid_for(w->cells), 256, 0, w->stream>>>(w->cells, w->root, w->rootq, w->effd, w->cq,
                                                                  w->P);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  float* t = w->plant;
  w->plant = w->plant_next;
  w->plant_next = t;
  return cudaSuccess;
}

}  // namespace shy
