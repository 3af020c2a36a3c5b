// shy_exact.cu -- the exact (sequential, live) erosion mode and the per-cell
// helper kernels (field gather/scatter, record rebuild, normals).
//
// The exact mode runs the reference's World::erode / Drop::descend /
// World::cascade (source/world.h:54-168, source/water.h:58-156) on one GPU
// thread, in the reference's order, on the live device maps.  It exists for
// parity: with the same erf values it reproduces the reference bit for bit.
#include "shy_device.cuh"

namespace shy {

namespace {

const int kBlock = 256;

int blocks_for(long long n, int block = kBlock) {
  long long b = (n + block - 1) / block;
  return (int)(b > 1048576 ? 1048576 : (b < 1 ? 1 : b));
}

// 1 + entrainment * erf(0.4 d) (source/water.h:127, source/cellpool.h:242-244)
// and max(0, depositionRate * (1 - rootdensity)) (source/water.h:86-87).
__global__ void rebuild_records_kernel(float4* __restrict__ rec, float* __restrict__ effd,
                                       CellQ* __restrict__ cq, const float* __restrict__ root,
                                       long long cells, shy_params P) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < cells;
       i += (long long)gridDim.x * blockDim.x) {
    float4 r = rec[i];
    r.w = 1.0f + P.entrainment * shy_erff_ff(0.4f * r.z);
    rec[i] = r;
    const float e = P.deposition_rate * (1.0f - root[i]);
    effd[i] = e < 0.0f ? 0.0f : e;
    cq[i].effd = e < 0.0f ? 0.0f : e;  // the batched mode's copy
  }
}

// World::erode's closing blend (source/world.h:81-86) from float tracks.
__global__ void exact_blend_kernel(float4* __restrict__ rec, const float* __restrict__ td,
                                   const float* __restrict__ tmx, const float* __restrict__ tmy,
                                   long long n, shy_params P) {
  const float a = 1.0f - P.lrate, b = P.lrate;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    float4 r = rec[i];
    r.z = a * r.z + b * td[i];
    r.x = a * r.x + b * tmx[i];
    r.y = a * r.y + b * tmy[i];
    r.w = 1.0f + P.entrainment * shy_erff_ff(0.4f * r.z);
    rec[i] = r;
  }
}

__global__ void exact_erode_kernel(Terrain T, float* h, const float4* rec, const float* effd,
                                   float* td, float* tmx, float* tmy, const int2* spawns, int n,
                                   shy_params P, DevStats* st) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  const shy_evap E = shy_evap_make(P.evap_rate);  // water.h:135-136 constants
  double gain = 0.0, loss = 0.0;
  unsigned long long steps = 0, oobs = 0, drops = 0, skipped = 0;
  for (int i = 0; i < n; ++i) {
    const int2 s = spawns[i];
    // (double)h < 0.1: no float lies between 0.1 and 0.1f
    if (oob(s.x, s.y, T.nx, T.ny) || h[(long long)s.x * T.ny + s.y] < 0.1f) {
      ++skipped;  // source/world.h:71
      continue;
    }
    ++drops;
    DropS d = {0, (float)s.x, (float)s.y, 0.0f, 0.0f, 1.0f, 0.0f};
    while (descend_live(h, rec, effd, td, tmx, tmy, T.nx, T.ny, d, P, gain, loss, steps, oobs, E)) {
    }
  }
  st->drops += drops;
  st->skipped += skipped;
  st->steps += steps;
  st->oob += oobs;
  st->gain_exact += gain;
  st->loss_exact += loss;
}

__global__ void drop_descend_kernel(Terrain T, float* h, const float4* rec, const float* effd,
                                    float* td, float* tmx, float* tmy, shy_drop* drop, int* more,
                                    shy_params P, DevStats* st) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  const shy_evap E = shy_evap_make(P.evap_rate);  // water.h:135-136 constants
  DropS d = {drop->age, drop->pos[0], drop->pos[1], drop->speed[0], drop->speed[1], drop->volume,
             drop->sediment};
  double gain = 0.0, loss = 0.0;
  unsigned long long steps = 0, oobs = 0;
  const bool m = descend_live(h, rec, effd, td, tmx, tmy, T.nx, T.ny, d, P, gain, loss, steps, oobs, E);
  drop->age = d.age;
  drop->pos[0] = d.px;
  drop->pos[1] = d.py;
  drop->speed[0] = d.sx;
  drop->speed[1] = d.sy;
  drop->volume = d.vol;
  drop->sediment = d.sed;
  *more = m ? 1 : 0;
  st->steps += steps;
  st->oob += oobs;
  st->gain_exact += gain;
  st->loss_exact += loss;
}

__global__ void drop_run_kernel(Terrain T, float* h, const float4* rec, const float* effd,
                                float* td, float* tmx, float* tmy, float x, float y, float* trace,
                                int max_records, int* n_out, shy_params P, DevStats* st) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  const shy_evap E = shy_evap_make(P.evap_rate);  // water.h:135-136 constants
  DropS d = {0, x, y, 0.0f, 0.0f, 1.0f, 0.0f};
  double gain = 0.0, loss = 0.0;
  unsigned long long steps = 0, oobs = 0;
  int n = 0;
  for (;;) {
    const bool m = descend_live(h, rec, effd, td, tmx, tmy, T.nx, T.ny, d, P, gain, loss, steps, oobs, E);
    if (n < max_records) {
      float* r = trace + 8 * (long long)n;
      r[0] = m ? 1.0f : 0.0f;
      r[1] = (float)d.age;
      r[2] = d.px;
      r[3] = d.py;
      r[4] = d.sx;
      r[5] = d.sy;
      r[6] = d.vol;
      r[7] = d.sed;
    }
    ++n;
    if (!m) break;
  }
  *n_out = n;
  st->drops += 1;
  st->steps += steps;
  st->oob += oobs;
  st->gain_exact += gain;
  st->loss_exact += loss;
}

__global__ void cascade_kernel(Terrain T, float* h, float x, float y, shy_params P) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  const int ix = (int)x, iy = (int)y;
  if (oob(ix, iy, T.nx, T.ny)) return;
  cascade_live(h, T.nx, T.ny, x, y, P);
}

__global__ void normals_kernel(Terrain T, const float* h, float* out3, float ms) {
  const long long n = (long long)T.nx * T.ny;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const int x = (int)(i / T.ny), y = (int)(i - (long long)x * T.ny);
    const float3 v = normal_from(PlainHeights{h, T.nx, T.ny}, x, y, T.nx, T.ny, ms);
    out3[3 * i + 0] = v.x;
    out3[3 * i + 1] = v.y;
    out3[3 * i + 2] = v.z;
  }
}

__global__ void gather_rec_kernel(const float4* rec, float* out, long long n, int comp) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const float4 r = rec[i];
    out[i] = comp == 0 ? r.x : (comp == 1 ? r.y : (comp == 2 ? r.z : r.w));
  }
}

__global__ void scatter_rec_kernel(float4* rec, const float* in, long long n, int comp) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    float4 r = rec[i];
    if (comp == 0) r.x = in[i];
    else if (comp == 1) r.y = in[i];
    else if (comp == 2) r.z = in[i];
    else r.w = in[i];
    rec[i] = r;
  }
}

}  // namespace

cudaError_t launch_rebuild_records(shy_world* w, int) {
  rebuild_records_kernel<<<blocks_for(w->cells), kBlock, 0, w->stream>>>(w->rec, w->effd, w->cq, w->root,
                                                                         w->cells, w->P);
  return cudaGetLastError();
}

cudaError_t launch_exact_erode(shy_world* w, int t, int n) {
  const Terrain& T = w->terrains[t];
  const long long b = T.cell_base, N = w->cells;
  exact_erode_kernel<<<1, 32, 0, w->stream>>>(T, w->h + b, w->rec + b, w->effd + b, w->track_f + b,
                                              w->track_f + N + b, w->track_f + 2 * N + b, w->dspawn,
                                              n, w->P, w->stats);
  return cudaGetLastError();
}

cudaError_t launch_exact_blend(shy_world* w, int t) {
  const Terrain& T = w->terrains[t];
  const long long b = T.cell_base, N = w->cells, n = (long long)T.nx * T.ny;
  exact_blend_kernel<<<blocks_for(n), kBlock, 0, w->stream>>>(
      w->rec + b, w->track_f + b, w->track_f + N + b, w->track_f + 2 * N + b, n, w->P);
  return cudaGetLastError();
}

cudaError_t launch_drop_descend(shy_world* w, int t) {
  const Terrain& T = w->terrains[t];
  const long long b = T.cell_base, N = w->cells;
  drop_descend_kernel<<<1, 32, 0, w->stream>>>(T, w->h + b, w->rec + b, w->effd + b, w->track_f + b,
                                               w->track_f + N + b, w->track_f + 2 * N + b, w->ddrop,
                                               w->dint, w->P, w->stats);
  return cudaGetLastError();
}

cudaError_t launch_drop_run(shy_world* w, int t, float x, float y, int max_records) {
  const Terrain& T = w->terrains[t];
  const long long b = T.cell_base, N = w->cells;
  drop_run_kernel<<<1, 32, 0, w->stream>>>(T, w->h + b, w->rec + b, w->effd + b, w->track_f + b,
                                           w->track_f + N + b, w->track_f + 2 * N + b, x, y,
                                           w->dtrace, max_records, w->dint, w->P, w->stats);
  return cudaGetLastError();
}

cudaError_t launch_cascade(shy_world* w, int t, float x, float y) {
  const Terrain& T = w->terrains[t];
  cascade_kernel<<<1, 32, 0, w->stream>>>(T, w->h + T.cell_base, x, y, w->P);
  return cudaGetLastError();
}

cudaError_t launch_normals(shy_world* w, int t, float* out3) {
  const Terrain& T = w->terrains[t];
  normals_kernel<<<blocks_for((long long)T.nx * T.ny), kBlock, 0, w->stream>>>(
      T, w->h + T.cell_base, out3, w->P.map_scale);
  return cudaGetLastError();
}

// one component (0 x, 1 y, 2 z, 3 w) of rec <-> a contiguous float array
cudaError_t launch_gather_comp(shy_world* w, int t, int comp, float* out) {
  const Terrain& T = w->terrains[t];
  const long long n = (long long)T.nx * T.ny;
  gather_rec_kernel<<<blocks_for(n), kBlock, 0, w->stream>>>(w->rec + T.cell_base, out, n, comp);
  return cudaGetLastError();
}

cudaError_t launch_scatter_comp(shy_world* w, int t, int comp, const float* in) {
  const Terrain& T = w->terrains[t];
  const long long n = (long long)T.nx * T.ny;
  scatter_rec_kernel<<<blocks_for(n), kBlock, 0, w->stream>>>(w->rec + T.cell_base, in, n, comp);
  return cudaGetLastError();
}

namespace {

// discharge and momentum into the per-cell records in one pass (null: keep),
// with 1 + entrainment * erf(0.4 d) when the discharge changes
// (source/water.h:127, source/cellpool.h:242-244)
__global__ void pack_state_kernel(float4* __restrict__ rec, const float* __restrict__ d,
                                  const float* __restrict__ mx, const float* __restrict__ my, long long n,
                                  shy_params P) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    float4 r = rec[i];
    if (mx) r.x = mx[i];
    if (my) r.y = my[i];
    if (d) {
      r.z = d[i];
      r.w = 1.0f + P.entrainment * shy_erff_ff(0.4f * r.z);
    }
    rec[i] = r;
  }
}

__global__ void unpack_state_kernel(const float4* __restrict__ rec, float* __restrict__ d, float* __restrict__ mx,
                                    float* __restrict__ my, long long n) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const float4 r = rec[i];
    if (mx) mx[i] = r.x;
    if (my) my[i] = r.y;
    if (d) d[i] = r.z;
  }
}

}  // namespace

cudaError_t launch_pack_state(shy_world* w, int t, const float* d, const float* mx, const float* my) {
  const Terrain& T = w->terrains[t];
  const long long n = (long long)T.nx * T.ny;
  pack_state_kernel<<<blocks_for(n), kBlock, 0, w->stream>>>(w->rec + T.cell_base, d, mx, my, n, w->P);
  return cudaGetLastError();
}

cudaError_t launch_pack_state_all(shy_world* w, const float* d, const float* mx, const float* my) {
  pack_state_kernel<<<blocks_for(w->cells), kBlock, 0, w->stream>>>(w->rec, d, mx, my, w->cells, w->P);
  return cudaGetLastError();
}

cudaError_t launch_unpack_state_all(shy_world* w, float* d, float* mx, float* my) {
  unpack_state_kernel<<<blocks_for(w->cells), kBlock, 0, w->stream>>>(w->rec, d, mx, my, w->cells);
  return cudaGetLastError();
}

cudaError_t launch_unpack_state(shy_world* w, int t, float* d, float* mx, float* my) {
  const Terrain& T = w->terrains[t];
  const long long n = (long long)T.nx * T.ny;
  unpack_state_kernel<<<blocks_for(n), kBlock, 0, w->stream>>>(w->rec + T.cell_base, d, mx, my, n);
  return cudaGetLastError();
}

}  // namespace shy
