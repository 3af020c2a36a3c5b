// shy_noalloc.cu -- batched erosion without any device allocation.
//
// shy_erode_noalloc (include/shy.h) runs the same lock-step cycles as
// shy_erode on maps the caller already holds in device memory.  Everything
// else the cycles need -- fixed-point cell records, track sums, per-cell
// records, drop slots, the steep-cascade queue, counters -- lives in one
// file-scope device array below, sized for at most SHY_NOALLOC_MAX_CELLS
// cells and SHY_NOALLOC_MAX_DROPS drops per cycle.  Every GPU that loads the
// library holds that array until the process exits; every call on a device
// shares it and starts by clearing what must start at zero.
#include <mutex>

#include "shy_device.cuh"

namespace shy {

namespace {

struct NoallocScratch {
  CellQ cq[SHY_NOALLOC_MAX_CELLS];
  Tracks trk[SHY_NOALLOC_MAX_CELLS];
  float4 rec[SHY_NOALLOC_MAX_CELLS];
  float effd[SHY_NOALLOC_MAX_CELLS];
  float track_f[3 * SHY_NOALLOC_MAX_CELLS];
  float voltab[SHY_NOALLOC_MAX_AGE + 3];
  SteepCell steep[SHY_NOALLOC_MAX_DROPS];
  // arrivals bitmaps, two step parities of ceil(nx / 8) * ceil(ny / 8)
  // <= cells / 64 + (nx + ny) / 8 + 1 words each
  unsigned long long arr[2 * (SHY_NOALLOC_MAX_CELLS / 64 + (SHY_NOALLOC_MAX_CELLS + 1) / 8 + 2)];
  float2 pos[SHY_NOALLOC_MAX_DROPS], spd[SHY_NOALLOC_MAX_DROPS];
  float sed[SHY_NOALLOC_MAX_DROPS];
  long long own[SHY_NOALLOC_MAX_DROPS];
  int cell[SHY_NOALLOC_MAX_DROPS], ctr[SHY_NOALLOC_MAX_DROPS];
  int age[SHY_NOALLOC_MAX_DROPS], terr[SHY_NOALLOC_MAX_DROPS];
  Terrain terrain;
  GridBar bar;
  DevStats st;
};

// The scratch.  In host code this name is only a stand-in for the symbol,
// not a device address: the host reaches it through cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char shy_noalloc_scratch[sizeof(NoallocScratch)];

const int kMaxDevices = 64;
std::mutex g_mu;
NoallocScratch* g_scratch[kMaxDevices] = {};

// The scratch's device address on the current device, looked up once per
// device (the first call on a device does this).
cudaError_t scratch_for_device(NoallocScratch** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> lock(g_mu);
  if (!g_scratch[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, shy_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_scratch[dev] = static_cast<NoallocScratch*>(p);
  }
  *out = g_scratch[dev];
  return cudaSuccess;
}

// The terrain entry and the counters, cleared for a fresh run; the volume
// table (source/water.h:136) for this evaporation rate.
__global__ void noalloc_init_kernel(NoallocScratch* s, Terrain T, unsigned long long cycle0, float evap, int nvol) {
  if (blockIdx.x != 0 || threadIdx.x != 0) return;
  s->terrain = T;
  GridBar b = {};
  b.cycle = cycle0;
  s->bar = b;
  DevStats z = {};
  s->st = z;
  float v = 1.0f;
  for (int k = 0; k < nvol; ++k) {
    s->voltab[k] = v;
    v = (float)((double)v * (1.0 - (double)evap));
  }
}

// The caller's maps into the batched mode's state: heights to 32.32 fixed
// point (and re-rounded), per-cell records (source/water.h:86-87,127), track
// sums and pending sums cleared.
__global__ void noalloc_pack_kernel(NoallocScratch* s, int n, long long words, float* h, const float* d,
                                    const float* mx, const float* my, const float* root, shy_params P) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const long long q = shy_q32(h[i]);
    CellQ c;
    c.hq = q;
    c.e = 0;
    const float e = P.deposition_rate * (1.0f - root[i]);
    c.effd = e < 0.0f ? 0.0f : e;
    c.spare = 0;
    c.cnt[0] = 0;
    c.cnt[1] = 0;
    s->cq[i] = c;
    h[i] = shy_unq(q);
    s->rec[i] = make_float4(mx[i], my[i], d[i], 1.0f + P.entrainment * shy_erff_ff(0.4f * d[i]));
    s->effd[i] = c.effd;
    Tracks t;
    t.td = t.tmx = t.tmy = t.pad = 0;
    s->trk[i] = t;
  }
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < words;
       i += (long long)gridDim.x * blockDim.x)
    s->arr[i] = 0;
}

// Discharge and momentum back to the caller's maps.
__global__ void noalloc_unpack_kernel(const NoallocScratch* s, int n, float* d, float* mx, float* my) {
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
    const float4 r = s->rec[i];
    mx[i] = r.x;
    my[i] = r.y;
    d[i] = r.z;
  }
}

}  // namespace

}  // namespace shy

using namespace shy;

extern "C" int shy_erode_noalloc(int nx, int ny, const shy_params* params, uint64_t seed, uint64_t cycle0,
                                 int drops, int cycles, float* height, float* discharge, float* momentum_x,
                                 float* momentum_y, const float* root_density, void* stream, shy_stats* stats) {
  if (!params || !height || !discharge || !momentum_x || !momentum_y || !root_density) {
    set_error("shy_erode_noalloc: null parameters or map pointer");
    return SHY_ERR_INVALID_ARG;
  }
  if (nx < 1 || ny < 1 || (long long)nx * ny > SHY_NOALLOC_MAX_CELLS) {
    set_error("shy_erode_noalloc: %d x %d map exceeds the fixed scratch of %d cells", nx, ny,
              SHY_NOALLOC_MAX_CELLS);
    return SHY_ERR_INVALID_ARG;
  }
  if (2 * arr_words(nx, ny) > (long long)(sizeof(((NoallocScratch*)nullptr)->arr) / sizeof(unsigned long long))) {
    set_error("shy_erode_noalloc: %d x %d map exceeds the fixed arrivals bitmap", nx, ny);
    return SHY_ERR_INVALID_ARG;
  }
  if (drops < 0 || drops > SHY_NOALLOC_MAX_DROPS || cycles < 0) {
    set_error("shy_erode_noalloc: %d drops per cycle exceeds the fixed scratch of %d (or cycles < 0)", drops,
              SHY_NOALLOC_MAX_DROPS);
    return SHY_ERR_INVALID_ARG;
  }
  // the allocating path's checks (NaN fails them), plus the table's limit
  if (!params_valid(params) || params->max_age > (float)SHY_NOALLOC_MAX_AGE) {
    set_error("shy_erode_noalloc: invalid parameters (max_age must lie in [0, %d], evap_rate in [0, 1), "
              "map_scale finite)", SHY_NOALLOC_MAX_AGE);
    return SHY_ERR_INVALID_ARG;
  }
  if (params->cascade_passes != 0) {
    set_error("shy_erode_noalloc: cascade_passes must be 0 (the relax stencil needs a second height buffer)");
    return SHY_ERR_INVALID_ARG;
  }
  cudaStream_t s = static_cast<cudaStream_t>(stream);
  NoallocScratch* sc = nullptr;
  cudaError_t e = scratch_for_device(&sc);
  if (e != cudaSuccess) return cuda_fail(e, "shy_erode_noalloc: scratch address");
  int dev = 0, sms = 0;
  if ((e = cudaGetDevice(&dev)) != cudaSuccess) return cuda_fail(e, "shy_erode_noalloc: device");
  if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess)
    return cuda_fail(e, "shy_erode_noalloc: device attributes");
  // Every map must be device (or managed) memory of the current device: a
  // host pointer would otherwise become a fault inside the first kernel.
  // cudaPointerGetAttributes allocates nothing.
  const void* maps[5] = {height, discharge, momentum_x, momentum_y, root_density};
  static const char* const names[5] = {"height", "discharge", "momentum_x", "momentum_y", "root_density"};
  for (int i = 0; i < 5; ++i) {
    cudaPointerAttributes at;
    e = cudaPointerGetAttributes(&at, maps[i]);
    if (e != cudaSuccess) {
      cudaGetLastError();  // an unknown pointer leaves no sticky error
      set_error("shy_erode_noalloc: %s is not a CUDA pointer", names[i]);
      return SHY_ERR_INVALID_ARG;
    }
    const bool dev_mem = at.type == cudaMemoryTypeDevice || at.type == cudaMemoryTypeManaged;
    if (!dev_mem || (at.type == cudaMemoryTypeDevice && at.device != dev)) {
      set_error("shy_erode_noalloc: %s is not device memory of the current device", names[i]);
      return SHY_ERR_INVALID_ARG;
    }
  }

  const int n = nx * ny;
  Terrain T;
  T.cell_base = 0;
  T.arr_base = 0;
  T.nx = nx;
  T.ny = ny;
  T.drop_base = 0;
  T.drops = drops;
  T.seed = seed;
  const int blocks = (n + 255) / 256 < 1024 ? (n + 255) / 256 : 1024;
  noalloc_init_kernel<<<1, 32, 0, s>>>(sc, T, cycle0, params->evap_rate, (int)params->max_age + 3);
  noalloc_pack_kernel<<<blocks, 256, 0, s>>>(sc, n, 2 * arr_words(nx, ny), height, discharge, momentum_x,
                                             momentum_y, root_density, *params);
  if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(e, "shy_erode_noalloc: set-up kernels");

  CycleBuffers b;
  b.terrains = &sc->terrain;
  b.n_terrains = 1;
  b.total_drops = drops;
  b.cells = n;
  b.h = height;
  b.cq = sc->cq;
  b.rec = sc->rec;
  b.voltab = sc->voltab;
  b.trk = sc->trk;
  b.track_f = sc->track_f;
  b.pos = sc->pos;
  b.spd = sc->spd;
  b.sed = sc->sed;
  b.age = sc->age;
  b.own = sc->own;
  b.terr = sc->terr;
  b.cell = sc->cell;
  b.ctr = sc->ctr;
  b.steep = sc->steep;
  b.arr = sc->arr;
  b.arr_words = arr_words(nx, ny);
  b.st = &sc->st;
  b.bar = &sc->bar;
  b.P = *params;
  b.sm_count = sms;
  for (int c = 0; c < cycles; ++c)
    if ((e = launch_cycle_buffers(b, s)) != cudaSuccess) return cuda_fail(e, "shy_erode_noalloc: cycle");
  noalloc_unpack_kernel<<<blocks, 256, 0, s>>>(sc, n, discharge, momentum_x, momentum_y);
  if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail(e, "shy_erode_noalloc: unpack");

  int err = 0;
  DevStats st;
  if ((e = cudaMemcpyAsync(&err, &sc->bar.error, sizeof(int), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
      (e = cudaMemcpyAsync(&st, &sc->st, sizeof(st), cudaMemcpyDeviceToHost, s)) != cudaSuccess ||
      (e = cudaStreamSynchronize(s)) != cudaSuccess)
    return cuda_fail(e, "shy_erode_noalloc: status");
  if (err != 0) {
    set_error(err == SHY_ERR_TIMEOUT ? "shy_erode_noalloc: a grid barrier timed out"
                                     : "shy_erode_noalloc: cycle ended with drops still descending");
    return err;
  }
  if (stats) {
    stats->cycles = st.cycles;
    stats->drops = st.drops;
    stats->drops_skipped = st.skipped;
    stats->drops_oob = st.oob;
    stats->drop_steps = st.steps;
    stats->evap_gain = (double)st.gain_q / 4294967296.0;
    stats->boundary_loss = (double)st.loss_q / 4294967296.0;
  }
  return SHY_OK;
}
