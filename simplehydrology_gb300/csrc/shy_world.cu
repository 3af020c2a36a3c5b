// shy_world.cu -- the C ABI (include/shy.h): world lifecycle, field I/O,
// erosion entry points, counters and timing.  Host code only; the kernels
// live in shy_exact.cu and shy_lockstep.cu.
#include <atomic>
#include <math.h>
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <vector>

#include "shy_internal.h"

namespace shy {

namespace {
thread_local char g_err[512] = "";
}

void set_error(const char* fmt, ...) {
  va_list ap;
  va_start(ap, fmt);
  vsnprintf(g_err, sizeof(g_err), fmt, ap);
  va_end(ap);
}

int cuda_fail(cudaError_t e, const char* what) {
  set_error("%s: %s (%s)", what, cudaGetErrorString(e), cudaGetErrorName(e));
  if (e == cudaErrorMemoryAllocation) return SHY_ERR_OUT_OF_MEMORY;
  if (e == cudaErrorNoDevice || e == cudaErrorInsufficientDriver) return SHY_ERR_NO_DEVICE;
  return SHY_ERR_CUDA;
}

cudaError_t timing_begin(shy_world* w, int kind, int* slot) {
  *slot = -1;
  if (!w->timing.on) return cudaSuccess;
  cudaEvent_t ev[2];
  for (int i = 0; i < 2; ++i) {
    if (!w->timing.spare.empty()) {
      ev[i] = w->timing.spare.back();
      w->timing.spare.pop_back();
    } else {
      cudaError_t e = cudaEventCreate(&ev[i]);
      if (e != cudaSuccess) return e;
    }
  }
  cudaError_t e = cudaEventRecord(ev[0], w->stream);
  if (e != cudaSuccess) return e;
  w->timing.pending.push_back({ev[0], ev[1], kind});
  *slot = (int)w->timing.pending.size() - 1;
  return cudaSuccess;
}

cudaError_t timing_end(shy_world* w, int slot) {
  if (slot < 0) return cudaSuccess;
  return cudaEventRecord(w->timing.pending[slot].b, w->stream);
}

static cudaError_t timing_collect(shy_world* w) {
  for (auto& p : w->timing.pending) {
    cudaError_t e = cudaEventSynchronize(p.b);
    if (e != cudaSuccess) return e;
    float ms = 0.0f;
    e = cudaEventElapsedTime(&ms, p.a, p.b);
    if (e != cudaSuccess) return e;
    w->timing.ms[p.kind] += ms;
    w->timing.launches[p.kind] += 1;
    w->timing.spare.push_back(p.a);
    w->timing.spare.push_back(p.b);
  }
  w->timing.pending.clear();
  return cudaSuccess;
}

std::atomic<unsigned long long> g_debug_stall_ns{0};
unsigned long long debug_stall_ns() { return g_debug_stall_ns.load(std::memory_order_relaxed); }

// Written so that a NaN in any tested field fails the test.
bool params_valid(const shy_params* p) {
  return p && p->max_age >= 0.0f && p->max_age < 1.0e6f && p->evap_rate >= 0.0f &&
         p->evap_rate < 1.0f && p->cascade_passes >= 0 && p->cascade_passes <= 64 &&
         isfinite(p->map_scale);
}

}  // namespace shy

using namespace shy;

namespace {

template <class T> cudaError_t dalloc(T** p, size_t n) {
  return cudaMalloc((void**)p, sizeof(T) * (n ? n : 1));
}

void free_world(shy_world* w) {
  if (!w) return;
  if (w->stream) cudaStreamSynchronize(w->stream);
  if (w->gexec) cudaGraphExecDestroy(w->gexec);
  void* ptrs[] = {w->h, w->root, w->plant, w->track_f, w->rec, w->effd, w->trk, w->cq, w->scratch, w->relax, w->dpos, w->dspd, w->dsed, w->dage,
                  w->dterr, w->dcell, w->dctr, w->dterrains, w->stats, w->bar, w->ddrop,
                  w->dtrace, w->dint, w->dspawn, w->normals, w->hq_relax, w->voltab, w->down,
                  w->plant_next, w->rootq, w->veg_claim, w->arr, w->feed, w->crand, w->plants, w->stage, w->dorder, w->dkey, w->drank, w->dhist,
                  w->dsteep, w->dpos2, w->dspd2, w->dsed2, w->dage2, w->dterr2, w->dresort};
  for (void* p : ptrs)
    if (p) cudaFree(p);
  for (auto& p : w->timing.pending) {
    cudaEventDestroy(p.a);
    cudaEventDestroy(p.b);
  }
  for (auto e : w->timing.spare) cudaEventDestroy(e);
  if (w->stream) cudaStreamDestroy(w->stream);
  delete w;
}

int alloc_drop_slots(shy_world* w, int n) {
  if (n <= w->max_drops) return SHY_OK;
  void* ptrs[] = {w->dpos, w->dspd, w->dsed, w->dage, w->dterr, w->dcell, w->dctr, w->down,
                  w->dsteep, w->dorder, w->dkey, w->drank, w->dpos2, w->dspd2, w->dsed2, w->dage2, w->dterr2};
  SHY_CHECK_CUDA(cudaStreamSynchronize(w->stream), "synchronize");
  for (void* p : ptrs)
    if (p) cudaFree(p);
  w->dpos = w->dspd = nullptr;
  w->dsed = nullptr;
  w->dage = w->dterr = nullptr;
  w->down = nullptr;
  w->dsteep = nullptr;
  w->dorder = w->dkey = w->drank = nullptr;
  w->dcell = w->dctr = nullptr;
  w->dpos2 = w->dspd2 = nullptr;
  w->dsed2 = nullptr;
  w->dage2 = w->dterr2 = nullptr;
  w->max_drops = 0;
  SHY_CHECK_CUDA(dalloc(&w->dpos, n), "allocate drop slots");
  SHY_CHECK_CUDA(dalloc(&w->dspd, n), "allocate drop slots");
  SHY_CHECK_CUDA(dalloc(&w->dsed, n), "allocate drop slots");
  SHY_CHECK_CUDA(dalloc(&w->dage, n), "allocate drop slots");
  SHY_CHECK_CUDA(dalloc(&w->dterr, n), "allocate drop slots");
  SHY_CHECK_CUDA(dalloc(&w->dcell, n), "allocate drop slots");
  SHY_CHECK_CUDA(dalloc(&w->dctr, n), "allocate drop slots");
  SHY_CHECK_CUDA(dalloc(&w->down, n), "allocate drop slots");
  SHY_CHECK_CUDA(dalloc(&w->dsteep, n), "allocate drop slots");
  SHY_CHECK_CUDA(dalloc(&w->dorder, n), "allocate drop slots");
  SHY_CHECK_CUDA(dalloc(&w->dkey, n), "allocate drop slots");
  SHY_CHECK_CUDA(dalloc(&w->drank, n), "allocate drop slots");
  SHY_CHECK_CUDA(dalloc(&w->dpos2, n), "allocate drop slots");
  SHY_CHECK_CUDA(dalloc(&w->dspd2, n), "allocate drop slots");
  SHY_CHECK_CUDA(dalloc(&w->dsed2, n), "allocate drop slots");
  SHY_CHECK_CUDA(dalloc(&w->dage2, n), "allocate drop slots");
  SHY_CHECK_CUDA(dalloc(&w->dterr2, n), "allocate drop slots");
  if (!w->dhist) SHY_CHECK_CUDA(dalloc(&w->dhist, 65536), "allocate drop slots");
  if (!w->dresort) SHY_CHECK_CUDA(dalloc(&w->dresort, shy::kResortBuckets), "allocate drop slots");
  w->max_drops = n;
  return SHY_OK;
}

int upload_terrains(shy_world* w) {
  int base = 0;
  for (auto& T : w->terrains) {
    T.drop_base = base;
    base += T.drops;
  }
  int rc = alloc_drop_slots(w, base);
  if (rc != SHY_OK) return rc;
  SHY_CHECK_CUDA(cudaMemcpyAsync(w->dterrains, w->terrains.data(), sizeof(Terrain) * w->terrains.size(),
                                 cudaMemcpyHostToDevice, w->stream),
                 "upload terrain table");
  SHY_CHECK_CUDA(cudaStreamSynchronize(w->stream), "synchronize");
  return SHY_OK;
}

// Drop volume after k evaporations, (float)((double)v * (1 - evap)) applied k
// times from 1 (source/water.h:136): volume depends on nothing else, so the
// batched kernel looks it up by age.
int upload_volume_table(shy_world* w) {
  const int n = (int)w->P.max_age + 3;
  std::vector<float> v((size_t)n);
  v[0] = 1.0f;
  for (int k = 1; k < n; ++k) v[k] = (float)((double)v[k - 1] * (1.0 - (double)w->P.evap_rate));
  if (n > w->voltab_len) {
    if (w->voltab) cudaFree(w->voltab);
    w->voltab = nullptr;
    w->voltab_len = 0;
    SHY_CHECK_CUDA(cudaMalloc((void**)&w->voltab, sizeof(float) * n), "allocate volume table");
    w->voltab_len = n;
  }
  SHY_CHECK_CUDA(cudaMemcpyAsync(w->voltab, v.data(), sizeof(float) * n, cudaMemcpyHostToDevice, w->stream),
                 "upload volume table");
  SHY_CHECK_CUDA(cudaStreamSynchronize(w->stream), "synchronize");
  return SHY_OK;
}

// A batched call's device status.  On an error the cycle's leftovers are
// cleared (launch_batched_recover) so that the world stays usable; its
// heights are those the failed cycle had reached.
int check_device_error(shy_world* w) {
  GridBar b;
  SHY_CHECK_CUDA(cudaMemcpyAsync(&b, w->bar, sizeof(b), cudaMemcpyDeviceToHost, w->stream), "read status");
  SHY_CHECK_CUDA(cudaStreamSynchronize(w->stream), "synchronize");
  if (b.error != 0) {
    SHY_CHECK_CUDA(launch_batched_recover(w), "clear after a failed cycle");
    SHY_CHECK_CUDA(cudaStreamSynchronize(w->stream), "synchronize");
    set_error(b.error == SHY_ERR_TIMEOUT ? "a grid barrier of the lock-step kernel timed out"
                                         : "lock-step kernel ended with drops still descending");
    return b.error;
  }
  return SHY_OK;
}

int create_world(int n, const int* nx, const int* ny, const int* drops, const uint64_t* seeds,
                 const shy_params* params, shy_world** out) {
  if (!out) {
    set_error("null output handle");
    return SHY_ERR_INVALID_ARG;
  }
  *out = nullptr;
  if (n <= 0 || n > 65536 || !nx || !ny || !seeds) {
    set_error("invalid terrain list");
    return SHY_ERR_INVALID_ARG;
  }
  shy_params P;
  if (params) {
    if (!params_valid(params)) {
      set_error("invalid parameters");
      return SHY_ERR_INVALID_ARG;
    }
    P = *params;
  } else {
    shy_params_default(&P);
  }
  long long cells = 0;
  long long words = 0;  // arrivals bitmap
  long long total_drops = 0;
  std::vector<Terrain> terr(n);
  for (int i = 0; i < n; ++i) {
    if (nx[i] < 1 || ny[i] < 1 || (long long)nx[i] * ny[i] > (1ll << 31)) {
      set_error("terrain %d: invalid size %d x %d", i, nx[i], ny[i]);
      return SHY_ERR_INVALID_ARG;
    }
    const int dn = drops ? drops[i] : 0;
    if (dn < 0) {
      set_error("terrain %d: negative drop count", i);
      return SHY_ERR_INVALID_ARG;
    }
    terr[i].cell_base = cells;
    terr[i].arr_base = words;
    terr[i].nx = nx[i];
    terr[i].ny = ny[i];
    terr[i].drops = dn;
    terr[i].drop_base = 0;
    terr[i].seed = seeds[i];
    cells += (long long)nx[i] * ny[i];
    words += arr_words(nx[i], ny[i]);
    total_drops += dn;
  }
  if (total_drops > (1ll << 30)) {
    set_error("too many drops per cycle");
    return SHY_ERR_INVALID_ARG;
  }
  int ndev = 0;
  cudaError_t ce = cudaGetDeviceCount(&ndev);
  if (ce != cudaSuccess || ndev == 0) {
    set_error("no CUDA device: %s", ce != cudaSuccess ? cudaGetErrorString(ce) : "count is 0");
    return SHY_ERR_NO_DEVICE;
  }
  shy_world* w = new shy_world();
  w->P = P;
  w->terrains = terr;
  w->cells = cells;
  int rc = SHY_OK;
  auto fail = [&](cudaError_t e, const char* what) {
    rc = cuda_fail(e, what);
    free_world(w);
    return rc;
  };
  cudaError_t e;
  if ((e = cudaGetDevice(&w->device)) != cudaSuccess) return fail(e, "get device");
  if ((e = cudaDeviceGetAttribute(&w->sm_count, cudaDevAttrMultiProcessorCount, w->device)) != cudaSuccess)
    return fail(e, "device attributes");
  int l2 = 0;
  if ((e = cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, w->device)) != cudaSuccess)
    return fail(e, "device attributes");
  w->l2_bytes = l2;
  if ((e = cudaStreamCreateWithFlags(&w->stream, cudaStreamNonBlocking)) != cudaSuccess)
    return fail(e, "create stream");
  const size_t N = (size_t)cells;
  if ((e = dalloc(&w->h, N)) != cudaSuccess) return fail(e, "allocate maps");
  if ((e = dalloc(&w->root, N)) != cudaSuccess) return fail(e, "allocate maps");
  if ((e = dalloc(&w->plant, N)) != cudaSuccess) return fail(e, "allocate maps");
  if ((e = dalloc(&w->track_f, 3 * N)) != cudaSuccess) return fail(e, "allocate maps");
  if ((e = dalloc(&w->rec, N)) != cudaSuccess) return fail(e, "allocate maps");
  if ((e = dalloc(&w->effd, N)) != cudaSuccess) return fail(e, "allocate maps");
  if ((e = dalloc(&w->trk, N)) != cudaSuccess) return fail(e, "allocate maps");
  if ((e = dalloc(&w->cq, N)) != cudaSuccess) return fail(e, "allocate maps");
  if ((e = dalloc(&w->scratch, N)) != cudaSuccess) return fail(e, "allocate maps");
  if ((e = dalloc(&w->relax, N)) != cudaSuccess) return fail(e, "allocate maps");
  if ((e = dalloc(&w->arr, 2 * (size_t)words)) != cudaSuccess) return fail(e, "allocate maps");
  w->arr_words = words;
  if ((e = dalloc(&w->dterrains, (size_t)n)) != cudaSuccess) return fail(e, "allocate terrain table");
  if ((e = dalloc(&w->stats, 1)) != cudaSuccess) return fail(e, "allocate counters");
  if ((e = dalloc(&w->bar, 1)) != cudaSuccess) return fail(e, "allocate counters");
  if ((e = dalloc(&w->ddrop, 1)) != cudaSuccess) return fail(e, "allocate drop");
  if ((e = dalloc(&w->dint, 16)) != cudaSuccess) return fail(e, "allocate scratch");
  cudaStream_t s = w->stream;
  cudaMemsetAsync(w->h, 0, sizeof(float) * N, s);
  cudaMemsetAsync(w->root, 0, sizeof(float) * N, s);
  cudaMemsetAsync(w->plant, 0, sizeof(float) * N, s);
  cudaMemsetAsync(w->track_f, 0, sizeof(float) * 3 * N, s);
  cudaMemsetAsync(w->rec, 0, sizeof(float4) * N, s);
  cudaMemsetAsync(w->trk, 0, sizeof(Tracks) * N, s);
  cudaMemsetAsync(w->cq, 0, sizeof(CellQ) * N, s);
  cudaMemsetAsync(w->arr, 0, sizeof(unsigned long long) * 2 * (size_t)words, s);
  cudaMemsetAsync(w->stats, 0, sizeof(DevStats), s);
  cudaMemsetAsync(w->bar, 0, sizeof(GridBar), s);
  if ((e = cudaGetLastError()) != cudaSuccess) return fail(e, "initialise maps");
  if ((e = launch_rebuild_records(w, -1)) != cudaSuccess) return fail(e, "initialise records");
  w->ceq_source = ERF_DEVICE;
  if ((rc = upload_volume_table(w)) != SHY_OK) {
    free_world(w);
    return rc;
  }
  rc = upload_terrains(w);
  if (rc != SHY_OK) {
    free_world(w);
    return rc;
  }
  *out = w;
  return SHY_OK;
}

bool valid_field(int f) { return f >= 0 && f < SHY_FIELD_COUNT; }

// positions handed to a kernel: finite and well inside int range
bool finite_pos(float x, float y) {
  return isfinite(x) && isfinite(y) && fabsf(x) < 16777216.0f && fabsf(y) < 16777216.0f;
}

// rec component of a field stored inside the per-cell record, else -1
int rec_comp(int field) {
  switch (field) {
    case SHY_FIELD_MOMENTUM_X: return 0;
    case SHY_FIELD_MOMENTUM_Y: return 1;
    case SHY_FIELD_DISCHARGE: return 2;
    default: return -1;
  }
}

float* plain_field(shy_world* w, int t, int field) {
  const long long b = w->terrains[t].cell_base, N = w->cells;
  switch (field) {
    case SHY_FIELD_HEIGHT: return w->h + b;
    case SHY_FIELD_DISCHARGE_TRACK: return w->track_f + b;
    case SHY_FIELD_MOMENTUM_X_TRACK: return w->track_f + N + b;
    case SHY_FIELD_MOMENTUM_Y_TRACK: return w->track_f + 2 * N + b;
    case SHY_FIELD_ROOT_DENSITY: return w->root + b;
    case SHY_FIELD_PLANT_SIZE: return w->plant + b;
    default: return nullptr;
  }
}

// Brings the ceqfac component of the records to the world's erf source.
int ensure_ceq(shy_world* w, int source) {
  if (w->ceq_source == source) return SHY_OK;
  if (source == ERF_DEVICE) {
    SHY_CHECK_CUDA(launch_rebuild_records(w, -1), "rebuild records");
    w->ceq_source = ERF_DEVICE;
    return SHY_OK;
  }
  // The C library's erff on the host, as the reference calls it
  // (source/cellpool.h:242-244), for bit parity with a reference build.
  std::vector<float> d;
  for (size_t t = 0; t < w->terrains.size(); ++t) {
    const long long n = (long long)w->terrains[t].nx * w->terrains[t].ny;
    d.resize((size_t)n);
    SHY_CHECK_CUDA(launch_gather_comp(w, (int)t, 2, w->scratch), "gather discharge");
    SHY_CHECK_CUDA(cudaMemcpyAsync(d.data(), w->scratch, sizeof(float) * n, cudaMemcpyDeviceToHost, w->stream),
                   "download discharge");
    SHY_CHECK_CUDA(cudaStreamSynchronize(w->stream), "synchronize");
    for (long long i = 0; i < n; ++i) d[i] = 1.0f + w->P.entrainment * erff(0.4f * d[i]);
    SHY_CHECK_CUDA(cudaMemcpyAsync(w->scratch, d.data(), sizeof(float) * n, cudaMemcpyHostToDevice, w->stream),
                   "upload records");
    SHY_CHECK_CUDA(launch_scatter_comp(w, (int)t, 3, w->scratch), "scatter records");
    SHY_CHECK_CUDA(cudaStreamSynchronize(w->stream), "synchronize");
  }
  w->ceq_source = ERF_HOST_LIBM;
  return SHY_OK;
}

int check_world(shy_world* w) {
  if (!w) {
    set_error("null world");
    return SHY_ERR_INVALID_ARG;
  }
  return SHY_OK;
}

int check_terrain(shy_world* w, int t) {
  int rc = check_world(w);
  if (rc) return rc;
  if (t < 0 || t >= (int)w->terrains.size()) {
    set_error("terrain index %d out of range", t);
    return SHY_ERR_INVALID_ARG;
  }
  return SHY_OK;
}

}  // namespace

namespace shy {
// world construction and teardown for the other translation units
int world_create(int n, const int* nx, const int* ny, const int* drops, const uint64_t* seeds,
                 const shy_params* params, shy_world** out) {
  return create_world(n, nx, ny, drops, seeds, params, out);
}
void world_free(shy_world* w) { free_world(w); }
int world_check(shy_world* w) { return check_world(w); }
}  // namespace shy

extern "C" {

int shy_version(void) { return SHY_ABI_VERSION; }

int shy_debug_stall_waits(uint64_t ns) {
  if (ns > 10000000000ull) {
    set_error("shy_debug_stall_waits: %llu ns is beyond the 10 s a test may wait", (unsigned long long)ns);
    return SHY_ERR_INVALID_ARG;
  }
  g_debug_stall_ns.store(ns, std::memory_order_relaxed);
  return SHY_OK;
}

const char* shy_last_error(void) { return g_err; }

int shy_params_default(shy_params* p) {
  if (!p) {
    set_error("null params");
    return SHY_ERR_INVALID_ARG;
  }
  memset(p, 0, sizeof(*p));
  p->evap_rate = 0.001f;          // source/water.h:43
  p->deposition_rate = 0.1f;      // :44
  p->min_vol = 0.01f;             // :45
  p->max_age = 500.0f;            // :46
  p->entrainment = 10.0f;         // :48
  p->gravity = 1.0f;              // :49
  p->momentum_transfer = 1.0f;    // :50
  p->lrate = 0.1f;                // source/world.h:42
  p->max_diff = 0.01f;            // :43
  p->settling = 0.8f;             // :44
  p->map_scale = 80.0f;           // source/cellpool.h:165
  p->plant_max_size = 1.5f;       // source/vegetation.h:38
  p->plant_grow_rate = 0.05f;     // :39
  p->plant_max_steep = 0.8f;      // :40
  p->plant_max_discharge = 0.3f;  // :41
  p->plant_max_height = 0.8f;     // :42
  p->plant_spawn_prob = 1e-4f;
  p->plant_death_prob = 0.001f;   // :71
  p->plant_spread_prob = 0.05f;   // :160
  p->cascade_weight = 0.125f;
  p->cascade_passes = 0;
  return SHY_OK;
}

int shy_world_create(int nx, int ny, const shy_params* params, uint64_t seed, shy_world** out) {
  const int zero = 0;
  return create_world(1, &nx, &ny, &zero, &seed, params, out);
}

int shy_batch_create(int n_terrains, const int* nx, const int* ny, const int* drops_per_cycle,
                     const uint64_t* seeds, const shy_params* params, shy_world** out) {
  if (!drops_per_cycle) {
    set_error("null drop counts");
    return SHY_ERR_INVALID_ARG;
  }
  return create_world(n_terrains, nx, ny, drops_per_cycle, seeds, params, out);
}

int shy_world_destroy(shy_world* w) {
  if (!w) return SHY_OK;
  free_world(w);
  return SHY_OK;
}

int shy_world_set_params(shy_world* w, const shy_params* p) {
  int rc = check_world(w);
  if (rc) return rc;
  if (!params_valid(p)) {
    set_error("invalid parameters");
    return SHY_ERR_INVALID_ARG;
  }
  w->P = *p;
  SHY_CHECK_CUDA(launch_rebuild_records(w, -1), "rebuild records");
  w->ceq_source = ERF_DEVICE;
  SHY_CHECK_CUDA(cudaStreamSynchronize(w->stream), "synchronize");
  return upload_volume_table(w);
}

int shy_world_get_params(shy_world* w, shy_params* out) {
  int rc = check_world(w);
  if (rc) return rc;
  if (!out) {
    set_error("null output");
    return SHY_ERR_INVALID_ARG;
  }
  *out = w->P;
  return SHY_OK;
}

int shy_world_size(shy_world* w, int* nx, int* ny) {
  int rc = check_world(w);
  if (rc) return rc;
  if (nx) *nx = w->terrains[0].nx;
  if (ny) *ny = w->terrains[0].ny;
  return SHY_OK;
}

int shy_batch_size(shy_world* w, int* n_terrains) {
  int rc = check_world(w);
  if (rc) return rc;
  if (n_terrains) *n_terrains = (int)w->terrains.size();
  return SHY_OK;
}

int shy_terrain_size(shy_world* w, int t, int* nx, int* ny, int* drops_per_cycle) {
  int rc = check_terrain(w, t);
  if (rc) return rc;
  if (nx) *nx = w->terrains[t].nx;
  if (ny) *ny = w->terrains[t].ny;
  if (drops_per_cycle) *drops_per_cycle = w->terrains[t].drops;
  return SHY_OK;
}

int shy_terrain_set_field(shy_world* w, int t, int field, const float* host, size_t count) {
  int rc = check_terrain(w, t);
  if (rc) return rc;
  const long long n = (long long)w->terrains[t].nx * w->terrains[t].ny;
  if (!valid_field(field) || !host || count != (size_t)n) {
    set_error("set_field: bad field %d, pointer or count %zu (want %lld)", field, count, n);
    return SHY_ERR_INVALID_ARG;
  }
  const int comp = rec_comp(field);
  float* dst = comp >= 0 ? w->scratch : plain_field(w, t, field);
  SHY_CHECK_CUDA(cudaMemcpyAsync(dst, host, sizeof(float) * n, cudaMemcpyHostToDevice, w->stream), "upload field");
  if (field == SHY_FIELD_HEIGHT) w->hq_stale = true;
  if (comp >= 0) SHY_CHECK_CUDA(launch_scatter_comp(w, t, comp, w->scratch), "scatter field");
  if (field == SHY_FIELD_DISCHARGE || field == SHY_FIELD_ROOT_DENSITY) {
    SHY_CHECK_CUDA(launch_rebuild_records(w, -1), "rebuild records");
    w->ceq_source = ERF_DEVICE;
  }
  SHY_CHECK_CUDA(cudaStreamSynchronize(w->stream), "synchronize");
  return SHY_OK;
}

int shy_terrain_get_field(shy_world* w, int t, int field, float* host, size_t count) {
  int rc = check_terrain(w, t);
  if (rc) return rc;
  const long long n = (long long)w->terrains[t].nx * w->terrains[t].ny;
  if (!valid_field(field) || !host || count != (size_t)n) {
    set_error("get_field: bad field %d, pointer or count %zu (want %lld)", field, count, n);
    return SHY_ERR_INVALID_ARG;
  }
  const int comp = rec_comp(field);
  const float* src = plain_field(w, t, field);
  if (comp >= 0) {
    SHY_CHECK_CUDA(launch_gather_comp(w, t, comp, w->scratch), "gather field");
    src = w->scratch;
  }
  SHY_CHECK_CUDA(cudaMemcpyAsync(host, src, sizeof(float) * n, cudaMemcpyDeviceToHost, w->stream), "download field");
  SHY_CHECK_CUDA(cudaStreamSynchronize(w->stream), "synchronize");
  return SHY_OK;
}

// The state a front end exchanges every frame, in one call each way: three
// staging buffers (scratch, the relax buffer, stage) hold the record
// components on the device.
int shy_terrain_set_state(shy_world* w, int t, const float* height, const float* discharge,
                          const float* momentum_x, const float* momentum_y, size_t count) {
  int rc = check_terrain(w, t);
  if (rc) return rc;
  const long long n = (long long)w->terrains[t].nx * w->terrains[t].ny;
  if (count != (size_t)n) {
    set_error("set_state: count %zu, want %lld", count, n);
    return SHY_ERR_INVALID_ARG;
  }
  if (momentum_y && !w->stage) SHY_CHECK_CUDA(dalloc(&w->stage, (size_t)w->cells), "allocate staging");
  const size_t bytes = sizeof(float) * (size_t)n;
  cudaStream_t s = w->stream;
  if (height) {
    SHY_CHECK_CUDA(cudaMemcpyAsync(w->h + w->terrains[t].cell_base, height, bytes, cudaMemcpyHostToDevice, s),
                   "upload heights");
    w->hq_stale = true;
  }
  if (discharge) SHY_CHECK_CUDA(cudaMemcpyAsync(w->scratch, discharge, bytes, cudaMemcpyHostToDevice, s), "upload");
  if (momentum_x) SHY_CHECK_CUDA(cudaMemcpyAsync(w->relax, momentum_x, bytes, cudaMemcpyHostToDevice, s), "upload");
  if (momentum_y) SHY_CHECK_CUDA(cudaMemcpyAsync(w->stage, momentum_y, bytes, cudaMemcpyHostToDevice, s), "upload");
  if (discharge || momentum_x || momentum_y)
    SHY_CHECK_CUDA(launch_pack_state(w, t, discharge ? w->scratch : nullptr, momentum_x ? w->relax : nullptr,
                                     momentum_y ? w->stage : nullptr),
                   "pack state");
  if (discharge) w->ceq_source = ERF_DEVICE;
  SHY_CHECK_CUDA(cudaStreamSynchronize(s), "synchronize");
  return SHY_OK;
}

int shy_terrain_get_state(shy_world* w, int t, float* height, float* discharge, float* momentum_x,
                          float* momentum_y, size_t count) {
  int rc = check_terrain(w, t);
  if (rc) return rc;
  const long long n = (long long)w->terrains[t].nx * w->terrains[t].ny;
  if (count != (size_t)n) {
    set_error("get_state: count %zu, want %lld", count, n);
    return SHY_ERR_INVALID_ARG;
  }
  if (momentum_y && !w->stage) SHY_CHECK_CUDA(dalloc(&w->stage, (size_t)w->cells), "allocate staging");
  const size_t bytes = sizeof(float) * (size_t)n;
  cudaStream_t s = w->stream;
  if (discharge || momentum_x || momentum_y)
    SHY_CHECK_CUDA(launch_unpack_state(w, t, discharge ? w->scratch : nullptr, momentum_x ? w->relax : nullptr,
                                       momentum_y ? w->stage : nullptr),
                   "unpack state");
  if (height)
    SHY_CHECK_CUDA(cudaMemcpyAsync(height, w->h + w->terrains[t].cell_base, bytes, cudaMemcpyDeviceToHost, s),
                   "download heights");
  if (discharge) SHY_CHECK_CUDA(cudaMemcpyAsync(discharge, w->scratch, bytes, cudaMemcpyDeviceToHost, s), "download");
  if (momentum_x) SHY_CHECK_CUDA(cudaMemcpyAsync(momentum_x, w->relax, bytes, cudaMemcpyDeviceToHost, s), "download");
  if (momentum_y) SHY_CHECK_CUDA(cudaMemcpyAsync(momentum_y, w->stage, bytes, cudaMemcpyDeviceToHost, s), "download");
  SHY_CHECK_CUDA(cudaStreamSynchronize(s), "synchronize");
  return SHY_OK;
}

// Every terrain's state in one call each way: the arrays hold all cells,
// terrain after terrain in creation order (the world's own packing).
int shy_world_set_state(shy_world* w, const float* height, const float* discharge, const float* momentum_x,
                        const float* momentum_y, size_t count) {
  int rc = check_world(w);
  if (rc) return rc;
  if (count != (size_t)w->cells) {
    set_error("shy_world_set_state: count %zu, want %lld (all terrains' cells)", count, w->cells);
    return SHY_ERR_INVALID_ARG;
  }
  if (momentum_y && !w->stage) SHY_CHECK_CUDA(dalloc(&w->stage, (size_t)w->cells), "allocate staging");
  const size_t bytes = sizeof(float) * (size_t)w->cells;
  cudaStream_t s = w->stream;
  if (height) {
    SHY_CHECK_CUDA(cudaMemcpyAsync(w->h, height, bytes, cudaMemcpyHostToDevice, s), "upload heights");
    w->hq_stale = true;
  }
  if (discharge) SHY_CHECK_CUDA(cudaMemcpyAsync(w->scratch, discharge, bytes, cudaMemcpyHostToDevice, s), "upload");
  if (momentum_x) SHY_CHECK_CUDA(cudaMemcpyAsync(w->relax, momentum_x, bytes, cudaMemcpyHostToDevice, s), "upload");
  if (momentum_y) SHY_CHECK_CUDA(cudaMemcpyAsync(w->stage, momentum_y, bytes, cudaMemcpyHostToDevice, s), "upload");
  if (discharge || momentum_x || momentum_y)
    SHY_CHECK_CUDA(launch_pack_state_all(w, discharge ? w->scratch : nullptr, momentum_x ? w->relax : nullptr,
                                         momentum_y ? w->stage : nullptr),
                   "pack state");
  if (discharge) w->ceq_source = ERF_DEVICE;
  SHY_CHECK_CUDA(cudaStreamSynchronize(s), "synchronize");
  return SHY_OK;
}

int shy_world_get_state(shy_world* w, float* height, float* discharge, float* momentum_x, float* momentum_y,
                        size_t count) {
  int rc = check_world(w);
  if (rc) return rc;
  if (count != (size_t)w->cells) {
    set_error("shy_world_get_state: count %zu, want %lld (all terrains' cells)", count, w->cells);
    return SHY_ERR_INVALID_ARG;
  }
  if (momentum_y && !w->stage) SHY_CHECK_CUDA(dalloc(&w->stage, (size_t)w->cells), "allocate staging");
  const size_t bytes = sizeof(float) * (size_t)w->cells;
  cudaStream_t s = w->stream;
  if (discharge || momentum_x || momentum_y)
    SHY_CHECK_CUDA(launch_unpack_state_all(w, discharge ? w->scratch : nullptr, momentum_x ? w->relax : nullptr,
                                           momentum_y ? w->stage : nullptr),
                   "unpack state");
  if (height) SHY_CHECK_CUDA(cudaMemcpyAsync(height, w->h, bytes, cudaMemcpyDeviceToHost, s), "download heights");
  if (discharge) SHY_CHECK_CUDA(cudaMemcpyAsync(discharge, w->scratch, bytes, cudaMemcpyDeviceToHost, s), "download");
  if (momentum_x) SHY_CHECK_CUDA(cudaMemcpyAsync(momentum_x, w->relax, bytes, cudaMemcpyDeviceToHost, s), "download");
  if (momentum_y) SHY_CHECK_CUDA(cudaMemcpyAsync(momentum_y, w->stage, bytes, cudaMemcpyDeviceToHost, s), "download");
  SHY_CHECK_CUDA(cudaStreamSynchronize(s), "synchronize");
  return SHY_OK;
}

// device pointers of the state calls: device (or managed) memory of the
// world's device, or null
static int check_device_ptrs(shy_world* w, const char* fn, const void* const* p, int n) {
  for (int i = 0; i < n; ++i) {
    if (!p[i]) continue;
    cudaPointerAttributes at;
    if (cudaPointerGetAttributes(&at, p[i]) != cudaSuccess) {
      cudaGetLastError();
      set_error("%s: argument %d is not a CUDA pointer", fn, i);
      return SHY_ERR_INVALID_ARG;
    }
    if (!(at.type == cudaMemoryTypeManaged || (at.type == cudaMemoryTypeDevice && at.device == w->device))) {
      set_error("%s: argument %d is not device memory of the world's device", fn, i);
      return SHY_ERR_INVALID_ARG;
    }
  }
  return SHY_OK;
}

int shy_terrain_set_state_device(shy_world* w, int t, const float* height, const float* discharge,
                                 const float* momentum_x, const float* momentum_y, size_t count) {
  int rc = check_terrain(w, t);
  if (rc) return rc;
  const long long n = (long long)w->terrains[t].nx * w->terrains[t].ny;
  if (count != (size_t)n) {
    set_error("set_state_device: count %zu, want %lld", count, n);
    return SHY_ERR_INVALID_ARG;
  }
  const void* ptrs[4] = {height, discharge, momentum_x, momentum_y};
  if ((rc = check_device_ptrs(w, "set_state_device", ptrs, 4)) != SHY_OK) return rc;
  cudaStream_t s = w->stream;
  if (height) {
    SHY_CHECK_CUDA(cudaMemcpyAsync(w->h + w->terrains[t].cell_base, height, sizeof(float) * (size_t)n,
                                   cudaMemcpyDeviceToDevice, s),
                   "copy heights");
    w->hq_stale = true;
  }
  if (discharge || momentum_x || momentum_y)
    SHY_CHECK_CUDA(launch_pack_state(w, t, discharge, momentum_x, momentum_y), "pack state");
  if (discharge) w->ceq_source = ERF_DEVICE;
  SHY_CHECK_CUDA(cudaStreamSynchronize(s), "synchronize");
  return SHY_OK;
}

int shy_terrain_get_state_device(shy_world* w, int t, float* height, float* discharge, float* momentum_x,
                                 float* momentum_y, size_t count) {
  int rc = check_terrain(w, t);
  if (rc) return rc;
  const long long n = (long long)w->terrains[t].nx * w->terrains[t].ny;
  if (count != (size_t)n) {
    set_error("get_state_device: count %zu, want %lld", count, n);
    return SHY_ERR_INVALID_ARG;
  }
  const void* ptrs[4] = {height, discharge, momentum_x, momentum_y};
  if ((rc = check_device_ptrs(w, "get_state_device", ptrs, 4)) != SHY_OK) return rc;
  cudaStream_t s = w->stream;
  if (discharge || momentum_x || momentum_y)
    SHY_CHECK_CUDA(launch_unpack_state(w, t, discharge, momentum_x, momentum_y), "unpack state");
  if (height)
    SHY_CHECK_CUDA(cudaMemcpyAsync(height, w->h + w->terrains[t].cell_base, sizeof(float) * (size_t)n,
                                   cudaMemcpyDeviceToDevice, s),
                   "copy heights");
  SHY_CHECK_CUDA(cudaStreamSynchronize(s), "synchronize");
  return SHY_OK;
}

int shy_world_set_field(shy_world* w, int field, const float* host, size_t count) {
  return shy_terrain_set_field(w, 0, field, host, count);
}

int shy_world_get_field(shy_world* w, int field, float* host, size_t count) {
  return shy_terrain_get_field(w, 0, field, host, count);
}

int shy_world_set_launch(shy_world* w, int grid, int order) {
  int rc = check_world(w);
  if (rc) return rc;
  if (grid < 0 || order < -1 || order > 1) {
    set_error("shy_world_set_launch: grid must be >= 0 and order -1, 0 or 1");
    return SHY_ERR_INVALID_ARG;
  }
  w->batch_grid = grid;
  w->batch_order = order;
  return SHY_OK;
}

int shy_world_set_block(shy_world* w, int threads, int smem_slots) {
  int rc = check_world(w);
  if (rc) return rc;
  if ((threads != 64 && threads != 128 && threads != 256) || smem_slots < 0 || smem_slots > 1) {
    set_error("shy_world_set_block: threads must be 64, 128 or 256 and smem_slots 0 or 1");
    return SHY_ERR_INVALID_ARG;
  }
  w->batch_block = threads;
  w->batch_smem = smem_slots;
  return SHY_OK;
}

int shy_world_set_resort(shy_world* w, int steps) {
  int rc = check_world(w);
  if (rc) return rc;
  if (steps < -1 || steps > 4096) {
    set_error("shy_world_set_resort: steps must be -1 (automatic), 0 (never) or lie in [1, 4096]");
    return SHY_ERR_INVALID_ARG;
  }
  w->batch_resort = steps;
  return SHY_OK;
}

int shy_world_set_settle(shy_world* w, int mode) {
  int rc = check_world(w);
  if (rc) return rc;
  if (mode < -1 || mode > 1) {
    set_error("shy_world_set_settle: mode must be -1 (automatic), 0 or 1");
    return SHY_ERR_INVALID_ARG;
  }
  w->batch_settle = mode;
  return SHY_OK;
}

int shy_world_set_graph(shy_world* w, int cycles_per_graph) {
  int rc = check_world(w);
  if (rc) return rc;
  if (cycles_per_graph < 0 || cycles_per_graph > 4096) {
    set_error("shy_world_set_graph: cycles per graph must lie in [0, 4096]");
    return SHY_ERR_INVALID_ARG;
  }
  w->graph_cycles = cycles_per_graph;
  return SHY_OK;
}

int shy_world_sync(shy_world* w) {
  int rc = check_world(w);
  if (rc) return rc;
  SHY_CHECK_CUDA(cudaStreamSynchronize(w->stream), "synchronize");
  return SHY_OK;
}

int shy_world_stream(shy_world* w, void** stream) {
  int rc = check_world(w);
  if (rc) return rc;
  if (!stream) {
    set_error("null output");
    return SHY_ERR_INVALID_ARG;
  }
  *stream = (void*)w->stream;
  return SHY_OK;
}

int shy_world_stats(shy_world* w, shy_stats* out) {
  int rc = check_world(w);
  if (rc) return rc;
  if (!out) {
    set_error("null output");
    return SHY_ERR_INVALID_ARG;
  }
  DevStats s;
  SHY_CHECK_CUDA(cudaMemcpyAsync(&s, w->stats, sizeof(s), cudaMemcpyDeviceToHost, w->stream), "read counters");
  SHY_CHECK_CUDA(cudaStreamSynchronize(w->stream), "synchronize");
  out->cycles = s.cycles;
  out->drops = s.drops;
  out->drops_skipped = s.skipped;
  out->drops_oob = s.oob;
  out->drop_steps = s.steps;
  out->evap_gain = s.gain_exact + (double)s.gain_q / 4294967296.0;
  out->boundary_loss = s.loss_exact + (double)s.loss_q / 4294967296.0;
  return SHY_OK;
}

int shy_world_reset_stats(shy_world* w) {
  int rc = check_world(w);
  if (rc) return rc;
  SHY_CHECK_CUDA(cudaMemsetAsync(w->stats, 0, sizeof(DevStats), w->stream), "reset counters");
  SHY_CHECK_CUDA(cudaStreamSynchronize(w->stream), "synchronize");
  return SHY_OK;
}

int shy_world_set_cycle(shy_world* w, uint64_t cycle) {
  int rc = check_world(w);
  if (rc) return rc;
  unsigned long long c = cycle;
  SHY_CHECK_CUDA(cudaMemcpyAsync(&w->bar->cycle, &c, sizeof(c), cudaMemcpyHostToDevice, w->stream), "set cycle");
  SHY_CHECK_CUDA(cudaStreamSynchronize(w->stream), "synchronize");
  return SHY_OK;
}

int shy_world_get_cycle(shy_world* w, uint64_t* cycle) {
  int rc = check_world(w);
  if (rc) return rc;
  if (!cycle) {
    set_error("null output");
    return SHY_ERR_INVALID_ARG;
  }
  unsigned long long c = 0;
  SHY_CHECK_CUDA(cudaMemcpyAsync(&c, &w->bar->cycle, sizeof(c), cudaMemcpyDeviceToHost, w->stream), "get cycle");
  SHY_CHECK_CUDA(cudaStreamSynchronize(w->stream), "synchronize");
  *cycle = c;
  return SHY_OK;
}

int shy_world_enable_timing(shy_world* w, int on) {
  int rc = check_world(w);
  if (rc) return rc;
  SHY_CHECK_CUDA(timing_collect(w), "collect timing");
  w->timing.on = on != 0;
  for (int k = 0; k < SHY_KERNEL_KINDS; ++k) {
    w->timing.ms[k] = 0.0;
    w->timing.launches[k] = 0;
  }
  return SHY_OK;
}

int shy_world_timing(shy_world* w, shy_timing* out) {
  int rc = check_world(w);
  if (rc) return rc;
  if (!out) {
    set_error("null output");
    return SHY_ERR_INVALID_ARG;
  }
  SHY_CHECK_CUDA(timing_collect(w), "collect timing");
  memset(out, 0, sizeof(*out));
  for (int k = 0; k < SHY_KERNEL_KINDS; ++k) {
    out->ms[k] = w->timing.ms[k];
    out->launches[k] = w->timing.launches[k];
  }
  return SHY_OK;
}

int shy_world_lockstep_profile(shy_world* w, double* phase_ms, uint64_t* iterations) {
  int rc = check_world(w);
  if (rc) return rc;
  GridBar b;
  SHY_CHECK_CUDA(cudaMemcpyAsync(&b, w->bar, sizeof(b), cudaMemcpyDeviceToHost, w->stream), "read profile");
  SHY_CHECK_CUDA(cudaStreamSynchronize(w->stream), "synchronize");
  if (phase_ms)
    for (int i = 0; i < 6; ++i) phase_ms[i] = (double)b.phase_ns[i] * 1e-6;
  if (iterations) *iterations = b.iterations;
  return SHY_OK;
}

int shy_world_set_erf_source(shy_world* w, int source) {
  int rc = check_world(w);
  if (rc) return rc;
  if (source != SHY_ERF_DEVICE && source != SHY_ERF_HOST_LIBM) {
    set_error("unknown erf source %d", source);
    return SHY_ERR_INVALID_ARG;
  }
  w->erf_source = source;
  return SHY_OK;
}

namespace {

// FNV-1a over what a captured batched cycle bakes in on the host: the
// parameters, the terrain table, the launch shape and every buffer pointer
// the launches take.  A graph is captured again when any of it changed.
unsigned long long launch_key(const shy_world* w) {
  unsigned long long h = 1469598103934665603ull;
  auto mix = [&](const void* p, size_t n) {
    const unsigned char* b = static_cast<const unsigned char*>(p);
    for (size_t i = 0; i < n; ++i) {
      h ^= b[i];
      h *= 1099511628211ull;
    }
  };
  mix(&w->P, sizeof(w->P));
  for (const auto& T : w->terrains) mix(&T, sizeof(T));
  const int shape[8] = {w->batch_grid, w->batch_order, w->batch_block, w->batch_smem, w->graph_cycles, w->sm_count,
                        w->batch_resort, w->batch_settle};
  mix(shape, sizeof(shape));
  const void* ptrs[] = {w->h, w->cq, w->rec, w->voltab, w->trk, w->track_f, w->dpos, w->dspd, w->dsed, w->dage,
                        w->down, w->dterr, w->dcell, w->dctr, w->dsteep, w->arr, w->dorder, w->dkey,
                        w->drank, w->dhist, w->dterrains, w->stats, w->bar, w->relax, w->hq_relax,
                        w->dpos2, w->dspd2, w->dsed2, w->dage2, w->dterr2, w->dresort};
  mix(ptrs, sizeof(ptrs));
  return h;
}

// `cycles` batched cycles: with graph_cycles = K > 0 (and per-kernel timing
// off), runs of K cycles go as one CUDA graph, captured on first use and
// again whenever the launch key changes; the rest launch one by one.  The
// cycle index and the counters live on the device, so every replay takes
// the next spawns.
int run_batched_cycles(shy_world* w, int cycles) {
  const int K = w->graph_cycles;
  int c = 0;
  if (K > 0 && !w->timing.on && cycles >= K) {
    const unsigned long long key = launch_key(w);
    if (w->gexec && w->graph_key != key) {
      cudaGraphExecDestroy(w->gexec);
      w->gexec = nullptr;
    }
    if (!w->gexec) {
      cudaGraph_t g = nullptr;
      SHY_CHECK_CUDA(cudaStreamBeginCapture(w->stream, cudaStreamCaptureModeRelaxed), "begin graph capture");
      cudaError_t e = cudaSuccess;
      for (int i = 0; i < K && e == cudaSuccess; ++i) e = launch_batched_cycle(w);
      const cudaError_t e2 = cudaStreamEndCapture(w->stream, &g);
      if (e == cudaSuccess) e = e2;
      if (e == cudaSuccess) e = cudaGraphInstantiate(&w->gexec, g, 0);
      if (g) cudaGraphDestroy(g);
      if (e != cudaSuccess) {
        w->gexec = nullptr;
        return cuda_fail(e, "capture batched cycles into a CUDA graph");
      }
      w->graph_key = key;
    }
    for (; cycles - c >= K; c += K) SHY_CHECK_CUDA(cudaGraphLaunch(w->gexec, w->stream), "launch graph");
  }
  for (; c < cycles; ++c) SHY_CHECK_CUDA(launch_batched_cycle(w), "batched cycle");
  return SHY_OK;
}

}  // namespace

int shy_batch_erode(shy_world* w, int cycles) {
  int rc = check_world(w);
  if (rc) return rc;
  if (cycles < 0) {
    set_error("negative cycle count");
    return SHY_ERR_INVALID_ARG;
  }
  if ((rc = ensure_ceq(w, ERF_DEVICE)) != SHY_OK) return rc;
  if (w->hq_stale) {
    SHY_CHECK_CUDA(launch_heights_to_fixed(w), "heights to fixed point");
    w->hq_stale = false;
  }
  if (w->P.cascade_passes > 0 && !w->hq_relax)
    SHY_CHECK_CUDA(dalloc(&w->hq_relax, (size_t)w->cells), "allocate relax buffer");
  if ((rc = run_batched_cycles(w, cycles)) != SHY_OK) return rc;
  return check_device_error(w);
}

int shy_erode(shy_world* w, int drops, int cycles) {
  int rc = check_world(w);
  if (rc) return rc;
  if (drops < 0 || cycles < 0 || drops > (1 << 30)) {
    set_error("invalid drops %d or cycles %d", drops, cycles);
    return SHY_ERR_INVALID_ARG;
  }
  if (w->terrains.size() != 1) {
    set_error("shy_erode takes a single-terrain world; use shy_batch_erode");
    return SHY_ERR_STATE;
  }
  if (w->terrains[0].drops != drops) {
    w->terrains[0].drops = drops;
    if ((rc = upload_terrains(w)) != SHY_OK) return rc;
  }
  return shy_batch_erode(w, cycles);
}

int shy_terrain_erode_exact(shy_world* w, int t, const int32_t* spawn_xy, int n) {
  int rc = check_terrain(w, t);
  if (rc) return rc;
  if (n < 0 || (n > 0 && !spawn_xy)) {
    set_error("invalid spawn list");
    return SHY_ERR_INVALID_ARG;
  }
  const Terrain& T = w->terrains[t];
  for (int i = 0; i < n; ++i)
    if (spawn_xy[2 * i] < 0 || spawn_xy[2 * i] >= T.nx || spawn_xy[2 * i + 1] < 0 ||
        spawn_xy[2 * i + 1] >= T.ny) {
      set_error("spawn %d at (%d, %d) is outside the %d x %d map", i, spawn_xy[2 * i], spawn_xy[2 * i + 1],
                T.nx, T.ny);
      return SHY_ERR_INVALID_ARG;
    }
  if ((rc = ensure_spawn_capacity(w, n)) != SHY_OK) return rc;
  if (n > 0)
    SHY_CHECK_CUDA(cudaMemcpyAsync(w->dspawn, spawn_xy, sizeof(int2) * n, cudaMemcpyHostToDevice, w->stream),
                   "upload spawns");
  return exact_erode_device_spawns(w, t, n);
}

}  // extern "C"

namespace shy {

int ensure_spawn_capacity(shy_world* w, int n) {
  if (n <= w->dspawn_cap) return SHY_OK;
  if (w->dspawn) cudaFree(w->dspawn);
  w->dspawn = nullptr;
  w->dspawn_cap = 0;
  SHY_CHECK_CUDA(dalloc(&w->dspawn, (size_t)n), "allocate spawn list");
  w->dspawn_cap = n;
  return SHY_OK;
}

int exact_erode_device_spawns(shy_world* w, int t, int n) {
  int rc;
  if ((rc = ensure_ceq(w, w->erf_source)) != SHY_OK) return rc;
  const Terrain& T = w->terrains[t];
  const long long b = T.cell_base, N = w->cells, cn = (long long)T.nx * T.ny;
  for (int k = 0; k < 3; ++k)  // source/world.h:56-61
    SHY_CHECK_CUDA(cudaMemsetAsync(w->track_f + k * N + b, 0, sizeof(float) * cn, w->stream), "zero tracks");
  w->hq_stale = true;
  SHY_CHECK_CUDA(launch_exact_erode(w, t, n), "exact erode");
  SHY_CHECK_CUDA(launch_exact_blend(w, t), "exact blend");
  w->ceq_source = ERF_DEVICE;  // the blend rebuilt ceqfac with the device erf
  SHY_CHECK_CUDA(cudaStreamSynchronize(w->stream), "synchronize");
  return SHY_OK;
}

}  // namespace shy

extern "C" {

int shy_erode_exact(shy_world* w, const int32_t* spawn_xy, int n) {
  return shy_terrain_erode_exact(w, 0, spawn_xy, n);
}

int shy_drop_descend(shy_world* w, shy_drop* drop, int* more) {
  int rc = check_world(w);
  if (rc) return rc;
  if (!drop || !more) {
    set_error("null drop or result");
    return SHY_ERR_INVALID_ARG;
  }
  if (!finite_pos(drop->pos[0], drop->pos[1]) || !isfinite(drop->speed[0]) || !isfinite(drop->speed[1]) ||
      !isfinite(drop->volume) || !isfinite(drop->sediment)) {
    set_error("drop state must be finite, |pos| < 2^24");
    return SHY_ERR_INVALID_ARG;
  }
  if ((rc = ensure_ceq(w, w->erf_source)) != SHY_OK) return rc;
  SHY_CHECK_CUDA(cudaMemcpyAsync(w->ddrop, drop, sizeof(shy_drop), cudaMemcpyHostToDevice, w->stream), "upload drop");
  w->hq_stale = true;
  SHY_CHECK_CUDA(launch_drop_descend(w, 0), "descend");
  SHY_CHECK_CUDA(cudaMemcpyAsync(drop, w->ddrop, sizeof(shy_drop), cudaMemcpyDeviceToHost, w->stream), "download drop");
  int m = 0;
  SHY_CHECK_CUDA(cudaMemcpyAsync(&m, w->dint, sizeof(int), cudaMemcpyDeviceToHost, w->stream), "download result");
  SHY_CHECK_CUDA(cudaStreamSynchronize(w->stream), "synchronize");
  *more = m;
  return SHY_OK;
}

int shy_drop_run(shy_world* w, float x, float y, float* trace, int max_records, int* n_records) {
  int rc = check_world(w);
  if (rc) return rc;
  if (max_records < 0 || (max_records > 0 && !trace)) {
    set_error("invalid trace buffer");
    return SHY_ERR_INVALID_ARG;
  }
  if (!finite_pos(x, y)) {
    set_error("drop position must be finite, |pos| < 2^24");
    return SHY_ERR_INVALID_ARG;
  }
  if ((rc = ensure_ceq(w, w->erf_source)) != SHY_OK) return rc;
  if (max_records > w->dtrace_cap) {
    if (w->dtrace) cudaFree(w->dtrace);
    w->dtrace = nullptr;
    w->dtrace_cap = 0;
    SHY_CHECK_CUDA(dalloc(&w->dtrace, (size_t)max_records * 8), "allocate trace");
    w->dtrace_cap = max_records;
  }
  w->hq_stale = true;
  SHY_CHECK_CUDA(launch_drop_run(w, 0, x, y, max_records), "drop run");
  int n = 0;
  SHY_CHECK_CUDA(cudaMemcpyAsync(&n, w->dint, sizeof(int), cudaMemcpyDeviceToHost, w->stream), "download count");
  SHY_CHECK_CUDA(cudaStreamSynchronize(w->stream), "synchronize");
  const int keep = n < max_records ? n : max_records;
  if (keep > 0)
    SHY_CHECK_CUDA(cudaMemcpy(trace, w->dtrace, sizeof(float) * 8 * keep, cudaMemcpyDeviceToHost), "download trace");
  if (n_records) *n_records = n;
  return SHY_OK;
}

int shy_cascade(shy_world* w, float x, float y) {
  int rc = check_world(w);
  if (rc) return rc;
  if (!finite_pos(x, y)) {
    set_error("cascade position must be finite, |pos| < 2^24");
    return SHY_ERR_INVALID_ARG;
  }
  w->hq_stale = true;
  SHY_CHECK_CUDA(launch_cascade(w, 0, x, y), "cascade");
  SHY_CHECK_CUDA(cudaStreamSynchronize(w->stream), "synchronize");
  return SHY_OK;
}

int shy_terrain_generate(shy_world* w, int t, uint64_t seed, int octaves) {
  int rc = check_terrain(w, t);
  if (rc) return rc;
  if (octaves < 1 || octaves > 24) {
    set_error("octaves %d out of range [1, 24]", octaves);
    return SHY_ERR_INVALID_ARG;
  }
  const long long n = (long long)w->terrains[t].nx * w->terrains[t].ny;
  double* raw = nullptr;
  unsigned long long* mm = nullptr;
  SHY_CHECK_CUDA(cudaMallocAsync((void**)&raw, sizeof(double) * n, w->stream), "allocate noise buffer");
  cudaError_t e = cudaMallocAsync((void**)&mm, 2 * sizeof(unsigned long long), w->stream);
  w->hq_stale = true;
  if (e == cudaSuccess) e = launch_value_noise(w, t, seed, octaves, raw, mm);
  cudaFreeAsync(raw, w->stream);
  if (mm) cudaFreeAsync(mm, w->stream);
  if (e != cudaSuccess) return cuda_fail(e, "generate terrain");
  SHY_CHECK_CUDA(cudaStreamSynchronize(w->stream), "synchronize");
  return SHY_OK;
}

int shy_terrain_init(shy_world* w, int t, int32_t seed) {
  int rc = check_terrain(w, t);
  if (rc) return rc;
  unsigned* mm = nullptr;
  SHY_CHECK_CUDA(cudaMallocAsync((void**)&mm, 2 * sizeof(unsigned), w->stream), "allocate terrain scratch");
  w->hq_stale = true;
  cudaError_t e = launch_reference_terrain(w, t, seed, mm);
  cudaFreeAsync(mm, w->stream);
  if (e != cudaSuccess) return cuda_fail(e, "initialise terrain");
  SHY_CHECK_CUDA(cudaStreamSynchronize(w->stream), "synchronize");
  return SHY_OK;
}

int shy_vegetation_step(shy_world* w, int steps) {
  int rc = check_world(w);
  if (rc) return rc;
  if (steps < 0) {
    set_error("negative step count");
    return SHY_ERR_INVALID_ARG;
  }
  if (!w->plant_next) {
    SHY_CHECK_CUDA(dalloc(&w->plant_next, (size_t)w->cells), "allocate vegetation buffers");
    SHY_CHECK_CUDA(dalloc(&w->rootq, (size_t)w->cells), "allocate vegetation buffers");
    SHY_CHECK_CUDA(dalloc(&w->veg_claim, (size_t)w->cells), "allocate vegetation buffers");
    SHY_CHECK_CUDA(cudaMemsetAsync(w->rootq, 0, sizeof(long long) * w->cells, w->stream), "clear");
    SHY_CHECK_CUDA(cudaMemsetAsync(w->veg_claim, 0xFF, sizeof(unsigned) * w->cells, w->stream), "clear");
  }
  for (int k = 0; k < steps; ++k) {
    SHY_CHECK_CUDA(launch_vegetation_step(w), "vegetation step");
    w->veg_step += 1;
  }
  SHY_CHECK_CUDA(cudaStreamSynchronize(w->stream), "synchronize");
  return SHY_OK;
}

int shy_world_set_vegetation_step(shy_world* w, uint64_t step) {
  int rc = check_world(w);
  if (rc) return rc;
  w->veg_step = step;
  return SHY_OK;
}

int shy_normals(shy_world* w, float* host_xyz, size_t count) {
  int rc = check_world(w);
  if (rc) return rc;
  const long long n = (long long)w->terrains[0].nx * w->terrains[0].ny;
  if (!host_xyz || count != (size_t)(3 * n)) {
    set_error("normals: want %lld floats", 3 * n);
    return SHY_ERR_INVALID_ARG;
  }
  if (!w->normals) SHY_CHECK_CUDA(dalloc(&w->normals, 3 * (size_t)w->cells), "allocate normals");
  SHY_CHECK_CUDA(launch_normals(w, 0, w->normals), "normals");
  SHY_CHECK_CUDA(cudaMemcpyAsync(host_xyz, w->normals, sizeof(float) * 3 * n, cudaMemcpyDeviceToHost, w->stream),
                 "download normals");
  SHY_CHECK_CUDA(cudaStreamSynchronize(w->stream), "synchronize");
  return SHY_OK;
}

}  // extern "C"
