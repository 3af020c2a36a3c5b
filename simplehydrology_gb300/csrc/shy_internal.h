// shy_internal.h -- engine internals shared by the .cu translation units.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <string>
#include <vector>

#include "../../include/shy.h"

struct shy_crand;  // the C-library generator state (shy_math.h)

namespace shy {

// One terrain of a world, as the kernels see it.  A world holds one or more
// terrains packed back to back in every per-cell array; cell (x, y) of
// terrain t is element cell_base + x * ny + y (x-major like the reference's
// math::flatten, source/include/math.h:11-14).
// Buckets of cells the batched mode's re-deal sorts live drops into, at
// most (a launch uses about four per run of drops, in multiples of
// kResortBucketStep); and its default steps between re-deals.
const int kResortBuckets = 65536;
const int kResortBucketStep = 4096;
const int kResortSteps = 16;

struct Terrain {
  long long cell_base;
  long long arr_base;  // first word of this terrain's arrivals bitmap
  int nx, ny;
  int drop_base;   // first drop slot of this terrain in a batched cycle
  int drops;       // drops per batched cycle
  unsigned long long seed;
};

// Per-cell 32.32 fixed-point accumulators of the batched mode.
// Track sums over a cycle: one 32-byte sector per cell, so a drop-step's
// three track atomics share one L2 sector.
struct alignas(32) Tracks {
  long long td;   // discharge track (source/water.h:115)
  long long tmx;  // momentum-x track (:116)
  long long tmy;  // momentum-y track (:117)
  long long pad;
};
// Batched-mode state of a cell: one 32-byte sector, so that a drop's reads
// and writes of its cell's height, pending changes and count share it.
struct alignas(32) CellQ {
  long long hq;   // height, 32.32 fixed point
  long long e;    // erosion / deposition of the current step (phase A sums)
  float effd;     // max(0, depositionRate * (1 - rootdensity)), a copy of the map
  int spare;
  int cnt[2];     // drops at the cell at the start of a step, by step parity
};

// Arrivals bitmap of the batched mode: one bit per cell, set while a
// cascade is claimed at the cell in the current step.  Cells are grouped in
// 8 x 8 tiles, one 64-bit word each (bit (x % 8) * 8 + y % 8), so that the
// 5 x 5 block around any cell lies in at most 2 x 2 words.
__host__ __device__ inline long long arr_words(int nx, int ny) {
  return (long long)((nx + 7) >> 3) * ((ny + 7) >> 3);
}

// Device-side counters (see shy_stats).
struct DevStats {
  unsigned long long cycles, drops, skipped, oob, steps;
  long long gain_q, loss_q;  // batched mode, 32.32 fixed point
  double gain_exact, loss_exact;  // exact (sequential) mode
};

// A cascade of the current step that will move height.  Phase scan queues
// its centre, the nine heights it starts from, and the arrivals-bitmap words
// around it from which its overlap counts are taken (aw[2 * i + j]: tile
// column tx0 + i, tile row ty0 + j).  Its transfers are then worked out in
// place: the 32.32 change of each neighbour (by neighbour index) and of the
// centre replace those inputs until settle adds them.
struct alignas(16) SteepCell {
  long long c2;
  int ti;
  float h0;
  union {
    struct {
      float v[8];
      unsigned long long aw[4];
      int tx0, ty0, ix, iy;
    } in;
    struct {
      long long dq[8];  // neighbour changes
      long long dc;     // centre change
    } out;
  } u;
};

// Grid barrier state of the persistent lock-step kernel.
struct GridBar {
  unsigned long long arrive;  // arrivals * 2^32 + drops still descending (the lock-step kernel's barrier)
  int abort;                  // set when a bounded wait gives up
  int error;                  // first error code seen on the device
  unsigned long long live;    // unused (the live count rides on `arrive`)
  unsigned long long tick;    // unused
  unsigned long long cycle;   // batched cycle index (spawn RNG)
  // CTA 0's view of the lock-step phases: descend, wait, scan, wait,
  // settle, wait
  unsigned long long phase_ns[6];
  unsigned long long iterations;  // lock-step steps run
};

enum ErfSource { ERF_DEVICE = 0, ERF_HOST_LIBM = 1 };

// Per-kernel CUDA-event timing: events are recorded around each launch on the
// world's stream and only read back (and summed) when the caller asks.
struct Timing {
  bool on = false;
  double ms[SHY_KERNEL_KINDS] = {0, 0, 0, 0};
  unsigned long long launches[SHY_KERNEL_KINDS] = {0, 0, 0, 0};
  struct Pair { cudaEvent_t a, b; int kind; };
  std::vector<Pair> pending;
  std::vector<cudaEvent_t> spare;
};

}  // namespace shy

struct shy_world {
  int device = 0;
  cudaStream_t stream = nullptr;
  shy_params P;
  std::vector<shy::Terrain> terrains;  // host copy
  long long cells = 0;                 // all terrains
  int max_drops = 0;                   // drop slots allocated
  int sm_count = 0;
  long long l2_bytes = 0;

  // reference-visible per-cell fields
  float* h = nullptr;         // height (in batched mode: hq rounded to float)
  float* root = nullptr;      // rootdensity
  float* plant = nullptr;     // per-cell plant size (vegetation)
  float* plant_next = nullptr;  // second plant buffer of a vegetation step
  long long* rootq = nullptr;   // root-density sums of a vegetation step, 32.32
  unsigned* veg_claim = nullptr;  // per-cell new-plant claims (step tags)
  unsigned long long veg_step = 0;
  float* track_f = nullptr;   // 3 x cells: float tracks (d, mx, my)
  // engine-internal per-cell state
  float4* rec = nullptr;      // {momentumx, momentumy, discharge, 1 + entrainment*erf(0.4 d)}
  float* effd = nullptr;      // max(0, depositionRate * (1 - rootdensity))
  shy::Tracks* trk = nullptr; // batched track sums
  shy::CellQ* cq = nullptr;   // batched-mode cell state (fixed-point heights)
  long long* hq_relax = nullptr;  // second fixed-point buffer of the relax stencil
  float* voltab = nullptr;    // drop volume after k evaporations
  int voltab_len = 0;
  bool hq_stale = true;       // h changed outside the batched mode (cq.hq stale)
  float* scratch = nullptr;   // cells floats, gather/scatter staging
  float* relax = nullptr;     // cells floats, second height buffer of the relax stencil

  // drop slots (struct of arrays)
  float2* dpos = nullptr;
  float2* dspd = nullptr;
  float* dsed = nullptr;      // sediment (a drop's volume is the volume table's entry for its age)
  int* dage = nullptr;        // -1: not descending
  long long* down = nullptr;  // the drop's own height change this step, 32.32
  int* dterr = nullptr;       // terrain of the slot
  int* dcell = nullptr;       // cell of this step's exchange within its terrain, -1 if none
  int* dctr = nullptr;        // cascade centre this slot runs this step, within its terrain, -1 if none
  shy::SteepCell* dsteep = nullptr;  // steep-cascade queue (one entry per drop slot at most)
  unsigned long long* arr = nullptr;  // arrivals bitmaps (two step parities), all terrains
  long long arr_words = 0;            // words of one parity's bitmap
  int* dorder = nullptr;      // drop run by each slot in a batched cycle (spawn-cell order)
  int* dkey = nullptr;        // spawn-order scratch: run of each drop's spawn cell
  int* drank = nullptr;       //   and its place within the run
  int* dhist = nullptr;       //   runs' counts, then offsets (at most 65,536)
  // second set of the slots' persistent fields (the re-deal moves the live
  // drops between the two sets), and its bucket counts (kResortBuckets)
  float2* dpos2 = nullptr;
  float2* dspd2 = nullptr;
  float* dsed2 = nullptr;
  int* dage2 = nullptr;
  int* dterr2 = nullptr;
  int* dresort = nullptr;
  float* stage = nullptr;             // cells floats, third staging buffer of the state calls
  float* feed = nullptr;              // staging buffer of shy_feed for host output
  size_t feed_len = 0;
  // the reference's frame loop: C-library random stream and plant agents
  shy_crand* crand = nullptr;         // device generator state (seeded lazily with 1)
  int rand_order = 1;                 // evaluation order of two rand() arguments (1: g++'s)
  float3* plants = nullptr;           // (x, y, size) per plant, list order
  int plant_cap = 0;
  int plant_count = 0;

  shy::Terrain* dterrains = nullptr;
  shy::DevStats* stats = nullptr;
  shy::GridBar* bar = nullptr;
  shy_drop* ddrop = nullptr;  // single-drop state for shy_drop_descend
  float* dtrace = nullptr;    // trace buffer for shy_drop_run
  int dtrace_cap = 0;
  int* dint = nullptr;        // small scratch (returned flags, counts)
  int2* dspawn = nullptr;     // exact-mode spawn list
  int dspawn_cap = 0;

  int erf_source = shy::ERF_DEVICE;
  int ceq_source = -1;        // erf source of the current ceqfac values (-1 stale)
  int track_mode = 0;         // 0: track_f holds the last call's tracks
  int batch_grid = 0;         // CTAs of the lock-step kernel at most (0: all resident)
  int batch_order = -1;       // slots in spawn-cell order: -1 when the cell state outgrows L2, 0 never, 1 always
  int batch_block = 256;      // threads per CTA of the lock-step kernel: 64, 128 or 256
  int batch_smem = 1;         // 0: drop slots in global memory even where shared memory would hold them
  int batch_resort = -1;      // steps between re-deals of the live drops (-1: kResortSteps with
                              // spawn-ordered slots in global memory, else never; 0 never)
  int batch_settle = -1;      // with re-deals: 1 the first drop in a cell settles it, 0 every drop
                              // its own change, -1 the first when the slots outgrow L2
  int graph_cycles = 0;       // batched cycles per CUDA graph (0: launched one by one)
  cudaGraphExec_t gexec = nullptr;  // the captured cycles
  unsigned long long graph_key = 0; // what they were captured with (launch_key)

  shy::Timing timing;
  float* normals = nullptr;   // 3 x cells, lazily allocated
};

namespace shy {

// Device buffers of one batched cycle, for launching it on memory the
// caller laid out (the no-allocation entry point).
struct CycleBuffers {
  const Terrain* terrains;
  int n_terrains;
  int total_drops;
  long long cells;
  float* h;
  CellQ* cq;
  float4* rec;
  const float* voltab;
  Tracks* trk;
  float* track_f;
  float2 *pos, *spd;
  float* sed;
  int* age;
  long long* own;
  int* terr;
  int* cell;
  int* ctr;
  SteepCell* steep;
  unsigned long long* arr;  // two bitmaps of arr_words words
  long long arr_words;
  DevStats* st;
  GridBar* bar;
  shy_params P;
  int sm_count;
};

// ---- launchers (defined in the .cu files) --------------------------------
cudaError_t launch_cycle_buffers(const CycleBuffers& b, cudaStream_t stream);
cudaError_t launch_rebuild_records(shy_world* w, int kind_for_timing);
int world_create(int n, const int* nx, const int* ny, const int* drops, const uint64_t* seeds,
                 const shy_params* params, shy_world** out);
void world_free(shy_world* w);
int world_check(shy_world* w);
// exact-mode World::erode of terrain t with the n spawns already in w->dspawn
int ensure_spawn_capacity(shy_world* w, int n);
int exact_erode_device_spawns(shy_world* w, int t, int n);
cudaError_t launch_exact_erode(shy_world* w, int terrain, int n);
cudaError_t launch_exact_blend(shy_world* w, int terrain);
cudaError_t launch_drop_descend(shy_world* w, int terrain);
cudaError_t launch_drop_run(shy_world* w, int terrain, float x, float y, int max_records);
cudaError_t launch_cascade(shy_world* w, int terrain, float x, float y);
cudaError_t launch_normals(shy_world* w, int terrain, float* out3);
cudaError_t launch_batched_cycle(shy_world* w);
cudaError_t launch_heights_to_fixed(shy_world* w);
// clears what a batched cycle that gave up left behind (pending sums, drop
// counts, barrier state)
cudaError_t launch_batched_recover(shy_world* w);
// the bounded-wait test hook (shy_debug_stall_waits): 0, or how long the
// first bounded wait of each kernel waits for an event that never comes
unsigned long long debug_stall_ns();
cudaError_t launch_vegetation_step(shy_world* w);
// the reference's init terrain (source/cellpool.h:349-409) into terrain t's
// heights; `minmax` is two device words of scratch
cudaError_t launch_reference_terrain(shy_world* w, int terrain, int32_t seed, unsigned* minmax);
cudaError_t launch_value_noise(shy_world* w, int terrain, unsigned long long seed, int octaves,
                               double* raw, unsigned long long* minmax);
cudaError_t launch_gather_comp(shy_world* w, int terrain, int comp, float* out);
cudaError_t launch_scatter_comp(shy_world* w, int terrain, int comp, const float* in);
// discharge / momentum (device arrays, null: keep) into terrain t's records,
// erf records included; and back out
cudaError_t launch_pack_state(shy_world* w, int t, const float* d, const float* mx, const float* my);
cudaError_t launch_unpack_state(shy_world* w, int t, float* d, float* mx, float* my);
// the same over every terrain's cells at once (arrays of w->cells floats)
cudaError_t launch_pack_state_all(shy_world* w, const float* d, const float* mx, const float* my);
cudaError_t launch_unpack_state_all(shy_world* w, float* d, float* mx, float* my);
// timing: open a launch interval of `kind` (returns the pair index or -1)
cudaError_t timing_begin(shy_world* w, int kind, int* slot);
cudaError_t timing_end(shy_world* w, int slot);

// the parameter checks every entry point that takes a shy_params applies
bool params_valid(const shy_params* p);

void set_error(const char* fmt, ...);
int cuda_fail(cudaError_t e, const char* what);

// return the C ABI's error status when a CUDA call fails
#define SHY_CHECK_CUDA(expr, what)                         \
  do {                                                     \
    cudaError_t e_ = (expr);                               \
    if (e_ != cudaSuccess) return shy::cuda_fail(e_, what); \
  } while (0)

}  // namespace shy
