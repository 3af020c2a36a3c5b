/* shy.h -- C ABI of simplehydrology_gb300, the GB300 (sm_103a) erosion engine.
 *
 * The reference (weigert/SimpleHydrology) is header-only C++ with process-wide
 * statics and no FFI.  Its erosion entry points are
 *   World::erode(int cycles)          source/world.h:33, body :54-88
 *   World::cascade(vec2 pos)          source/world.h:34, body :90-168
 *   Drop::Drop(vec2) / Drop::descend  source/water.h:14,37, body :58-156
 *   quad::map accessors               source/cellpool.h:413-447
 *   Vegetation::grow()                source/vegetation.h:49, body :122-188
 * This header replaces them with plain C entry points over an opaque world
 * handle.  A world owns one terrain on one GPU, its device maps and one CUDA
 * stream; calls on one world are not reentrant (the reference's
 * World::cascade uses a function-static array and is not reentrant either).
 * Every call returns SHY_OK or a negative status and never throws; the
 * message of the last failure on the calling thread is in shy_last_error().
 *
 * Maps are x-major like the reference (math::flatten, source/include/math.h:
 * 11-14): cell (x, y) of an nx-by-ny map is element x * ny + y.
 */
#ifndef SHY_H
#define SHY_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define SHY_ABI_VERSION 1

typedef struct shy_world shy_world;

/* status codes */
#define SHY_OK 0
#define SHY_ERR_INVALID_ARG (-1)
#define SHY_ERR_OUT_OF_MEMORY (-2)
#define SHY_ERR_CUDA (-3)
#define SHY_ERR_NO_DEVICE (-4)
#define SHY_ERR_TIMEOUT (-5)   /* a bounded device-side wait gave up */
#define SHY_ERR_STATE (-6)     /* call not valid in the world's current state */
#define SHY_ERR_IO (-7)        /* a checkpoint file could not be read or written */

/* Per-cell fields, in the order of quad::cell (source/cellpool.h:207-220). */
#define SHY_FIELD_HEIGHT 0
#define SHY_FIELD_DISCHARGE 1
#define SHY_FIELD_MOMENTUM_X 2
#define SHY_FIELD_MOMENTUM_Y 3
#define SHY_FIELD_DISCHARGE_TRACK 4
#define SHY_FIELD_MOMENTUM_X_TRACK 5
#define SHY_FIELD_MOMENTUM_Y_TRACK 6
#define SHY_FIELD_ROOT_DENSITY 7
#define SHY_FIELD_PLANT_SIZE 8  /* per-cell vegetation (no reference field) */
#define SHY_FIELD_COUNT 9

/* Model parameters.  Defaults (shy_params_default) are the reference's
 * static parameter values. */
typedef struct shy_params {
  /* struct Drop, source/water.h:43-50 */
  float evap_rate;          /* Drop::evapRate          0.001 */
  float deposition_rate;    /* Drop::depositionRate    0.1   */
  float min_vol;            /* Drop::minVol            0.01  */
  float max_age;            /* Drop::maxAge            500   */
  float entrainment;        /* Drop::entrainment       10    */
  float gravity;            /* Drop::gravity           1     */
  float momentum_transfer;  /* Drop::momentumTransfer  1     */
  /* class World, source/world.h:42-44 */
  float lrate;              /* World::lrate            0.1   */
  float max_diff;           /* World::maxdiff          0.01  */
  float settling;           /* World::settling         0.8   */
  /* namespace quad, source/cellpool.h:165 */
  float map_scale;          /* quad::mapscale          80    */
  /* struct Plant, source/vegetation.h:38-42 */
  float plant_max_size;       /* Plant::maxSize        1.5  */
  float plant_grow_rate;      /* Plant::growRate       0.05 */
  float plant_max_steep;      /* Plant::maxSteep       0.8  */
  float plant_max_discharge;  /* Plant::maxDischarge   0.3  */
  float plant_max_height;     /* Plant::maxTreeHeight  0.8  */
  /* per-cell vegetation rates: a plant dies with 1/1000 chance per step and
   * spreads with 1/20 chance (source/vegetation.h:71,160); new plants appear
   * with plant_spawn_prob per cell per step */
  float plant_spawn_prob;     /* 1e-4  */
  float plant_death_prob;     /* 0.001 */
  float plant_spread_prob;    /* 0.05  */
  /* Batched mode, optional extra slope relaxation at the end of each cycle:
   * cascade_passes passes of World::cascade's transfer rule as a symmetric
   * stencil over neighbour pairs next to visited cells, each pass moving
   * cascade_weight * settling * excess / 2 (no reference counterpart; the
   * reference's own per-step cascade always runs). */
  float cascade_weight;       /* 0.125 */
  int cascade_passes;         /* 0     */
  int reserved[7];
} shy_params;

/* Droplet state, struct Drop source/water.h:20-27. */
typedef struct shy_drop {
  int age;
  float pos[2];
  float speed[2];
  float volume;
  float sediment;
} shy_drop;

/* Counters accumulated on the device since creation or shy_world_reset_stats. */
typedef struct shy_stats {
  uint64_t cycles;         /* batched cycles run (shy_erode) */
  uint64_t drops;          /* drops that started descending */
  uint64_t drops_skipped;  /* spawns on cells below height 0.1 (world.h:71) */
  uint64_t drops_oob;      /* drops that left the map, sediment lost (water.h:139-142) */
  uint64_t drop_steps;     /* descend() calls that passed the termination checks */
  double evap_gain;        /* sediment created by evaporation (water.h:135), sum */
  double boundary_loss;    /* sediment carried off the map, sum */
} shy_stats;

/* Optional per-kernel timing (CUDA events on the world's stream). */
#define SHY_KERNEL_DROPS 0    /* batched descend kernel */
#define SHY_KERNEL_APPLY 1    /* height apply + lrate blend + record rebuild */
#define SHY_KERNEL_CASCADE 2  /* cascade stencil */
#define SHY_KERNEL_OTHER 3    /* everything else launched by the world */
#define SHY_KERNEL_KINDS 4
typedef struct shy_timing {
  double ms[SHY_KERNEL_KINDS];
  uint64_t launches[SHY_KERNEL_KINDS];
  uint64_t steps_timed;    /* drop steps done by the timed drop launches */
} shy_timing;

/* ---- library ---------------------------------------------------------- */
int shy_version(void);
const char* shy_last_error(void);
int shy_params_default(shy_params* out);

/* ---- world lifecycle (replaces World::map, source/world.h:22,40, and the
 *      cell pool, SimpleHydrology.cpp:11,36) --------------------------------- */
int shy_world_create(int nx, int ny, const shy_params* params, uint64_t seed,
                     shy_world** out);
int shy_world_destroy(shy_world* w);
int shy_world_set_params(shy_world* w, const shy_params* params);
int shy_world_get_params(shy_world* w, shy_params* out);
int shy_world_size(shy_world* w, int* nx, int* ny);
/* Host <-> device copies of one field (count = nx * ny floats). */
int shy_world_set_field(shy_world* w, int field, const float* host, size_t count);
int shy_world_get_field(shy_world* w, int field, float* host, size_t count);
int shy_world_sync(shy_world* w);
/* Height, discharge and momentum of terrain t -- the state a front end
 * exchanges every frame -- in one call each way, with one host
 * synchronisation (count = nx * ny each; a NULL pointer leaves that field
 * unchanged / unread).  Same effect as the matching set/get_field calls. */
int shy_terrain_set_state(shy_world* w, int terrain, const float* height, const float* discharge,
                          const float* momentum_x, const float* momentum_y, size_t count);
int shy_terrain_get_state(shy_world* w, int terrain, float* height, float* discharge, float* momentum_x,
                          float* momentum_y, size_t count);
/* The same for every terrain of the world at once (no reference
 * counterpart: the reference has one terrain): each non-NULL array holds all
 * cells, terrain after terrain in creation order, each terrain x-major
 * (count = the sum of nx * ny over the terrains).  One copy per field and one
 * host synchronisation, however many terrains. */
int shy_world_set_state(shy_world* w, const float* height, const float* discharge, const float* momentum_x,
                        const float* momentum_y, size_t count);
int shy_world_get_state(shy_world* w, float* height, float* discharge, float* momentum_x, float* momentum_y,
                        size_t count);
/* The same state calls on DEVICE memory (no reference counterpart: the
 * reference has no device): each non-NULL pointer is nx * ny floats of device
 * (or managed) memory of the world's device.  The copies run on the world's
 * stream; the data must be ready when the call is made (work that writes it
 * on another stream must have finished), and the call returns after the
 * world's stream finished the copies.  Used by the surrogate's warm start,
 * whose predictions never leave the device. */
int shy_terrain_set_state_device(shy_world* w, int terrain, const float* height, const float* discharge,
                                 const float* momentum_x, const float* momentum_y, size_t count);
int shy_terrain_get_state_device(shy_world* w, int terrain, float* height, float* discharge,
                                 float* momentum_x, float* momentum_y, size_t count);
/* The world's cudaStream_t, for callers that order their own work with it. */
int shy_world_stream(shy_world* w, void** stream);
int shy_world_stats(shy_world* w, shy_stats* out);
int shy_world_reset_stats(shy_world* w);
/* Batched-mode random stream position: the next shy_erode cycle uses this
 * cycle index for its spawn positions. */
int shy_world_set_cycle(shy_world* w, uint64_t cycle);
int shy_world_get_cycle(shy_world* w, uint64_t* cycle);
int shy_world_enable_timing(shy_world* w, int on);
int shy_world_timing(shy_world* w, shy_timing* out);
/* Where the batched kernel's time goes, as seen by its first CTA, summed
 * over all cycles since creation: phase_ms[6] = {descend phase, barrier
 * wait, cascade scan phase, barrier wait, settle phase (steep cascades,
 * height updates, retirements), barrier wait plus spawn, re-deals (see
 * shy_world_set_resort) and exit};
 * *iterations = lock-step steps run. */
int shy_world_lockstep_profile(shy_world* w, double* phase_ms, uint64_t* iterations);
/* Launch shape of the batched kernel: at most `grid` CTAs (0, the default:
 * every CTA that fits on the GPU at once, at least 32 drops each).  A CTA
 * keeps its drops in shared memory while they fit and in global memory
 * beyond that.  `order` puts the drops of a cycle into slots sorted by spawn
 * cell, so that each CTA works on a compact stretch of the maps: -1 (the
 * default) when the cell state is larger than L2, 0 never, 1 always.
 * Results do not depend on either setting. */
int shy_world_set_launch(shy_world* w, int grid, int order);
/* CTA size of the batched kernel: `threads` 64, 128 or 256 (the default)
 * threads per CTA, so that at full residency each CTA owns about that many
 * drops or fewer (the SM count times the resident CTAs of that size set the
 * grid); `smem_slots` 1 (default) keeps a CTA's drop slots in shared memory
 * where they fit without lowering occupancy, 0 always in global memory.
 * Results do not depend on either setting. */
int shy_world_set_block(shy_world* w, int threads, int smem_slots);
/* Re-deal of a batched cycle's drops: every `steps` lock-step steps, the
 * drops still descending are sorted by the cell they are in and dealt to
 * the CTAs in runs again, so that drops touching the same cells run
 * together while the drops drift from their spawn cells, and retired drops
 * leave the CTAs' slot ranges.  Only with drop slots in global memory.
 * -1 (the default): every 16 steps when the slots are in spawn-cell order
 * (see shy_world_set_launch), else never; 0 never; 1-4096 that many steps.
 * Results do not depend on it. */
int shy_world_set_resort(shy_world* w, int steps);
/* How a re-dealt batched cycle settles each step's height changes: 0 every
 * drop adds its own change to its cell; 1 the drop that registered first in
 * a cell adds the cell's whole pending sum (its slot then keeps no change of
 * its own: fewer bytes per step, one more wait in settle, which pays only
 * where the slots' loads miss L2 anyway); -1 (the default) 1 when the drop
 * slots outgrow L2, else 0.  Only with re-deals (shy_world_set_resort).
 * Results do not depend on it. */
int shy_world_set_settle(shy_world* w, int mode);
/* Batched cycles per CUDA graph: with k > 0, shy_erode / shy_batch_erode run
 * each k cycles as one graph (the lock-step and end-of-cycle launches of k
 * cycles), captured on the world's stream on first use and again whenever
 * the parameters, drops, launch shape or buffers change; leftover cycles and
 * calls with per-kernel timing on launch one by one.  0 (the default): no
 * graphs.  Results do not depend on it. */
int shy_world_set_graph(shy_world* w, int cycles_per_graph);

/* Test hook for the library's bounded device waits (no counterpart in the
 * reference, which has no device code).  While `ns` is non-zero, the first
 * bounded wait of every batched-erosion launch (its first grid barrier) and
 * of every surrogate TMA convolution (conv_tma path) waits for an event that
 * never happens, gives up after `ns` nanoseconds and takes the kernel's
 * give-up path: the batched call returns SHY_ERR_TIMEOUT (its world stays
 * usable: the failed cycle's pending sums and counts are cleared, its
 * heights are what the cycle had reached), the convolution's error shows in
 * shy_sg_status().  Nothing faults or hangs.  0 (the default) turns the hook
 * off; at most 1e10 ns.  Process-wide. */
int shy_debug_stall_waits(uint64_t ns);

/* Source of erf(0.4 * discharge) (source/cellpool.h:242-244) for the exact
 * mode.  SHY_ERF_DEVICE (default) is the library's own erf, evaluated on the
 * GPU and correctly rounded to float.  SHY_ERF_HOST_LIBM evaluates the host C
 * library's erff once per cell whenever the discharge map changed -- what a
 * reference build on the same host calls, so that the exact mode reproduces
 * that build bit for bit.  The batched mode always uses SHY_ERF_DEVICE. */
#define SHY_ERF_DEVICE 0
#define SHY_ERF_HOST_LIBM 1
int shy_world_set_erf_source(shy_world* w, int source);

/* ---- erosion ------------------------------------------------------------ */

/* Batched erosion: `cycles` times World::erode(drops) (source/world.h:54-88)
 * with all `drops` of a cycle descending at once, one GPU thread slot each,
 * in lock step.  In step t every live drop takes one Drop::descend step
 * against the heights left by step t-1; World::cascade then runs once at
 * every cell a drop moved to; then all height changes apply.  Drops sharing a
 * cell share its sediment exchange (each uses depositionRate / n, so a cell
 * gets one drop's worth of exchange per step; n = 1 is the reference).
 * Height changes and the three track maps are summed in 32.32 fixed point
 * with integer atomics, so the result is the same bits for any thread
 * schedule.  Discharge and momentum stay fixed during a cycle, as in the
 * reference, and take the lrate blend (world.h:81-86) at its end.  Spawn
 * positions come from a counter-based generator keyed by (seed, cycle, drop
 * index); spawns on cells below height 0.1 are skipped (world.h:71). */
int shy_erode(shy_world* w, int drops, int cycles);

/* Exact erosion: one World::erode(n) call (source/world.h:54-88) with the
 * reference's sequential semantics -- every drop sees all earlier edits and
 * World::cascade runs after every step -- with the n spawn positions given
 * (spawn_xy[2i], spawn_xy[2i+1]), in place of the reference's rand() draws.
 * Runs on one GPU thread; meant for parity and small maps. */
int shy_erode_exact(shy_world* w, const int32_t* spawn_xy, int n);

/* One Drop::descend() call (source/water.h:58-156) on the world, live, with
 * the drop state held by the caller.  *more receives descend()'s result. */
int shy_drop_descend(shy_world* w, shy_drop* drop, int* more);

/* Drop d(pos); while (d.descend()); (source/world.h:74-76), recording the
 * state after every descend() call as 8 floats: returned, age, pos.x, pos.y,
 * speed.x, speed.y, volume, sediment.  *n_records receives the number of
 * descend() calls (records beyond max_records are not written). */
int shy_drop_run(shy_world* w, float x, float y, float* trace, int max_records,
                 int* n_records);

/* World::cascade(pos), source/world.h:90-168, on the live heights. */
int shy_cascade(shy_world* w, float x, float y);

/* Vegetation::grow() (source/vegetation.h:122-188), `steps` times, per cell
 * and for every terrain of the world: each cell holds at most one plant
 * (SHY_FIELD_PLANT_SIZE > 0), which grows, dies on discharge, height or a
 * plant_death_prob draw, and spreads with plant_spread_prob to a cell up to 4
 * away; empty cells where Plant::spawn allows gain a plant with
 * plant_spawn_prob.  Plants add and remove root density with the reference's
 * 3 x 3 weights 1, 0.6, 0.4, which lowers the deposition rate of the batched
 * and exact erosion (source/water.h:86-87).  Draws come from a counter keyed
 * by the terrain seed, the step index and the cell; the result is
 * deterministic.  Equivalent to the reference's plant list in distribution,
 * not plant by plant. */
int shy_vegetation_step(shy_world* w, int steps);
/* Index of the next vegetation step (its random draws). */
int shy_world_set_vegetation_step(shy_world* w, uint64_t step);

/* quad::map::normal (source/cellpool.h:182-204) of every cell, 3 floats per
 * cell, x-major. */
int shy_normals(shy_world* w, float* host_xyz, size_t count);

/* ---- batches of terrains ---------------------------------------------------
 * A world created by shy_batch_create holds n independent terrains of their
 * own sizes, seeds and drops per cycle, packed into one set of device maps;
 * shy_batch_erode runs every terrain's cycle in the same lock-step launch.
 * The single-terrain calls above act on terrain 0. */
int shy_batch_create(int n_terrains, const int* nx, const int* ny, const int* drops_per_cycle,
                     const uint64_t* seeds, const shy_params* params, shy_world** out);
int shy_batch_erode(shy_world* w, int cycles);
int shy_batch_size(shy_world* w, int* n_terrains);
int shy_terrain_size(shy_world* w, int terrain, int* nx, int* ny, int* drops_per_cycle);
int shy_terrain_set_field(shy_world* w, int terrain, int field, const float* host, size_t count);
int shy_terrain_get_field(shy_world* w, int terrain, int field, float* host, size_t count);
int shy_terrain_erode_exact(shy_world* w, int terrain, const int32_t* spawn_xy, int n);

/* Terrain input: fill a terrain's heights with seeded fractal value noise
 * (`octaves` octaves, lacunarity 2, gain 0.5, base frequency 4 per longer
 * side) min-max normalised to [0, 1], generated on the device.  Replaces the
 * reference's FastNoiseLite initialisation (source/cellpool.h:323-411) with
 * the workloads' recipe; the normalisation is the reference's (:382-409). */
int shy_terrain_generate(shy_world* w, int terrain, uint64_t seed, int octaves);

/* Terrain input: the reference's own map initialisation, quad::map::init
 * (source/cellpool.h:323-411).  Eight layers of FastNoiseLite OpenSimplex2
 * FBm noise at frequencies 2^o and weights 0.6^(o+1), sampled at
 * (x / nx, y / ny, seed % 10000) with the library's default settings, then
 * min-max normalised with the minimum and maximum starting at 0.  Generated
 * on the device with the reference's float operations in its order: the
 * heights are the reference's bit for bit (pinned against the reference's
 * own init at 512 x 512).  `seed` is the reference's int SEED. */
int shy_terrain_init(shy_world* w, int terrain, int32_t seed);

/* ---- batched erosion without allocation ------------------------------------
 * No counterpart in the reference (which has no GPU path); the library adds
 * it for callers that cannot allocate device memory themselves or through
 * the library: a frame loop or plugin running under a host application
 * that owns all device memory (its own caching allocator has reserved the
 * GPU, so cudaMalloc fails or is forbidden), or code that must not stall or
 * fragment the allocator at run time.  Such callers hold the maps in memory
 * they already own and pass device pointers.
 *
 * Runs `cycles` batched cycles (the same lock-step cycles as shy_erode, keyed
 * by seed and by cycle index cycle0, cycle0 + 1, ...) on one nx-by-ny terrain
 * whose maps the caller holds in DEVICE memory (nx * ny floats each,
 * x-major): height, discharge and momentum are read and updated in place,
 * root_density is read.  Each call starts from the float maps (heights are
 * rounded into the batched mode's 32.32 fixed point on entry), so a call
 * equals a fresh world created from the same maps.  `stream` is a
 * cudaStream_t (NULL for the legacy default stream); the call returns after
 * the stream finished the work.  `stats` (host, may be NULL) receives the
 * call's counters.
 *
 * It allocates nothing: no cudaMalloc or cudaFree and no allocating library
 * routine.  Its working memory is one fixed device array of about 9 MiB
 * inside the library, sized for at most SHY_NOALLOC_MAX_CELLS cells,
 * SHY_NOALLOC_MAX_DROPS drops per cycle and max_age SHY_NOALLOC_MAX_AGE
 * (larger requests fail with SHY_ERR_INVALID_ARG), and cascade_passes must be
 * 0.  Every GPU that loads the library holds that array until the process
 * exits.  All calls on a device share it: calls that overlap on the GPU (from
 * other threads or other streams) race and corrupt each other's results, so
 * serialise them.  The call copies its status to the host and synchronizes
 * `stream` before it returns, so it must not be issued on a stream that is
 * being captured into a CUDA graph.  The first call on each device also looks
 * up the array's device address (cudaGetSymbolAddress); while another stream
 * of the process is being captured, make sure that first call has already
 * happened.  Each map must be device (or managed) memory of the current
 * device; anything else fails with SHY_ERR_INVALID_ARG before any launch. */
#define SHY_NOALLOC_MAX_CELLS (256 * 256)
#define SHY_NOALLOC_MAX_DROPS 16384
#define SHY_NOALLOC_MAX_AGE 4096
int shy_erode_noalloc(int nx, int ny, const shy_params* params, uint64_t seed, uint64_t cycle0,
                      int drops, int cycles, float* height, float* discharge, float* momentum_x,
                      float* momentum_y, const float* root_density, void* stream, shy_stats* stats);

/* ---- The reference's frame loop in its own random sequence ----------------
 * The reference draws World::erode's spawn positions (source/world.h:69) and
 * Vegetation::grow's plant events (source/vegetation.h:122-188) from one
 * C-library rand() stream.  A world carries that generator (the GNU C
 * library's default rand(), restated) on the device:
 *   shy_world_srand(w, s)        srand(s) for the world's stream (a stream
 *                                never seeded behaves as srand(1))
 *   shy_erode_rand(w, drops)     World::erode(drops) of terrain 0 in the exact
 *                                (sequential) mode, spawns drawn from the stream
 *   shy_vegetation_grow(w)       Vegetation::grow() on the world's plant list
 *   shy_plants(w, out, max, &n)  the plant list, (x, y, size) per plant in
 *                                list order (at most max copied, n = its size)
 * so that srand(s) followed by frames of World::erode(n); Vegetation::grow();
 * is reproduced with the reference's maps and plant list.
 * shy_world_set_rand_order selects which of the two rand() arguments of one
 * vector constructor is drawn first: 1 (default) the second one, as g++
 * evaluates them; 0 the first one.  These are parity paths run by one device
 * thread, like shy_erode_exact. */
int shy_world_srand(shy_world* w, uint32_t seed);
int shy_world_set_rand_order(shy_world* w, int order);
int shy_erode_rand(shy_world* w, int drops);
int shy_vegetation_grow(shy_world* w);
int shy_plants(shy_world* w, float* out, int max_plants, int* count);

/* ---- Checkpoint and resume (no reference counterpart: the reference keeps
 *      its state in process memory only) ---------------------------------
 * shy_world_save writes a world's state between calls -- terrains,
 * parameters, maps, fixed-point heights, cycle and vegetation-step counters,
 * counters, the C-library random stream and the plant list -- to `path`
 * (through a temporary file renamed into place).
 * shy_world_load creates a new world on the current device from such a file;
 * it continues bit for bit as the saved world would have.  The format is
 * versioned and ends in a hash of its contents; a damaged or foreign file
 * fails with SHY_ERR_IO. */
int shy_world_save(shy_world* w, const char* path);
int shy_world_load(const char* path, shy_world** out);

/* ---- Front-end data feed ---------------------------------------------------
 * What the reference's front end rebuilds from the maps after every erosion
 * frame and uploads to OpenGL (SimpleHydrology.cpp:322-355; updatenode,
 * source/cellpool.h:286-317), written into a plain buffer instead, one record
 * per cell of terrain `terrain`, cells x-major (x * ny + y):
 *   SHY_FEED_DISCHARGE_RGBA  4 floats: waterColor (92, 133, 142) / 255
 *                            (source/model.h:22) and erf(0.4 discharge)
 *   SHY_FEED_MOMENTUM_RGBA   4 floats: 0.5 (1 + erf(mx)), 0.5 (1 + erf(my)),
 *                            0.5, 1
 *   SHY_FEED_VERTICES        12 floats: position (x, mapscale h, y), normal
 *                            (quad::_normal), tangent T - P and bitangent
 *                            B - P toward the points at x + 1 and y + 1
 *                            (heights 0 outside the map)
 * count must be cells x floats per record.  out_is_device = 1: `out` is a
 * 16-byte aligned device pointer, written on the world's stream (order with
 * shy_world_stream or shy_world_sync); 0: `out` is host memory, filled before
 * the call returns.  erf is the library's correctly rounded erf. */
#define SHY_FEED_DISCHARGE_RGBA 0
#define SHY_FEED_MOMENTUM_RGBA 1
#define SHY_FEED_VERTICES 2
int shy_feed(shy_world* w, int terrain, int kind, float* out, size_t count, int out_is_device);

/* ---- Measurement ----------------------------------------------------------
 * L2 peaks of one device, measured by the library's own microbenchmarks (no
 * counterpart in the reference, which has no GPU path).  They are the
 * roofline of the batched kernel when a terrain's cell state fits in L2.
 * Allocates about 40 MiB of device memory for the duration of the call and
 * takes well under a second. */
typedef struct shy_l2_probe {
  uint64_t l2_bytes;                  /* L2 capacity (cudaDevAttrL2CacheSize) */
  uint64_t buffer_bytes;              /* probe buffer, a quarter of L2 at most */
  double read_gbs;                    /* streaming 16-byte loads that bypass L1 */
  double random_sector_reads_per_s;   /* 8-byte loads, one per random 32-byte sector */
  double red_per_s;                   /* 64-bit atomic adds without return, random addresses */
} shy_l2_probe;
int shy_measure_l2(int device, shy_l2_probe* out);

/* Self-check of the kernels' fast arithmetic on the current device, against
 * the library's reference restatements (integer or FP64):
 *  [0] the batched kernel's float -> 32.32 conversion on the hardware
 *      converter against llrintf(v * 2^32), over every float |v| < 2^31;
 *  [1] its 32.32 -> float conversion against (float)((double)q * 2^-32),
 *      over all |q| < 2^26, powers of two and their neighbours, and 2^31
 *      values spread over the int64 range;
 *  [2] the device kernels' float-float erf against the FP64 evaluation it
 *      reproduces, over every float;
 *  [3] the float evaporation roundings (float)((double)s / (1 - evap)) and
 *      (float)((double)v * (1 - evap)) against the integer restatement and
 *      the double expression, over every positive float, for the default
 *      evaporation rate and the rates 0.0005, 0.01 and 0.1;
 *  [4] the float edge height (float)((double)h - 0.002) against the double
 *      expression, over every float.
 * Each count of differing inputs is 0 on a conforming device.  Takes about
 * two seconds. */
int shy_check_conversions(uint64_t mismatches[5]);

#ifdef __cplusplus
}
#endif

#endif /* SHY_H */
