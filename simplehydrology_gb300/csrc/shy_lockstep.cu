// shy_lockstep.cu -- the batched erosion mode.
//
// One batched cycle is World::erode(drops) (source/world.h:54-88) with all
// drops of every terrain of the world descending at once, in lock step.  Each
// CTA owns a contiguous range of drop slots and keeps their state (and its
// queue of steep cascades) in shared memory when it fits, in the world's
// global drop arrays otherwise.  Step t is three phases separated by
// grid-wide barriers:
//   descend  each live drop takes one Drop::descend step
//      (source/water.h:58-156) against the heights after step t-1.  A drop
//      sharing its cell with n-1 other live drops exchanges sediment at rate
//      effD / n (n = 1 is the reference).  The height change goes to the
//      cell's pending erosion sum and the three tracks to its track record,
//      as 32.32 fixed-point integer atomics.  Each drop registers at its new
//      cell (the count of the next step); the first to arrive runs that
//      cell's cascade.
//   scan  World::cascade (source/world.h:90-168) at every claimed cell reads
//      the nine heights phase descend left (fixed point plus pending sum).
//      Cascades that move nothing end here.  The steep ones are queued in the
//      CTA with the heights they read and the words of an arrivals bitmap
//      (8 x 8 cells per word, loaded with the heights) that hold the claimed
//      centres of the 5 x 5 block around theirs.  While thread 0 waits at
//      the grid barrier, the CTA's other warps work out each queued
//      cascade's transfers from what scan read: its overlap counts from those
//      words (where the 3 x 3 blocks of k cascades overlap, a pair's transfer
//      is divided by k, the larger count of its two cells, so overlapping
//      cascades together move what one would), then the reference's
//      sequential transfer loop on one thread.
//   settle  the queued transfers go straight to the fixed-point heights (no
//      height is read in this phase).  Every drop adds its own height change
//      to its cell's fixed-point height and clears the cell's pending sum and
//      count (or, when the slots outgrow L2, only the drop that registered
//      first in the cell adds the cell's whole pending sum: see kLean);
//      finished drops retire.  The arrivals bitmap of the other step parity
//      is cleared for the next step.
// With the cell state larger than L2, each cycle's drops are sorted by spawn
// cell and dealt to the CTAs in runs of consecutive drops, round-robin: each
// run is a compact stretch of the maps, and every CTA samples stretches from
// the whole map, so live drops stay balanced across CTAs as drops retire.
// Drops drift from their spawn cells within tens of steps, so every `resort`
// steps (slots in global memory only) the live drops are sorted again, by
// the cell they are in, and dealt to the CTAs in runs once more: the drops
// that touch the same cells stay in the same runs, which run at about the
// same time, and the retired drops drop out of the slot ranges.  A drop's
// slot carries its whole state, so this changes no result.
// Heights live in 32.32 fixed point for the whole cycle (the float map is
// rewritten at its end), so every update is an integer addition.
// Integer sums make every result independent of thread timing: the same
// inputs give the same bits on every run, and oracle/hydro_oracle.cpp
// (Lockstep) restates the schedule on the CPU.
// Each phase is a latency chain, so the kernel keeps its arithmetic short:
// fixed point <-> float on the hardware converters (shy_unq_dev,
// shy_q32_dev) and the reference's FP64 roundings in float-float
// (shy_evap_div_ff, shy_minus_0002), each with the bits of the library's
// restatement (checked on the device by shy_check_conversions).
//
// The end-of-cycle kernel converts the tracks to float, applies the lrate
// blend (source/world.h:81-86) and rebuilds the per-cell records.
#include <mutex>

#include "shy_device.cuh"

namespace shy {

namespace {

// CTA sizes of the lock-step kernel (threads, one drop slot each while a
// CTA's slots fit in one pass); 256 unless the world asks otherwise
const int kLockBlock = 256;
const int kSmemTerrains = 128;
// With kLean (slots in global memory, larger than L2), a slot's age field
// carries, besides the age (below 2^30: max_age < 1e6), this flag: the drop
// was the first to register at the cell it is in.  In settle that drop alone
// adds the cell's pending sum (every drop's change there, the same integer
// sum) to its height and clears the cell's sum and count, so no slot needs
// to keep its own change (8 B written and 8 B read per drop-step fewer).
// The pending sum's load is a round trip in settle, which only pays where
// the slots' own loads already miss L2.
const int kFirstAtCell = 1 << 30;
// shared-memory bytes per drop slot: its state plus one steep-queue entry
const int kSlotBytes = 2 * 8 + 8 + 5 * 4 + (int)sizeof(SteepCell);
// A grid barrier gives up (and flags SHY_ERR_TIMEOUT) after this long.
const unsigned long long kBarrierLimitNs = 2000000000ull;

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ unsigned long long ld_acquire_u64(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.acquire.gpu.global.u64 %0, [%1];" : "=l"(v) : "l"(p) : "memory");
  return v;
}
__device__ __forceinline__ void red_release_add_u64(unsigned long long* p, unsigned long long v) {
  asm volatile("red.release.gpu.global.add.u64 [%0], %1;" ::"l"(p), "l"(v) : "memory");
}
__device__ __forceinline__ int ld_relaxed_i32(const int* p) {
  int v;
  asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

__device__ __forceinline__ void add_i64(long long* p, long long v) {
  atomicAdd((unsigned long long*)p, (unsigned long long)v);
}

// A cell's whole 32-byte record in one load: fixed-point height, deposition
// rate and the two step-parity drop counts.
struct CellView {
  long long hq;
  long long e;  // the pending erosion sum (not needed by descend)
  float effd;
  int cnt0, cnt1;  // drop counts by step parity
};
__device__ __forceinline__ CellView load_cell(const CellQ* p) {
  unsigned long long w0, w1, w2, w3;
  asm volatile("ld.global.v4.u64 {%0, %1, %2, %3}, [%4];"
               : "=l"(w0), "=l"(w1), "=l"(w2), "=l"(w3)
               : "l"(p));
  CellView v;
  v.hq = (long long)w0;
  v.e = (long long)w1;
  v.effd = __uint_as_float((unsigned)(w2 & 0xffffffffull));
  v.cnt0 = (int)(unsigned)(w3 & 0xffffffffull);
  v.cnt1 = (int)(unsigned)(w3 >> 32);
  return v;
}

// an arrivals word, loaded where it stands in the program (not moved into
// the branch that uses it)
__device__ __forceinline__ unsigned long long load_arr(const unsigned long long* p) {
  unsigned long long v;
  asm volatile("ld.global.u64 %0, [%1];" : "=l"(v) : "l"(p));
  return v;
}

// word and bit of cell (x, y) in a terrain's arrivals bitmap
__device__ __forceinline__ long long arr_word(const Terrain& T, int x, int y) {
  return T.arr_base + (long long)(x >> 3) * ((T.ny + 7) >> 3) + (y >> 3);
}
__device__ __forceinline__ unsigned long long arr_bit(int x, int y) {
  return 1ull << (((x & 7) << 3) | (y & 7));
}

// Grid-wide barrier over a monotonically increasing arrival counter (reset to
// zero between launches).  `passed` counts the barriers this CTA has passed.
// The counter also carries the grid's live-drop count: each arrival adds
// 2^32 plus the CTA's change to that count (`delta`, from thread 0), so after
// n arrivals the counter is n * 2^32 + live, with 0 <= live < 2^32 once all
// of a barrier's arrivals are in (every change is added by then).  The wait
// ends when the counter reaches target * 2^32 -- exact, since before the last
// arrival the partial sum is below that -- and the low 32 bits of the value
// read then are the live count, left in `*live` for the whole CTA: arrivals
// at the next barrier (possible before this CTA reads) add 2^32 with no
// change, because the count changes only at spawn and at the end of a step.
// Every wait is bounded: past limit_ns the waiter sets bar->abort and every
// later barrier returns false at once, so the kernel always ends.  Warps 1
// and up run `work` while thread 0 waits: work that neither reads what other
// CTAs write before the barrier nor writes what they read.  `extra` arrivals
// beyond the grid's are awaited: the bounded-wait test hook
// (shy_debug_stall_waits) asks for one arrival that never comes, so the wait
// runs out.
// `retired`, if given, is a shared counter of drops the CTA's warps retired
// since the last barrier: thread 0 subtracts it from the live count (on top
// of `delta`) once every warp has arrived, and clears it.
template <class Work>
__device__ bool grid_barrier(GridBar* bar, unsigned& passed, unsigned long long* live, Work&& work,
                             unsigned extra = 0, unsigned long long limit_ns = kBarrierLimitNs,
                             long long delta = 0, unsigned* retired = nullptr) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x >= 32) work();
  if (threadIdx.x == 0) {
    if (retired) {
      delta -= (long long)*retired;
      *retired = 0;
    }
    const unsigned long long target = ((unsigned long long)(passed + 1) * gridDim.x + extra) << 32;
    red_release_add_u64(&bar->arrive, (1ull << 32) + (unsigned long long)delta);
    int ok = 1;
    unsigned long long t0 = 0;
    unsigned spins = 0;
    unsigned long long v;
    while ((v = ld_acquire_u64(&bar->arrive)) < target) {
      if (++spins < 64) continue;
      if (t0 == 0) t0 = global_ns();
      if (ld_relaxed_i32(&bar->abort)) {
        ok = 0;
        break;
      }
      if (global_ns() - t0 > limit_ns) {
        atomicExch(&bar->abort, 1);
        atomicCAS(&bar->error, 0, SHY_ERR_TIMEOUT);
        ok = 0;
        break;
      }
      __nanosleep(64);
    }
    if (live) *live = (v - target) & 0xffffffffull;
    s_ok = ok;
  }
  __syncthreads();
  ++passed;
  return s_ok != 0;
}

__device__ __forceinline__ bool grid_barrier(GridBar* bar, unsigned& passed, unsigned long long* live) {
  return grid_barrier(bar, passed, live, [] {});
}

// Drops sorted by spawn cell go to the CTAs in runs of this many, dealt
// round-robin: at least about eight runs per CTA, at most 256 drops per run.
__host__ __device__ __forceinline__ long long order_run(long long total, long long grid) {
  const long long r = total / (8 * grid);
  return r < 1 ? 1 : (r > 256 ? 256 : r);
}

// The drop slots of CTA b of `grid`: first slot `lo`, `nd` of them, storage
// for `cap` (the most any CTA of the launch has).  Unordered, the slots are
// consecutive drops.  Ordered, run k of the CTA's is run k * grid + b of the
// sorted drops, the runs being `run` drops long (the last one may be short).
struct SlotRange {
  long long lo;
  int nd, cap;
};
__host__ __device__ __forceinline__ SlotRange slot_range(long long total, long long grid, long long b, bool ordered) {
  SlotRange r;
  if (!ordered) {
    r.lo = b * total / grid;
    r.nd = (int)((b + 1) * total / grid - r.lo);
    r.cap = (int)((total + grid - 1) / grid);
    return r;
  }
  const long long R = order_run(total, grid);
  const long long runs = (total + R - 1) / R, q = runs / grid, m = runs % grid;
  const long long short_by = total % R ? R - total % R : 0;  // the last run's shortfall
  const long long last_owner = (runs - 1) % grid;
  r.nd = (int)((q + (b < m ? 1 : 0)) * R - (last_owner == b ? short_by : 0));
  r.lo = R * (b * q + (b < m ? b : m)) - (last_owner < b ? short_by : 0);
  r.cap = (int)((q + (m ? 1 : 0)) * R);
  return r;
}

struct LockArgs {
  const Terrain* terrains;
  int n_terrains;
  int total_drops;
  long long cells;
  const float* h;  // heights rounded to float at cycle start (spawn test)
  CellQ* cq;       // fixed-point heights, pending changes, drop counts
  const float4* rec;
  const float* voltab;  // volume after k evaporations (source/water.h:136)
  shy_evap ev;
  Tracks* trk;
  // global drop slots and steep queue (used when a CTA's range does not fit
  // in shared memory)
  float2* pos;
  float2* spd;
  float* sed;  // sediment (the volume is voltab[age])
  int* age;
  long long* own;   // the drop's own height change this step, 32.32
  int* terr;
  int* cell;
  int* ctr;
  SteepCell* steep;
  unsigned long long* arr;  // arrivals bitmaps, one per step parity, arr_words words each
  long long arr_words;
  const int* order;  // drops sorted by spawn cell (dealt to the CTAs in runs), or null: slot = drop
  // second set of the slots' persistent fields, for the re-deal (which
  // moves the live drops from one set to the other)
  float2* pos2;
  float2* spd2;
  float* sed2;
  int* age2;
  int* terr2;
  int* rhist;    // re-deal: live drops per bucket of cells, then offsets; zero between re-deals
  int rshift;    //   bucket = cell >> rshift
  int rbuckets;  //   buckets in use: a multiple of kResortBucketStep, at most kResortBuckets
  int resort;    //   steps between re-deals (0: never; only with slots in global memory)
  int lean;      // 1: the slots outgrow L2 (the kLean instantiation, with re-deals)
  int smem_slots;   // 1: drop slots and queue live in dynamic shared memory
  int smem_allowed;  // 0: keep the slots in global memory even when they would fit
  shy_params P;
  DevStats* st;
  GridBar* bar;
  int max_steps;
  unsigned long long stall_ns;  // test hook: the first barrier waits this long for a missing arrival
};

// The drop slots [lo, lo + n) of one CTA.
struct Slots {
  float2* pos;
  float2* spd;
  float* sed;  // sediment; a drop's volume is voltab[age] (it depends on nothing else)
  long long* own;
  int* cell;  // cell of this step's exchange within the slot's terrain, -1 if none
  int* ctr;   // cascade centre this slot runs this step, within its terrain, -1 if none
  int* age;         // >= 0 descending, -2 finished this step, -1 idle
  int* terr;
  SteepCell* steep;
};

// The slots from `lo` on in global memory, persistent fields from set `buf`
// (0: the first set, 1: the second).
__device__ __forceinline__ Slots slots_global(const LockArgs& a, int buf, long long lo) {
  Slots S;
  S.steep = a.steep + lo;
  S.pos = (buf ? a.pos2 : a.pos) + lo;
  S.spd = (buf ? a.spd2 : a.spd) + lo;
  S.sed = (buf ? a.sed2 : a.sed) + lo;
  S.own = a.own + lo;
  S.cell = a.cell + lo;
  S.ctr = a.ctr + lo;
  S.age = (buf ? a.age2 : a.age) + lo;
  S.terr = (buf ? a.terr2 : a.terr) + lo;
  return S;
}

__device__ __forceinline__ Slots slots_of(const LockArgs& a, unsigned char* smem, long long lo, int cap) {
  Slots S;
  if (a.smem_slots) {
    // 16-byte entries first, then 8-byte, then 4-byte arrays
    unsigned char* p = smem;
    S.steep = reinterpret_cast<SteepCell*>(p); p += sizeof(SteepCell) * cap;
    S.pos = reinterpret_cast<float2*>(p); p += 8 * cap;
    S.spd = reinterpret_cast<float2*>(p); p += 8 * cap;
    S.own = reinterpret_cast<long long*>(p); p += 8 * cap;
    S.cell = reinterpret_cast<int*>(p); p += 4 * cap;
    S.ctr = reinterpret_cast<int*>(p); p += 4 * cap;
    S.age = reinterpret_cast<int*>(p); p += 4 * cap;
    S.sed = reinterpret_cast<float*>(p); p += 4 * cap;
    S.terr = reinterpret_cast<int*>(p);
  } else {
    S = slots_global(a, 0, lo);
  }
  return S;
}

__device__ __forceinline__ int find_terrain(const Terrain* T, int n, int d) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (T[mid].drop_base <= d) lo = mid; else hi = mid - 1;
  }
  return lo;
}

template <int kBlock>
__device__ __forceinline__ unsigned long long block_sum_u64(unsigned long long v) {
  __shared__ unsigned long long red[kBlock / 32];
  for (int o = 16; o > 0; o >>= 1) v += __shfl_down_sync(0xffffffffu, v, o);
  __syncthreads();
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
  __syncthreads();
  unsigned long long s = 0;
  if (threadIdx.x == 0)
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += red[i];
  return s;  // valid in thread 0
}

// compare-exchange on (height, neighbour index) keys: a total order, so any
// sorting network yields exactly the stable sort by height that the
// reference's std::sort of <= 16 elements (an insertion sort) produces
__device__ __forceinline__ void cswap(float& ha, int& ka, float& hb, int& kb) {
  const bool sw = hb < ha || (hb == ha && kb < ka);
  const float th = sw ? hb : ha, uh = sw ? ha : hb;
  const int tk = sw ? kb : ka, uk = sw ? ka : kb;
  ha = th; ka = tk; hb = uh; kb = uk;
}

__device__ __forceinline__ void sort8(float* h, int* k) {
#define SHY_CS(i, j) cswap(h[i], k[i], h[j], k[j])
  SHY_CS(0, 2); SHY_CS(1, 3); SHY_CS(4, 6); SHY_CS(5, 7);
  SHY_CS(0, 4); SHY_CS(1, 5); SHY_CS(2, 6); SHY_CS(3, 7);
  SHY_CS(0, 1); SHY_CS(2, 3); SHY_CS(4, 5); SHY_CS(6, 7);
  SHY_CS(2, 4); SHY_CS(3, 5);
  SHY_CS(1, 4); SHY_CS(3, 6);
  SHY_CS(1, 2); SHY_CS(3, 4); SHY_CS(5, 6);
#undef SHY_CS
}

// quad::_normal (source/cellpool.h:182-204) from the five heights it reads;
// the diagonal in-bounds tests decide which triangles count.
__device__ __forceinline__ float3 normal5(float hp, float hxp, float hxm, float hyp, float hym, bool pp,
                                          bool mm, bool pm, bool mp, float ms) {
  float3 n = make_float3(0.0f, 0.0f, 0.0f);
  auto add = [&](float3 a, float3 b) {
    const float3 c = cross_scaled(a, b, ms);
    n = make_float3(n.x + c.x, n.y + c.y, n.z + c.z);
  };
  if (pp) add(make_float3(0.0f, hyp - hp, 1.0f), make_float3(1.0f, hxp - hp, 0.0f));
  if (mm) add(make_float3(0.0f, hym - hp, -1.0f), make_float3(-1.0f, hxm - hp, 0.0f));
  if (pm) add(make_float3(1.0f, hxp - hp, 0.0f), make_float3(0.0f, hym - hp, -1.0f));
  if (mp) add(make_float3(-1.0f, hxm - hp, 0.0f), make_float3(0.0f, hyp - hp, 1.0f));
  // length(n) > 0 (IEEE sqrt is +0 only at +0, so this is dd > 0, without
  // the square root on the critical path)
  const float dd = n.x * n.x + n.y * n.y + n.z * n.z;
  if (dd > 0.0f) {
    const float r = 1.0f / sqrtf(n.x * n.x + n.y * n.y + n.z * n.z);
    n = make_float3(n.x * r, n.y * r, n.z * r);
  }
  return n;
}

// the fixed-point height and this step's pending erosion of a cell, in one
// 16-byte load
__device__ __forceinline__ longlong2 hq_e(const CellQ* c) {
  return *reinterpret_cast<const longlong2*>(c);
}

// Overlap counts of a claimed cascade: the cascade centres of this step in the
// 5 x 5 block around (ix, iy) give, for the centre and each of its 8
// neighbours, how many cascades' 3 x 3 blocks hold that cell.  wij is the
// arrivals word of tile column tx0 + i, tile row ty0 + j (the block spans at
// most two of each).
__device__ __forceinline__ void overlap_counts(unsigned long long w00, unsigned long long w01,
                                               unsigned long long w10, unsigned long long w11, int tx0, int ty0,
                                               int ix, int iy, const Terrain& T, unsigned& kv, int& kc) {
  // row by row: row dx of the block is byte (x % 8) of the word(s) of its
  // tile column, the two tile rows side by side as 16 bits; cells outside
  // the map never have their bit set, rows outside it are skipped
  const bool two_rows = ((iy + 2 < T.ny ? iy + 2 : T.ny - 1) >> 3) != ty0;
  const int o = iy - 2 - 8 * ty0;  // bit of the 16 for dy = -2 (-2 .. 7)
  unsigned cen = 0;
#pragma unroll
  for (int r = 0; r < 5; ++r) {
    const int x = ix + r - 2;
    if (x < 0 || x >= T.nx) continue;
    const bool second = (x >> 3) != tx0;
    const int sh = (x & 7) * 8;
    unsigned row = (unsigned)(((second ? w10 : w00) >> sh) & 0xFFull);
    if (two_rows) row |= (unsigned)(((second ? w11 : w01) >> sh) & 0xFFull) << 8;
    const unsigned bits = (o >= 0 ? row >> o : row << (-o)) & 31u;
    cen |= bits << (5 * r);
  }
  // cascades whose 3 x 3 block holds cell (dx, dy): popcount of a window
  auto cover = [&](int dx, int dy) {
    const unsigned row = 7u << (dy + 1);  // 3 bits centred on dy
    const unsigned win = (row << (5 * (dx + 1))) | (row << (5 * (dx + 2))) | (row << (5 * (dx + 3)));
    return (unsigned)__popc(cen & win);
  };
  kv = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) kv |= cover(nb_dx(k), nb_dy(k)) << (4 * k);
  kc = (int)cover(0, 0);
}

// World::cascade's transfer loop (source/world.h:127-165) for one queued
// centre: the neighbours in the reference's stable height order, the live
// centre height, each transfer divided by the overlap count of its pair.
// Everything that does not depend on the live centre height is computed
// before the sequential loop.  The 32.32 changes replace the entry's inputs
// (all read first); `steep_apply` adds them to the heights.
__device__ __forceinline__ void steep_transfers(SteepCell& q, const Terrain& T, const shy_params& P) {
  unsigned kv;
  int kc;
  overlap_counts(q.u.in.aw[0], q.u.in.aw[1], q.u.in.aw[2], q.u.in.aw[3], q.u.in.tx0, q.u.in.ty0, q.u.in.ix,
                 q.u.in.iy, T, kv, kc);
  float v[8];
  int sk[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    v[k] = q.u.in.v[k];
    sk[k] = k;
  }
  sort8(v, sk);
  // per sorted neighbour: in the map, excess threshold, overlap divisor
  float thr[8];
  int kk[8];
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    const int k = sk[j];
    const float dist = (nb_dx(k) != 0 && nb_dy(k) != 0) ? sqrtf(2.0f) : 1.0f;
    // h > 0.1 in double is h >= 0.1f in float (no float lies between);
    // |diff| - 0 is |diff| exactly
    thr[j] = v[j] >= 0.1f ? dist * P.max_diff : 0.0f;
    const int kn = (int)((kv >> (4 * k)) & 15u);
    kk[j] = kc > kn ? kc : kn;
  }
  const float h0 = q.h0;
  float hcv = h0;
  float tr[8];
  bool moved = false;
#pragma unroll
  for (int j = 0; j < 8; ++j) {
    tr[j] = 0.0f;
    if (!(v[j] < __int_as_float(0x7f800000))) continue;  // outside the map
    const float diff = hcv - v[j];
    if (diff == 0.0f) continue;
    const float excess = fabsf(diff) - thr[j];
    if (excess <= 0.0f) continue;
    float transfer = P.settling * excess / 2.0f;
    if (kk[j] > 1) transfer = transfer / (float)kk[j];
    if (diff > 0.0f) {
      hcv -= transfer;
      tr[j] = transfer;
    } else {
      hcv += transfer;
      tr[j] = -transfer;
    }
    moved = true;
  }
#pragma unroll
  for (int k = 0; k < 8; ++k) q.u.out.dq[k] = 0;
#pragma unroll
  for (int j = 0; j < 8; ++j)
    if (tr[j] != 0.0f) q.u.out.dq[sk[j]] = shy_q32_dev(tr[j]);
  q.u.out.dc = moved ? shy_q32_dev(hcv - h0) : 0;
}

// The changes `steep_transfers` left in a queued entry, added to the
// fixed-point heights.
__device__ __forceinline__ void steep_apply(const SteepCell& q, const Terrain& T, CellQ* cq) {
  const long long c2 = q.c2;
#pragma unroll
  for (int k = 0; k < 8; ++k) {
    const long long d = q.u.out.dq[k];
    if (d != 0) add_i64(&cq[c2 + (long long)nb_dx(k) * T.ny + nb_dy(k)].hq, d);
  }
  if (q.u.out.dc != 0) add_i64(&cq[c2].hq, q.u.out.dc);
}

// Exclusive prefix sum of the n counts h[] in place (16-byte aligned; n a
// multiple of kResortBucketStep), by one CTA of kBlock threads: each thread
// sums a stretch of 4-int vectors (loaded four at a time, so that a stretch
// costs few round trips), the CTA scans the stretch sums, each thread
// writes its stretch's offsets.
template <int kBlock>
__device__ void cta_exclusive_scan(int* h, int n) {
  static_assert(kResortBucketStep % (16 * kBlock) == 0, "stretches of whole groups of four vectors");
  const int kVec = n / 4 / kBlock;  // vectors per thread, a multiple of 4
  __shared__ int s_w[kBlock / 32];
  int4* v = reinterpret_cast<int4*>(h) + threadIdx.x * kVec;
  int sum = 0;
  for (int g = 0; g < kVec; g += 4) {
    int4 q[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) q[u] = v[g + u];
#pragma unroll
    for (int u = 0; u < 4; ++u) sum += q[u].x + q[u].y + q[u].z + q[u].w;
  }
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  int x = sum;  // inclusive within the warp
  for (int o = 1; o < 32; o <<= 1) {
    const int y = __shfl_up_sync(0xffffffffu, x, o);
    if (lane >= o) x += y;
  }
  if (lane == 31) s_w[warp] = x;
  __syncthreads();
  if (warp == 0) {
    int w = lane < kBlock / 32 ? s_w[lane] : 0;
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, w, o);
      if (lane >= o) w += y;
    }
    if (lane < kBlock / 32) s_w[lane] = w;
  }
  __syncthreads();
  int run = x - sum + (warp ? s_w[warp - 1] : 0);
  for (int g = 0; g < kVec; g += 4) {
    int4 q[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) q[u] = v[g + u];
#pragma unroll
    for (int u = 0; u < 4; ++u) {
      int4 o;
      o.x = run; run += q[u].x;
      o.y = run; run += q[u].y;
      o.z = run; run += q[u].z;
      o.w = run; run += q[u].w;
      v[g + u] = o;
    }
  }
}

// The cell a live drop (inside its terrain) is in.
__device__ __forceinline__ long long drop_cell(const Terrain& T, float2 p) {
  return T.cell_base + (long long)(int)p.x * T.ny + (int)p.y;
}

// Re-deal between steps: the `live` drops still descending, sorted by the
// bucket of cells they are in, go to the CTAs in runs (run k of CTA b is run
// k * grid + b of the sorted drops, as at spawn), from one set of the slots'
// persistent fields to the other.  Three grid barriers: after the bucket
// counts, after CTA 0's prefix sum, after the moves.  Then each CTA clears
// its share of the counts and returns its new range, in the other set.  A
// drop's rank within its bucket is whatever the atomics give: no result
// depends on which slot a drop is in.  The CTA's slots pass as scalars
// (first slot `lo`, `nd` of them, set `buf`), so that the caller's slot
// pointers stay in registers rather than on the stack.
struct Redealt {
  long long lo;
  int nd;
  bool ok;
};
template <int kBlock>
__device__ __noinline__ Redealt redeal(const LockArgs& a, const Terrain* TT, long long lo, int nd, int buf,
                                       unsigned passed, long long live) {
  Redealt r;
  r.lo = lo;
  r.nd = nd;
  r.ok = false;
  const Slots S = slots_global(a, buf, lo);
  // each pass loads the next slot's fields before its own atomic, so that a
  // thread's slots cost overlapping round trips
  {
    int ag_n = -1, ti_n = 0;
    float2 p_n = make_float2(0.0f, 0.0f);
    if ((int)threadIdx.x < nd) {
      ag_n = S.age[threadIdx.x]; ti_n = S.terr[threadIdx.x]; p_n = S.pos[threadIdx.x];
    }
    for (int j = threadIdx.x; j < nd; j += kBlock) {
      const int ag = ag_n, ti = ti_n;
      const float2 p = p_n;
      if (j + kBlock < nd) {
        ag_n = S.age[j + kBlock]; ti_n = S.terr[j + kBlock]; p_n = S.pos[j + kBlock];
      }
      if (ag >= 0) atomicAdd(&a.rhist[drop_cell(TT[ti], p) >> a.rshift], 1);
    }
  }
  if (!grid_barrier(a.bar, passed, nullptr)) return r;
  if (blockIdx.x == 0) cta_exclusive_scan<kBlock>(a.rhist, a.rbuckets);
  if (!grid_barrier(a.bar, passed, nullptr)) return r;
  const long long R = order_run(live, gridDim.x);
  const Slots D = slots_global(a, buf ^ 1, 0);
  int ag_n = -1, ti_n = 0;
  float2 p_n = make_float2(0.0f, 0.0f), s_n = p_n;
  float e_n = 0.0f;
  if ((int)threadIdx.x < nd) {
    const int j = threadIdx.x;
    ag_n = S.age[j]; ti_n = S.terr[j]; p_n = S.pos[j]; s_n = S.spd[j]; e_n = S.sed[j];
  }
  for (int j = threadIdx.x; j < nd; j += kBlock) {
    const int ag = ag_n, ti = ti_n;
    const float2 p = p_n, sp = s_n;
    const float se = e_n;
    if (j + kBlock < nd) {
      const int jn = j + kBlock;
      ag_n = S.age[jn]; ti_n = S.terr[jn]; p_n = S.pos[jn]; s_n = S.spd[jn]; e_n = S.sed[jn];
    }
    if (ag < 0) continue;
    const long long k = atomicAdd(&a.rhist[drop_cell(TT[ti], p) >> a.rshift], 1);
    if (k >= live) {  // more drops than the live count: never expected
      atomicCAS(&a.bar->error, 0, SHY_ERR_STATE);
      continue;
    }
    const long long kr = k / R;
    const long long d = slot_range(live, gridDim.x, kr % gridDim.x, true).lo + (kr / gridDim.x) * R + k % R;
    D.pos[d] = p;
    D.spd[d] = sp;
    D.sed[d] = se;
    D.age[d] = ag;
    D.terr[d] = ti;
  }
  if (!grid_barrier(a.bar, passed, nullptr)) return r;
  const SlotRange sr = slot_range(live, gridDim.x, blockIdx.x, true);
  r.lo = sr.lo;
  r.nd = sr.nd;
  r.ok = true;
  const long long w0 = (long long)blockIdx.x * a.rbuckets / gridDim.x;
  const long long w1 = (long long)(blockIdx.x + 1) * a.rbuckets / gridDim.x;
  for (long long i = w0 + threadIdx.x; i < w1; i += kBlock) a.rhist[i] = 0;
  return r;
}

// 128 registers: two 256-thread CTAs per SM.  kRedeal: the instantiation
// with the re-deal (slots in global memory, a.resort > 0); the other has no
// trace of it, so that its slot pointers stay fixed for the whole cycle.
// kLean (with kRedeal only): first-registered drops settle whole cells.
template <int kBlock, bool kRedeal, bool kLean>
__global__ void __maxnreg__(128) lockstep_kernel(LockArgs a) {
  extern __shared__ __align__(16) unsigned char s_dyn[];
  __shared__ Terrain sT[kSmemTerrains];
  __shared__ int s_nq;                  // steep cascades queued this step
  __shared__ unsigned long long s_live;  // drops still descending
  __shared__ unsigned s_retired;        // drops this CTA retired in the current step
  const bool smem_t = a.n_terrains <= kSmemTerrains;
  if (smem_t)
    for (int i = threadIdx.x; i < a.n_terrains; i += blockDim.x) sT[i] = a.terrains[i];
  if (threadIdx.x == 0) {
    s_nq = 0;
    s_retired = 0;
  }
  __syncthreads();
  const Terrain* TT = smem_t ? sT : a.terrains;

  // this CTA's drop slots: [lo, lo + nd), storage for `cap`
  const SlotRange sr = slot_range(a.total_drops, gridDim.x, blockIdx.x, a.order != nullptr);
  long long lo = sr.lo;
  int nd = sr.nd;
  const int cap = sr.cap;
  Slots S = slots_of(a, s_dyn, lo, cap);
  const long long run = order_run(a.total_drops, gridDim.x);
  int buf = 0;  // which set of persistent slot fields the CTA's slots are in
  const bool redeals = kRedeal && a.resort > 0 && !a.smem_slots;
  const bool one_terrain = a.n_terrains == 1;  // every slot's terrain is 0: no need to load it

  const shy_params& P = a.P;
  const unsigned long long cycle = a.bar->cycle;
  // phase clock of CTA 0's thread 0, kept in shared memory so that the other
  // threads hold no registers for it
  __shared__ unsigned long long s_ph[7];  // 6 phases + the last stamp
  const bool timer = blockIdx.x == 0 && threadIdx.x == 0;
  if (timer) {
    for (int i = 0; i < 6; ++i) s_ph[i] = 0;
    s_ph[6] = global_ns();
  }
  auto lap = [&](int i) {
    if (timer) {
      const unsigned long long t = global_ns();
      s_ph[i] += t - s_ph[6];
      s_ph[6] = t;
    }
  };
  unsigned passed = 0;
  unsigned n_steps = 0, n_oob = 0, n_drops = 0, n_skipped = 0;  // this thread's, per cycle
  long long gain_q = 0, loss_q = 0;
  const shy_evap ev = a.ev;
  const int vmax = (int)P.max_age + 2;  // last entry of the volume table

  // both arrivals bitmaps start the cycle empty (this CTA's share of them)
  {
    const long long w0 = (long long)blockIdx.x * (2 * a.arr_words) / gridDim.x;
    const long long w1 = (long long)(blockIdx.x + 1) * (2 * a.arr_words) / gridDim.x;
    for (long long i = w0 + threadIdx.x; i < w1; i += blockDim.x) a.arr[i] = 0ull;
  }
  if (redeals) {  // and the re-deal's bucket counts
    const long long w0 = (long long)blockIdx.x * a.rbuckets / gridDim.x;
    const long long w1 = (long long)(blockIdx.x + 1) * a.rbuckets / gridDim.x;
    for (long long i = w0 + threadIdx.x; i < w1; i += blockDim.x) a.rhist[i] = 0;
  }

  // spawn (source/world.h:64-74)
  unsigned long long born = 0;
  for (int j = threadIdx.x; j < nd; j += blockDim.x) {
    const long long d = a.order ? a.order[((long long)(j / run) * gridDim.x + blockIdx.x) * run + j % run] : lo + j;
    const int t = find_terrain(TT, a.n_terrains, (int)d);
    const Terrain T = TT[t];
    int x, y;
    shy_spawn_xy(T.seed, cycle, (unsigned)(d - T.drop_base), T.nx, T.ny, &x, &y);
    const long long c = T.cell_base + (long long)x * T.ny + y;
    S.terr[j] = t;
    S.cell[j] = -1;
    S.ctr[j] = -1;
    // world.h:71; no float lies between 0.1 and 0.1f, so this is h < 0.1
    if (a.h[c] < 0.1f) {
      S.age[j] = -1;
      ++n_skipped;
      continue;
    }
    ++n_drops;
    ++born;
    S.pos[j] = make_float2((float)x, (float)y);
    S.spd[j] = make_float2(0.0f, 0.0f);
    S.sed[j] = 0.0f;
    if (kLean) {
      S.age[j] = atomicAdd(&a.cq[c].cnt[0], 1) == 0 ? kFirstAtCell : 0;
    } else {
      S.age[j] = 0;
      atomicAdd(&a.cq[c].cnt[0], 1);
    }
  }
  const unsigned long long born_all = block_sum_u64<kBlock>(born);  // valid in thread 0
  bool ok = grid_barrier(a.bar, passed, &s_live, [] {}, a.stall_ns ? 1u : 0u,
                         a.stall_ns ? a.stall_ns : kBarrierLimitNs, (long long)born_all);

  int step = 0;
  for (; ok && step < a.max_steps; ++step) {
    if (s_live == 0) break;
    const int par = step & 1;
    lap(5);

    // ---- descend: one Drop::descend step per live drop ----
    if (threadIdx.x == 0) s_nq = 0;  // everyone read it before the last barrier
    // Each iteration loads the next slot's state before working on its own,
    // so that with several slots per thread (slots in global memory) their
    // loads overlap the work instead of preceding it.
    // With re-deals (several slots per thread, in runs of cells), the three
    // phases sweep the slots in alternating directions, so that each phase
    // starts on the cells the one before ended on, while L2 still holds them:
    // descend forwards on even steps, scan backwards, settle forwards, and
    // the reverse on odd steps.  Slot order changes no result.
    const bool rev_d = redeals && (step & 1);
    int ag_n = 0, ti_n = 0;
    float2 p_n = make_float2(0.0f, 0.0f), s_n = p_n;
    float e_n = 0.0f;
    if ((int)threadIdx.x < nd) {
      const int j = rev_d ? nd - 1 - (int)threadIdx.x : (int)threadIdx.x;
      ag_n = S.age[j]; ti_n = one_terrain ? 0 : S.terr[j]; p_n = S.pos[j]; s_n = S.spd[j]; e_n = S.sed[j];
    }
    for (int i = threadIdx.x; i < nd; i += blockDim.x) {
      const int j = rev_d ? nd - 1 - i : i;
      const int agr = ag_n, ti = ti_n;
      float2 p = p_n, s = s_n;
      const float se = e_n;
      if (i + (int)blockDim.x < nd) {
        const int jn = rev_d ? nd - 1 - (i + (int)blockDim.x) : i + (int)blockDim.x;
        ag_n = S.age[jn]; ti_n = one_terrain ? 0 : S.terr[jn]; p_n = S.pos[jn]; s_n = S.spd[jn]; e_n = S.sed[jn];
      }
      if (agr < 0) continue;
      const int ag = kLean ? (agr & (kFirstAtCell - 1)) : agr;
      // {volume, sediment}: the volume after `ag` evaporations (water.h:136)
      float2 v = make_float2(__ldg(&a.voltab[ag < vmax ? ag : vmax]), se);
      const Terrain T = TT[ti];
      const CellQ* RT = a.cq + T.cell_base;
      const int ix = (int)p.x, iy = (int)p.y;
      const long long lc = (long long)ix * T.ny + iy;
      const long long c = T.cell_base + lc;
      // < 2^31 cells per terrain; with kLean only the cell's first drop settles it
      S.cell[j] = (!kLean || (agr & kFirstAtCell)) ? (int)lc : -1;
      // the five heights quad::_normal reads (0 outside the map)
      const bool xp = ix + 1 < T.nx, xm = ix > 0, yp = iy + 1 < T.ny, ym = iy > 0;
      // all loads issued together; a neighbour outside the map reads the
      // centre and is masked to height 0
      const CellView own = load_cell(RT + lc);
      const long long q0 = own.hq;
      const int nhere = par ? own.cnt1 : own.cnt0;
      long long qxp = RT[xp ? lc + T.ny : lc].hq;
      long long qxm = RT[xm ? lc - T.ny : lc].hq;
      long long qyp = RT[yp ? lc + 1 : lc].hq;
      long long qym = RT[ym ? lc - 1 : lc].hq;
      const float4 r = __ldg(&a.rec[c]);
      const float ed = own.effd;
      const float vnext = __ldg(&a.voltab[ag + 1 < vmax ? ag + 1 : vmax]);
      qxp = xp ? qxp : 0;
      qxm = xm ? qxm : 0;
      qyp = yp ? qyp : 0;
      qym = ym ? qym : 0;
      const float hp = shy_unq_dev(q0);
      const float3 n = normal5(hp, shy_unq_dev(qxp), shy_unq_dev(qxm), shy_unq_dev(qyp), shy_unq_dev(qym), xp && yp, xm && ym,
                               xp && ym, xm && yp, P.map_scale);
      if ((float)ag > P.max_age || v.x < P.min_vol) {  // water.h:74-83
        const long long dep = shy_q32_dev(v.y);
        add_i64(&a.cq[c].e, dep);
        if (!kLean) S.own[j] = dep;
        S.age[j] = -2;
        S.ctr[j] = -1;
        continue;
      }
      ++n_steps;
      s.x = s.x + (P.gravity * n.x) / v.x;  // water.h:95
      s.y = s.y + (P.gravity * n.z) / v.x;
      // length(v) > 0 is dot(v, v) > 0: IEEE sqrt is +0 only at +0
      if (dot2(r.x, r.y, r.x, r.y) > 0.0f && dot2(s.x, s.y, s.x, s.y) > 0.0f) {  // water.h:97-99
        const float rf = 1.0f / sqrtf(dot2(r.x, r.y, r.x, r.y));
        const float rs = 1.0f / sqrtf(dot2(s.x, s.y, s.x, s.y));
        const float k = (P.momentum_transfer * dot2(r.x * rf, r.y * rf, s.x * rs, s.y * rs)) / (v.x + r.z);
        s.x = s.x + k * r.x;
        s.y = s.y + k * r.y;
      }
      if (dot2(s.x, s.y, s.x, s.y) > 0.0f) {  // water.h:108-109
        const float root2 = sqrtf(2.0f);
        const float rs = 1.0f / sqrtf(dot2(s.x, s.y, s.x, s.y));
        const float ux = s.x * rs, uy = s.y * rs;
        s.x = root2 * ux;
        s.y = root2 * uy;
      }
      p.x = p.x + s.x;  // water.h:111
      p.y = p.y + s.y;
      const int jx = (int)p.x, jy = (int)p.y;
      const bool out = oob(jx, jy, T.nx, T.ny);
      const long long c2 = T.cell_base + (long long)jx * T.ny + jy;
      // the tracks need nothing from the next cell: out before its loads
      add_i64(&a.trk[c].td, shy_q32_dev(v.x));  // water.h:115-117
      add_i64(&a.trk[c].tmx, shy_q32_dev(v.x * s.x));
      add_i64(&a.trk[c].tmy, shy_q32_dev(v.x * s.y));
      // the next cell's height and the drop's registration there travel
      // together; the first drop to arrive runs the cell's cascade
      int arrived_before = 1;
      long long qn = 0;
      if (!out) {
        qn = a.cq[c2].hq;
        arrived_before = atomicAdd(&a.cq[c2].cnt[par ^ 1], 1);
      }
      const float h2 = out ? shy_minus_0002(hp) : shy_unq_dev(qn);  // water.h:120-124
      float ceq = r.w * (hp - h2);  // water.h:127-128
      if (ceq < 0.0f) ceq = 0.0f;
      const float edn = ed / (float)nhere;
      const float ex = edn * (ceq - v.y);  // water.h:129-132
      v.y += ex;
      const long long de = -shy_q32_dev(ex);
      add_i64(&a.cq[c].e, de);
      if (!kLean) S.own[j] = de;
      const float s0 = v.y;  // water.h:135-136, without the FP64 unit
      v.y = shy_evap_div_ff(v.y, &ev);
      v.x = vnext;
      // the evaporation gain, an exact difference (Sterbenz), goes straight
      // to the thread's integer total: no drop needs its own
      gain_q += shy_q32_dev(v.y - s0);
      if (out) {  // water.h:139-142
        ++n_oob;
        loss_q += shy_q32_dev(v.y);
        S.age[j] = -2;
        S.ctr[j] = -1;
        continue;
      }
      S.ctr[j] = arrived_before == 0 ? jx * T.ny + jy : -1;  // World::cascade(pos), water.h:151
      if (arrived_before == 0)
        atomicOr(&a.arr[par * a.arr_words + arr_word(T, jx, jy)], arr_bit(jx, jy));
      S.age[j] = (ag + 1) | (kLean && arrived_before == 0 ? kFirstAtCell : 0);
      S.pos[j] = p;
      S.spd[j] = s;
      S.sed[j] = v.y;
    }
    lap(0);
    if (!grid_barrier(a.bar, passed, nullptr)) { ok = false; break; }
    lap(1);

    // ---- scan: the nine heights of each claimed cascade; overlap counts of the steep ones ----
    // heights after phase descend: fixed point plus the step's erosion.  All
    // nine loads are issued together: a neighbour outside the map reads the
    // centre instead and is masked out.  The centre only changes through a
    // transfer, so without any excess to begin with the sequential loop moves
    // nothing and the cascade ends here.
    const bool rev_s = redeals && !(step & 1);
    int c2_n = -1;
    int ti_n2 = 0;
    if ((int)threadIdx.x < nd) {
      const int j = rev_s ? nd - 1 - (int)threadIdx.x : (int)threadIdx.x;
      c2_n = S.ctr[j];
      ti_n2 = one_terrain ? 0 : S.terr[j];
    }
    for (int i = threadIdx.x; i < nd; i += blockDim.x) {
      const int lc = c2_n;  // the claimed centre within the terrain, or -1
      const int ti = ti_n2;
      if (i + (int)blockDim.x < nd) {  // the next slot's claim, loaded ahead
        const int jn = rev_s ? nd - 1 - (i + (int)blockDim.x) : i + (int)blockDim.x;
        c2_n = S.ctr[jn];
        ti_n2 = one_terrain ? 0 : S.terr[jn];
      }
      if (lc < 0) continue;
      const Terrain T = TT[ti];
      const long long c2 = T.cell_base + lc;
      const int ix = lc / T.ny, iy = lc - ix * T.ny;
      longlong2 nv[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        const bool in = !oob(ix + nb_dx(k), iy + nb_dy(k), T.nx, T.ny);
        nv[k] = hq_e(&a.cq[in ? c2 + (long long)nb_dx(k) * T.ny + nb_dy(k) : c2]);
      }
      const longlong2 v0 = hq_e(&a.cq[c2]);
      // the arrivals of the 5 x 5 block: at most 2 x 2 bitmap words, loaded
      // with the heights
      const int tx0 = (ix >= 2 ? ix - 2 : 0) >> 3, tx1 = (ix + 2 < T.nx ? ix + 2 : T.nx - 1) >> 3;
      const int ty0 = (iy >= 2 ? iy - 2 : 0) >> 3, ty1 = (iy + 2 < T.ny ? iy + 2 : T.ny - 1) >> 3;
      const long long tyn = (T.ny + 7) >> 3;
      const unsigned long long* AW = a.arr + par * a.arr_words + T.arr_base;
      const unsigned long long aw00 = load_arr(AW + tx0 * tyn + ty0);
      const unsigned long long aw01 = load_arr(AW + tx0 * tyn + ty1);
      const unsigned long long aw10 = load_arr(AW + tx1 * tyn + ty0);
      const unsigned long long aw11 = load_arr(AW + tx1 * tyn + ty1);
      float sh[8];
#pragma unroll
      for (int k = 0; k < 8; ++k)
        sh[k] = oob(ix + nb_dx(k), iy + nb_dy(k), T.nx, T.ny) ? __int_as_float(0x7f800000)  // never used
                                                              : shy_unq_dev(nv[k].x + nv[k].y);
      const float h0 = shy_unq_dev(v0.x + v0.y);
      bool any = false;
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        const float diff = h0 - sh[k];
        const float dist = (nb_dx(k) != 0 && nb_dy(k) != 0) ? sqrtf(2.0f) : 1.0f;
        const float excess = sh[k] >= 0.1f ? fabsf(diff) - dist * P.max_diff : fabsf(diff);
        any |= (sh[k] < __int_as_float(0x7f800000)) && diff != 0.0f && excess > 0.0f;
      }
      if (any) {
        // one claim per drop slot, so the queue (cap entries) cannot overflow;
        // the transfers are worked out during the barrier, off this phase's tail
        SteepCell& q = S.steep[atomicAdd(&s_nq, 1)];
        q.c2 = c2;
        q.ti = ti;
        q.h0 = h0;
#pragma unroll
        for (int k = 0; k < 8; ++k) q.u.in.v[k] = sh[k];
        q.u.in.aw[0] = aw00;
        q.u.in.aw[1] = aw01;
        q.u.in.aw[2] = aw10;
        q.u.in.aw[3] = aw11;
        q.u.in.tx0 = tx0;
        q.u.in.ty0 = ty0;
        q.u.in.ix = ix;
        q.u.in.iy = iy;
      }
    }
    lap(2);
    // The queued cascades' transfers use only what scan read, so warps 1 and
    // up work them out while thread 0 waits; the entries go to the highest
    // threads first (those past the CTA's last drop slot) and each thread
    // adds its own entries' changes in settle.
    auto transfers = [&]() {
      const int nq = s_nq;
      for (int i = (int)blockDim.x - 1 - (int)threadIdx.x; i < nq; i += (int)blockDim.x - 32)
        steep_transfers(S.steep[i], TT[S.steep[i].ti], P);
    };
    if (!grid_barrier(a.bar, passed, nullptr, transfers)) { ok = false; break; }
    lap(3);

    // ---- settle: steep cascades, each drop's own change, retirements ----
    // Every addition here is an integer atomic on a fixed-point height that
    // nobody reads in this phase, so the order does not matter.
    if (threadIdx.x >= 32) {  // the entries each thread worked out during the barrier
      const int nq = s_nq;
      for (int i = (int)blockDim.x - 1 - (int)threadIdx.x; i < nq; i += (int)blockDim.x - 32)
        steep_apply(S.steep[i], TT[S.steep[i].ti], a.cq);
    }
    // the other parity's bitmap (last read in the previous step's scan)
    // starts empty for the next step's descend: this CTA's share of it
    {
      unsigned long long* other = a.arr + (par ^ 1) * a.arr_words;
      const long long w0 = (long long)blockIdx.x * a.arr_words / gridDim.x;
      const long long w1 = (long long)(blockIdx.x + 1) * a.arr_words / gridDim.x;
      for (long long i = w0 + threadIdx.x; i < w1; i += blockDim.x) other[i] = 0ull;
    }
    unsigned long long retired = 0;
    const bool rev_t = redeals && (step & 1);
    int ag_f = -1, lc_f = -1, ti_f = 0;
    long long own_f = 0;
    if ((int)threadIdx.x < nd) {
      const int j = rev_t ? nd - 1 - (int)threadIdx.x : (int)threadIdx.x;
      ag_f = S.age[j]; lc_f = S.cell[j]; ti_f = one_terrain ? 0 : S.terr[j];
      if (!kLean) own_f = S.own[j];
    }
    for (int i = threadIdx.x; i < nd; i += blockDim.x) {
      const int j = rev_t ? nd - 1 - i : i;
      const int ag = ag_f, lcs = lc_f, tis = ti_f;
      long long own = own_f;
      long long c = -1;
      if (ag != -1 && lcs >= 0) {
        c = TT[tis].cell_base + lcs;
        // kLean: the cell's whole pending sum (final since descend), loaded
        // before the next slot's fields so that the two round trips overlap
        if (kLean) own = a.cq[c].e;
      }
      if (i + (int)blockDim.x < nd) {  // the next slot, loaded ahead
        const int jn = rev_t ? nd - 1 - (i + (int)blockDim.x) : i + (int)blockDim.x;
        ag_f = S.age[jn]; lc_f = S.cell[jn]; ti_f = one_terrain ? 0 : S.terr[jn];
        if (!kLean) own_f = S.own[jn];
      }
      if (ag == -1) continue;
      if (c >= 0) {
        if (own != 0) add_i64(&a.cq[c].hq, own);
        a.cq[c].e = 0;
        a.cq[c].cnt[par] = 0;
      }
      if (ag == -2) {
        S.age[j] = -1;
        S.cell[j] = -1;
        ++retired;
      }
    }
    {  // per warp into the shared counter; the barrier takes it off the live count
      const unsigned r = __reduce_add_sync(0xffffffffu, (unsigned)retired);
      if ((threadIdx.x & 31) == 0 && r) atomicAdd(&s_retired, r);
    }
    lap(4);
    if (!grid_barrier(a.bar, passed, &s_live, [] {}, 0u, kBarrierLimitNs, 0, &s_retired)) {
      ok = false;
      break;
    }
    // every CTA sees the same step and live count, so all take the same
    // barriers
    if (redeals && (step + 1) % a.resort == 0 && s_live != 0) {
      const Redealt r = redeal<kBlock>(a, TT, lo, nd, buf, passed, (long long)s_live);
      passed += 3;
      if (!r.ok) {
        ok = false;
        break;
      }
      lo = r.lo;
      nd = r.nd;
      buf ^= 1;
      S = slots_global(a, buf, lo);
    }
  }
  lap(5);

  // counters
  {
    unsigned long long v;
    v = block_sum_u64<kBlock>(n_steps);   if (threadIdx.x == 0 && v) atomicAdd(&a.st->steps, v);
    v = block_sum_u64<kBlock>(n_oob);     if (threadIdx.x == 0 && v) atomicAdd(&a.st->oob, v);
    v = block_sum_u64<kBlock>(n_drops);   if (threadIdx.x == 0 && v) atomicAdd(&a.st->drops, v);
    v = block_sum_u64<kBlock>(n_skipped); if (threadIdx.x == 0 && v) atomicAdd(&a.st->skipped, v);
    v = block_sum_u64<kBlock>((unsigned long long)gain_q);
    if (threadIdx.x == 0 && v) atomicAdd((unsigned long long*)&a.st->gain_q, v);
    v = block_sum_u64<kBlock>((unsigned long long)loss_q);
    if (threadIdx.x == 0 && v) atomicAdd((unsigned long long*)&a.st->loss_q, v);
  }
  if (timer) {
    for (int i = 0; i < 6; ++i) a.bar->phase_ns[i] += s_ph[i];
    a.bar->iterations += (unsigned long long)step;
    if (ok && s_live != 0) atomicCAS(&a.bar->error, 0, SHY_ERR_STATE);
  }
}

// End of a batched cycle: tracks to float, lrate blend (source/world.h:81-86),
// records for the next cycle, accumulators cleared.
__global__ void cycle_end_kernel(Tracks* __restrict__ trk, float4* __restrict__ rec,
                                 float* __restrict__ track_f, const CellQ* __restrict__ cq,
                                 float* __restrict__ h, long long cells, shy_params P, GridBar* bar,
                                 DevStats* st) {
  const float a = 1.0f - P.lrate, b = P.lrate;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < cells;
       i += (long long)gridDim.x * blockDim.x) {
    h[i] = shy_unq(cq[i].hq);
    const Tracks q = trk[i];
    const float fd = shy_unq(q.td), fx = shy_unq(q.tmx), fy = shy_unq(q.tmy);
    track_f[i] = fd;
    track_f[cells + i] = fx;
    track_f[2 * cells + i] = fy;
    float4 r = rec[i];
    r.z = a * r.z + b * fd;
    r.x = a * r.x + b * fx;
    r.y = a * r.y + b * fy;
    r.w = 1.0f + P.entrainment * shy_erff_ff(0.4f * r.z);
    rec[i] = r;
    Tracks z;
    z.td = 0;
    z.tmx = 0;
    z.tmy = 0;
    z.pad = 0;
    trk[i] = z;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    bar->arrive = 0;
    bar->live = 0;
    bar->cycle += 1;
    st->cycles += 1;
  }
}

// Optional slope relaxation: World::cascade's transfer rule
// (source/world.h:138-164) as a symmetric stencil over neighbour pairs of
// which at least one cell was visited this cycle.  Reads (hin, hqin), writes
// (hout, hqout); transfers are summed in 32.32 fixed point.
__global__ void relax_kernel(const Terrain* __restrict__ terrains, int n_terrains,
                             const float* __restrict__ hin, const CellQ* __restrict__ cqin,
                             float* __restrict__ hout, long long* __restrict__ hqout,
                             const float* __restrict__ td, long long cells, shy_params P) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < cells;
       i += (long long)gridDim.x * blockDim.x) {
    int t = 0;
    while (t + 1 < n_terrains && terrains[t + 1].cell_base <= i) ++t;
    const Terrain T = terrains[t];
    const long long lc = i - T.cell_base;
    const int x = (int)(lc / T.ny), y = (int)(lc - (long long)x * T.ny);
    const float hc = hin[i];
    const bool mc = td[i] != 0.0f;
    long long sum = 0;
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      const int x2 = x + nb_dx(k), y2 = y + nb_dy(k);
      if (oob(x2, y2, T.nx, T.ny)) continue;
      const long long n = T.cell_base + (long long)x2 * T.ny + y2;
      if (!(mc || td[n] != 0.0f)) continue;
      const float hn = hin[n];
      const float diff = hc - hn;
      if (diff == 0.0f) continue;
      const float dist = (nb_dx(k) != 0 && nb_dy(k) != 0) ? sqrtf(2.0f) : 1.0f;
      const float lo = hc < hn ? hc : hn;
      const float excess = lo >= 0.1f ? fabsf(diff) - dist * P.max_diff : fabsf(diff);
      if (excess <= 0.0f) continue;
      const float transfer = P.cascade_weight * (P.settling * excess / 2.0f);
      sum += diff > 0.0f ? -shy_q32(transfer) : shy_q32(transfer);
    }
    const long long nh = cqin[i].hq + sum;
    hqout[i] = nh;
    hout[i] = shy_unq(nh);
  }
}

__global__ void relax_commit_kernel(CellQ* __restrict__ cq, const long long* __restrict__ hq, long long cells) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < cells;
       i += (long long)gridDim.x * blockDim.x)
    cq[i].hq = hq[i];
}

// Heights into the batched mode's fixed point, and the float maps re-rounded
// from it.
__global__ void heights_to_fixed_kernel(float* __restrict__ h, CellQ* __restrict__ cq, long long cells) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < cells;
       i += (long long)gridDim.x * blockDim.x) {
    const long long q = shy_q32(h[i]);
    cq[i].hq = q;
    h[i] = shy_unq(q);
  }
}

int cells_grid(long long cells) {
  long long b = (cells + 255) / 256;
  return (int)(b > 65536 ? 65536 : (b < 1 ? 1 : b));
}

}  // namespace

namespace {

// Slot order of a cycle: drops sorted by their spawn cell, in runs of
// 2^shift consecutive cells (x-major), so that each CTA's drops start in one
// compact stretch of the maps.  Which slot runs which drop does not change
// any result (every sum is an integer sum, and a cascade is the same
// whichever drop claims it); the order within a run is whatever the atomics
// give.
__global__ void order_count_kernel(const Terrain* __restrict__ terrains, int n_terrains, int total,
                                   const GridBar* __restrict__ bar, int shift, int* __restrict__ hist,
                                   int* __restrict__ key, int* __restrict__ rank) {
  const unsigned long long cycle = bar->cycle;
  for (int d = blockIdx.x * blockDim.x + threadIdx.x; d < total; d += gridDim.x * blockDim.x) {
    const Terrain T = terrains[find_terrain(terrains, n_terrains, d)];
    int x, y;
    shy_spawn_xy(T.seed, cycle, (unsigned)(d - T.drop_base), T.nx, T.ny, &x, &y);
    const int b = (int)((T.cell_base + (long long)x * T.ny + y) >> shift);
    key[d] = b;
    rank[d] = atomicAdd(&hist[b], 1);
  }
}

// exclusive prefix sum of hist[0 .. n) in place, one CTA of 1024 threads
__global__ void order_scan_kernel(int* __restrict__ hist, int n) {
  __shared__ int part[1024];
  const int per = (n + 1023) / 1024, b0 = threadIdx.x * per;
  int s = 0;
  for (int i = 0; i < per && b0 + i < n; ++i) s += hist[b0 + i];
  part[threadIdx.x] = s;
  __syncthreads();
  for (int o = 1; o < 1024; o <<= 1) {  // inclusive scan of the parts
    const int v = threadIdx.x >= (unsigned)o ? part[threadIdx.x - o] : 0;
    __syncthreads();
    part[threadIdx.x] += v;
    __syncthreads();
  }
  int run = threadIdx.x ? part[threadIdx.x - 1] : 0;
  for (int i = 0; i < per && b0 + i < n; ++i) {
    const int h = hist[b0 + i];
    hist[b0 + i] = run;
    run += h;
  }
}

__global__ void order_scatter_kernel(int total, const int* __restrict__ hist, const int* __restrict__ key,
                                     const int* __restrict__ rank, int* __restrict__ order) {
  for (int d = blockIdx.x * blockDim.x + threadIdx.x; d < total; d += gridDim.x * blockDim.x)
    order[hist[key[d]] + rank[d]] = d;
}

}  // namespace

// the bucket shift that keeps the spawn-order histogram at most 65,536 runs
int order_shift(long long cells) {
  int shift = 0;
  while ((cells >> shift) > 65535) ++shift;
  return shift;
}

// The re-deal's buckets for `total` drops on `cells` cells and a grid of
// `grid` CTAs: about four per run of drops (finer buckets order a run's
// drops along the map, coarser ones keep CTA 0's prefix sum short), at most
// kResortBuckets, the count used rounded up to whole kResortBucketStep.
void resort_buckets(long long cells, long long total, long long grid, int* shift, int* used) {
  const long long R = order_run(total, grid);
  long long want = 4 * ((total + R - 1) / R);
  if (want > kResortBuckets) want = kResortBuckets;
  int s = 0;
  while (((cells - 1) >> s) + 1 > want) ++s;
  const long long n = ((cells - 1) >> s) + 1;
  *shift = s;
  *used = (int)((n + kResortBucketStep - 1) / kResortBucketStep * kResortBucketStep);
}

cudaError_t launch_spawn_order(shy_world* w, int total) {
  const int shift = order_shift(w->cells);
  const int nb = (int)((w->cells - 1) >> shift) + 1;
  cudaError_t e;
  if ((e = cudaMemsetAsync(w->dhist, 0, sizeof(int) * (size_t)nb, w->stream)) != cudaSuccess) return e;
  const int grid = (int)(((long long)total + 255) / 256 < 4096 ? ((long long)total + 255) / 256 : 4096);
  order_count_kernel<<<grid < 1 ? 1 : grid, 256, 0, w->stream>>>(w->dterrains, (int)w->terrains.size(), total,
                                                                  w->bar, shift, w->dhist, w->dkey, w->drank);
  order_scan_kernel<<<1, 1024, 0, w->stream>>>(w->dhist, nb);
  order_scatter_kernel<<<grid < 1 ? 1 : grid, 256, 0, w->stream>>>(total, w->dhist, w->dkey, w->drank,
                                                                    w->dorder);
  return cudaGetLastError();
}

namespace {

// Launches one lock-step cycle with CTAs of kBlock threads.  The grid is
// the resident CTAs per SM times the SMs (fewer for small cycles: at least 32
// drops per CTA); each CTA's drop slots go to shared memory when they fit
// without lowering that occupancy (and the world allows it), else to the
// global arrays in `a`.
// What a launch of lockstep_kernel<kBlock, kRedeal, kLean> needs to know about the device,
// queried once per device and CTA size (and per dynamic shared-memory size
// for the occupancy with slots in shared memory) rather than every cycle.
struct LaunchFacts {
  bool valid = false;
  int optin = 0;               // opt-in shared memory per CTA
  long long static_smem = 0;   // the kernel's static shared memory
  int per0 = 0;                // resident CTAs per SM without dynamic shared memory
  long long smem_set = 0;      // dynamic shared memory the attribute allows
  long long last_b = -1;       // last dynamic size asked about, and its
  int last_per = 0;            //   resident CTAs per SM
};
const int kMaxDevices = 64;
std::mutex g_facts_mu;

template <int kBlock, bool kRedeal, bool kLean>
cudaError_t launch_facts(LaunchFacts** out) {
  static LaunchFacts facts[kMaxDevices];
  int dev = 0;
  cudaError_t e;
  if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDevices) return cudaErrorInvalidDevice;
  LaunchFacts& f = facts[dev];
  if (!f.valid) {
    if ((e = cudaDeviceGetAttribute(&f.optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev)) != cudaSuccess) return e;
    cudaFuncAttributes fa;
    if ((e = cudaFuncGetAttributes(&fa, lockstep_kernel<kBlock, kRedeal, kLean>)) != cudaSuccess) return e;
    f.static_smem = (long long)fa.sharedSizeBytes;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&f.per0, lockstep_kernel<kBlock, kRedeal, kLean>, kBlock,
                                                           0)) !=
        cudaSuccess)
      return e;
    f.valid = true;
  }
  *out = &f;
  return cudaSuccess;
}

// Launches one lock-step cycle with CTAs of kBlock threads.  The grid is
// the resident CTAs per SM times the SMs (fewer for small cycles: at least 32
// drops per CTA); each CTA's drop slots go to shared memory when they fit
// without lowering that occupancy (and the world allows it), else to the
// global arrays in `a`.
template <int kBlock>
cudaError_t launch_lockstep_n(LockArgs& a, int sm_count, int grid_hint, cudaStream_t stream) {
  std::lock_guard<std::mutex> lock(g_facts_mu);
  LaunchFacts* f = nullptr;
  cudaError_t e;
  if ((e = launch_facts<kBlock, false, false>(&f)) != cudaSuccess) return e;
  if (f->per0 < 1) return cudaErrorLaunchOutOfResources;
  const long long max_dyn = (long long)f->optin - f->static_smem;
  long long want = ((long long)a.total_drops + 31) / 32;
  if (want < 1) want = 1;
  if (grid_hint > 0 && want > grid_hint) want = grid_hint;

  const long long g = (long long)f->per0 * sm_count < want ? (long long)f->per0 * sm_count : want;
  const int grid = (int)g;
  const long long b = (long long)slot_range(a.total_drops, g, 0, a.order != nullptr).cap * kSlotBytes;
  size_t bytes = 0;
  a.smem_slots = 0;
  if (b <= max_dyn && a.smem_allowed) {
    if (b > 48 * 1024 && b > f->smem_set) {
      if ((e = cudaFuncSetAttribute(lockstep_kernel<kBlock, false, false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)b)) !=
          cudaSuccess)
        return e;
      f->smem_set = b;
    }
    if (b != f->last_b) {
      int per = 0;
      if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, lockstep_kernel<kBlock, false, false>, kBlock,
                                                             (size_t)b)) !=
          cudaSuccess)
        return e;
      f->last_b = b;
      f->last_per = per;
    }
    if ((long long)f->last_per * sm_count >= g) {  // the slots fit without costing occupancy
      a.smem_slots = 1;
      bytes = (size_t)b;
    }
  }
  void* args[] = {&a};
  if (!a.smem_slots && a.resort > 0) {
    // slots in global memory with re-deals: the other instantiation, with
    // its own residency (every CTA of a cooperative launch must fit at once)
    LaunchFacts* fr = nullptr;
    if ((e = (a.lean ? launch_facts<kBlock, true, true>(&fr) : launch_facts<kBlock, true, false>(&fr))) !=
        cudaSuccess)
      return e;
    if (fr->per0 < 1) return cudaErrorLaunchOutOfResources;
    const long long gr = (long long)fr->per0 * sm_count < want ? (long long)fr->per0 * sm_count : want;
    resort_buckets(a.cells, a.total_drops, gr, &a.rshift, &a.rbuckets);
    const void* k = a.lean ? (const void*)lockstep_kernel<kBlock, true, true>
                           : (const void*)lockstep_kernel<kBlock, true, false>;
    return cudaLaunchCooperativeKernel(k, dim3((int)gr), dim3(kBlock), args, 0, stream);
  }
  a.resort = 0;
  a.lean = 0;
  return cudaLaunchCooperativeKernel((const void*)lockstep_kernel<kBlock, false, false>, dim3(grid), dim3(kBlock), args, bytes,
                                     stream);
}

cudaError_t launch_lockstep(LockArgs& a, int sm_count, int grid_hint, int block, cudaStream_t stream) {
  switch (block) {
    case 64: return launch_lockstep_n<64>(a, sm_count, grid_hint, stream);
    case 128: return launch_lockstep_n<128>(a, sm_count, grid_hint, stream);
    default: return launch_lockstep_n<kLockBlock>(a, sm_count, grid_hint, stream);
  }
}

}  // namespace

cudaError_t launch_batched_cycle(shy_world* w) {
  LockArgs a;
  a.terrains = w->dterrains;
  a.n_terrains = (int)w->terrains.size();
  a.total_drops = 0;
  for (const auto& T : w->terrains) a.total_drops += T.drops;
  a.cells = w->cells;
  a.h = w->h;
  a.cq = w->cq;
  a.rec = w->rec;
  a.voltab = w->voltab;
  a.ev = shy_evap_make(w->P.evap_rate);
  a.trk = w->trk;
  a.pos = w->dpos;
  a.spd = w->dspd;
  a.sed = w->dsed;
  a.age = w->dage;
  a.own = w->down;
  a.terr = w->dterr;
  a.cell = w->dcell;
  a.ctr = w->dctr;
  a.steep = w->dsteep;
  a.arr = w->arr;
  a.arr_words = w->arr_words;
  // Drops sorted by spawn cell and dealt to the CTAs in runs when the cell
  // state outgrows L2: each run touches a compact stretch of the maps, and
  // every CTA holds runs from the whole map, so its live drops stay in
  // balance with the other CTAs'.  While the state fits in L2 the slots keep
  // the drop order.
  const long long state_bytes = w->cells * (long long)(sizeof(CellQ) + sizeof(Tracks) + sizeof(float4) + 4);
  const bool ordered = w->batch_order < 0 ? state_bytes > w->l2_bytes : w->batch_order != 0;
  a.order = ordered ? w->dorder : nullptr;
  a.pos2 = w->dpos2;
  a.spd2 = w->dspd2;
  a.sed2 = w->dsed2;
  a.age2 = w->dage2;
  a.terr2 = w->dterr2;
  a.rhist = w->dresort;
  a.rshift = 0;  // set with the grid (launch_lockstep_n)
  a.rbuckets = 0;
  a.resort = w->batch_resort < 0 ? (ordered ? kResortSteps : 0) : w->batch_resort;
  // the slots' persistent fields and per-step fields (about 40 B a drop)
  // larger than L2: their loads miss anyway, so settling whole cells from
  // their first drops costs no extra wait and saves the own-change bytes
  a.lean = w->batch_settle < 0 ? ((long long)a.total_drops * 40 > w->l2_bytes ? 1 : 0) : w->batch_settle;
  a.smem_slots = 0;
  a.P = w->P;
  a.st = w->stats;
  a.bar = w->bar;
  a.max_steps = (int)w->P.max_age + 3;
  a.stall_ns = debug_stall_ns();

  int slot = -1;
  cudaError_t e;
  if (a.order && a.total_drops > 0) {
    if ((e = timing_begin(w, SHY_KERNEL_OTHER, &slot)) != cudaSuccess) return e;
    if ((e = launch_spawn_order(w, a.total_drops)) != cudaSuccess) return e;
    if ((e = timing_end(w, slot)) != cudaSuccess) return e;
  }
  if ((e = timing_begin(w, SHY_KERNEL_DROPS, &slot)) != cudaSuccess) return e;
  a.smem_allowed = w->batch_smem;
  if ((e = launch_lockstep(a, w->sm_count, w->batch_grid, w->batch_block, w->stream)) != cudaSuccess) return e;
  if ((e = timing_end(w, slot)) != cudaSuccess) return e;

  if ((e = timing_begin(w, SHY_KERNEL_APPLY, &slot)) != cudaSuccess) return e;
  cycle_end_kernel<<<cells_grid(w->cells), 256, 0, w->stream>>>(w->trk, w->rec, w->track_f, w->cq, w->h,
                                                                w->cells, w->P, w->bar, w->stats);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if ((e = timing_end(w, slot)) != cudaSuccess) return e;

  for (int p = 0; p < w->P.cascade_passes; ++p) {
    if ((e = timing_begin(w, SHY_KERNEL_CASCADE, &slot)) != cudaSuccess) return e;
    relax_kernel<<<cells_grid(w->cells), 256, 0, w->stream>>>(w->dterrains, (int)w->terrains.size(), w->h,
                                                              w->cq, w->relax, w->hq_relax, w->track_f,
                                                              w->cells, w->P);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    e = cudaMemcpyAsync(w->h, w->relax, sizeof(float) * w->cells, cudaMemcpyDeviceToDevice, w->stream);
    if (e != cudaSuccess) return e;
    relax_commit_kernel<<<cells_grid(w->cells), 256, 0, w->stream>>>(w->cq, w->hq_relax, w->cells);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if ((e = timing_end(w, slot)) != cudaSuccess) return e;
  }
  return cudaSuccess;
}

// One batched cycle (lock-step kernel + end-of-cycle kernel) on buffers the
// caller provides; no relax passes.
cudaError_t launch_cycle_buffers(const CycleBuffers& b, cudaStream_t stream) {
  LockArgs a;
  a.terrains = b.terrains;
  a.n_terrains = b.n_terrains;
  a.total_drops = b.total_drops;
  a.cells = b.cells;
  a.h = b.h;
  a.cq = b.cq;
  a.rec = b.rec;
  a.voltab = b.voltab;
  a.ev = shy_evap_make(b.P.evap_rate);
  a.trk = b.trk;
  a.pos = b.pos;
  a.spd = b.spd;
  a.sed = b.sed;
  a.age = b.age;
  a.own = b.own;
  a.terr = b.terr;
  a.cell = b.cell;
  a.ctr = b.ctr;
  a.steep = b.steep;
  a.arr = b.arr;
  a.arr_words = b.arr_words;
  a.order = nullptr;
  a.pos2 = a.spd2 = nullptr;
  a.sed2 = nullptr;
  a.age2 = a.terr2 = a.rhist = nullptr;
  a.rshift = 0;
  a.rbuckets = 0;
  a.resort = 0;  // no second set of slots in the caller's buffers
  a.lean = 0;
  a.smem_slots = 0;
  a.P = b.P;
  a.st = b.st;
  a.bar = b.bar;
  a.max_steps = (int)b.P.max_age + 3;
  a.stall_ns = debug_stall_ns();
  a.smem_allowed = 1;
  cudaError_t e = launch_lockstep(a, b.sm_count, 0, kLockBlock, stream);
  if (e != cudaSuccess) return e;
  cycle_end_kernel<<<cells_grid(b.cells), 256, 0, stream>>>(b.trk, b.rec, b.track_f, b.cq, b.h, b.cells, b.P,
                                                            b.bar, b.st);
  return cudaGetLastError();
}

namespace {

// After a cycle that gave up (a timed-out barrier): the pending sums and
// drop counts it left behind are cleared and the barrier state reset, so the
// world's next batched call starts clean.
__global__ void batched_recover_kernel(CellQ* __restrict__ cq, long long cells, GridBar* bar) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < cells;
       i += (long long)gridDim.x * blockDim.x) {
    cq[i].e = 0;
    cq[i].cnt[0] = 0;
    cq[i].cnt[1] = 0;
  }
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    bar->arrive = 0;
    bar->live = 0;
    bar->abort = 0;
    bar->error = 0;
  }
}

}  // namespace

cudaError_t launch_batched_recover(shy_world* w) {
  batched_recover_kernel<<<cells_grid(w->cells), 256, 0, w->stream>>>(w->cq, w->cells, w->bar);
  return cudaGetLastError();
}

cudaError_t launch_heights_to_fixed(shy_world* w) {
  heights_to_fixed_kernel<<<cells_grid(w->cells), 256, 0, w->stream>>>(w->h, w->cq, w->cells);
  return cudaGetLastError();
}

}  // namespace shy
