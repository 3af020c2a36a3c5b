// shy_lockstep.cu -- the batched erosion mode.
//
// One batched cycle is World::erode(drops) (source/world.h:54-88) with all
// drops of every terrain of the world descending at once, one drop per
// thread slot, in lock step.  Step t is three phases separated by grid-wide
// barriers:
//   A  each live drop takes one Drop::descend step (source/water.h:58-156)
//      against the heights after step t-1.  A drop sharing its cell with n-1
//      other live drops exchanges sediment at rate effD / n (n = 1 is the
//      reference).  The height change goes to the cell's pending erosion sum
//      and the three tracks to its track record, as 32.32 fixed-point integer
//      atomics.  Each drop registers at its new cell (the count of the next
//      step); the first to arrive runs that cell's cascade.
//   C  World::cascade (source/world.h:90-168) at every claimed cell on the
//      heights as phase A left them; transfers go to the pending records.
//      Cascades that move nothing are settled by their own thread; the steep
//      ones are queued and run one per warp after one more barrier.
//      Where the 3 x 3 blocks of k cascades overlap, a pair's transfer is
//      divided by k (the larger count of its two cells), so overlapping
//      cascades together move what one would; the counts come from the
//      arrivals registered in the 5 x 5 block around the centre.
//   D  every drop adds its own height change to its cell's fixed-point
//      height and clears the cell's pending sum and count; each cascade adds
//      what it moved; finished drops retire.
// Heights live in 32.32 fixed point for the whole cycle (the float map is
// rewritten at its end), so every update is an integer addition.
// Integer sums make every result independent of thread timing: the same
// inputs give the same bits on every run, and oracle/hydro_oracle.cpp
// (Lockstep) restates the schedule on the CPU.
//
// The end-of-cycle kernel converts the tracks to float, applies the lrate
// blend (source/world.h:81-86) and rebuilds the per-cell records.
#include "shy_device.cuh"

namespace shy {

namespace {

const int kLockBlock = 256;
const int kSmemTerrains = 128;
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

// Grid-wide barrier over a monotonically increasing arrival counter (reset to
// zero between launches).  `passed` counts the barriers this CTA has passed.
// Every wait is bounded: past kBarrierLimitNs the waiter sets bar->abort and
// every later barrier returns false at once, so the kernel always ends.
__device__ bool grid_barrier(GridBar* bar, unsigned long long& passed) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned long long target = (passed + 1) * (unsigned long long)gridDim.x;
    red_release_add_u64(&bar->arrive, 1ull);
    int ok = 1;
    unsigned long long t0 = 0;
    unsigned spins = 0;
    while (ld_acquire_u64(&bar->arrive) < target) {
      if (++spins < 64) continue;
      if (t0 == 0) t0 = global_ns();
      if (ld_relaxed_i32(&bar->abort)) {
        ok = 0;
        break;
      }
      if (global_ns() - t0 > kBarrierLimitNs) {
        atomicExch(&bar->abort, 1);
        atomicCAS(&bar->error, 0, SHY_ERR_TIMEOUT);
        ok = 0;
        break;
      }
      __nanosleep(64);
    }
    s_ok = ok;
  }
  __syncthreads();
  ++passed;
  return s_ok != 0;
}

struct LockArgs {
  const Terrain* terrains;
  int n_terrains;
  int total_drops;
  long long cells;
  const float* h;  // heights rounded to float at cycle start (spawn test)
  CellQ* cq;       // fixed-point heights, pending changes, drop counts
  const float4* rec;
  const float* effd;
  const float* voltab;  // volume after k evaporations (source/water.h:136)
  shy_evap ev;
  Tracks* trk;
  float2* pos;
  float2* spd;
  float2* vs;
  int* age;
  long long* gain;  // evaporation gain of the drop so far, 32.32
  long long* own;   // the drop's own height change this step, 32.32
  int* terr;
  long long* cell;
  long long* ctr;
  int* cmask;
  SteepCell* steep;  // this step's steep cascades
  shy_params P;
  DevStats* st;
  GridBar* bar;
  int max_steps;
};

__device__ __forceinline__ int find_terrain(const Terrain* T, int n, int d) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (T[mid].drop_base <= d) lo = mid; else hi = mid - 1;
  }
  return lo;
}

__device__ __forceinline__ unsigned long long block_sum_u64(unsigned long long v) {
  __shared__ unsigned long long red[kLockBlock / 32];
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
  const float dd = n.x * n.x + n.y * n.y + n.z * n.z;
  if (sqrtf(dd) > 0.0f) {
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

__global__ void __launch_bounds__(kLockBlock) lockstep_kernel(LockArgs a) {
  __shared__ Terrain sT[kSmemTerrains];
  const bool smem_t = a.n_terrains <= kSmemTerrains;
  if (smem_t)
    for (int i = threadIdx.x; i < a.n_terrains; i += blockDim.x) sT[i] = a.terrains[i];
  __syncthreads();
  const Terrain* TT = smem_t ? sT : a.terrains;

  const long long G = (long long)gridDim.x * blockDim.x;
  const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const shy_params& P = a.P;
  const unsigned long long cycle = a.bar->cycle;
  const bool timer = blockIdx.x == 0 && threadIdx.x == 0;
  unsigned long long ph[6] = {0, 0, 0, 0, 0, 0};
  unsigned long long tprev = timer ? global_ns() : 0;
  auto lap = [&](int i) {
    if (timer) {
      const unsigned long long t = global_ns();
      ph[i] += t - tprev;
      tprev = t;
    }
  };
  unsigned long long passed = 0;
  unsigned long long n_steps = 0, n_oob = 0, n_drops = 0, n_skipped = 0;
  long long gain_q = 0, loss_q = 0;
  const shy_evap ev = a.ev;

  // spawn (source/world.h:64-74)
  unsigned long long born = 0;
  for (long long d = tid; d < a.total_drops; d += G) {
    const int t = find_terrain(TT, a.n_terrains, (int)d);
    const Terrain T = TT[t];
    int x, y;
    shy_spawn_xy(T.seed, cycle, (unsigned)(d - T.drop_base), T.nx, T.ny, &x, &y);
    const long long c = T.cell_base + (long long)x * T.ny + y;
    a.terr[d] = t;
    a.cell[d] = -1;
    a.ctr[d] = -1;
    // world.h:71; no float lies between 0.1 and 0.1f, so this is h < 0.1
    if (a.h[c] < 0.1f) {
      a.age[d] = -1;
      ++n_skipped;
      continue;
    }
    ++n_drops;
    ++born;
    a.age[d] = 0;
    a.pos[d] = make_float2((float)x, (float)y);
    a.spd[d] = make_float2(0.0f, 0.0f);
    a.vs[d] = make_float2(1.0f, 0.0f);
    a.gain[d] = 0;
    atomicAdd(&a.cq[c].cnt[0], 1);
  }
  {
    const unsigned long long s = block_sum_u64(born);
    if (threadIdx.x == 0 && s) atomicAdd(&a.bar->live, s);
  }
  bool ok = grid_barrier(a.bar, passed);

  int step = 0;
  for (; ok && step < a.max_steps; ++step) {
    if (*((volatile unsigned long long*)&a.bar->live) == 0) break;
    const int par = step & 1;
    lap(5);

    // ---- phase A: one descend step per live drop ----
    for (long long d = tid; d < a.total_drops; d += G) {
      const int ag = a.age[d];
      const int ti = a.terr[d];
      float2 p = a.pos[d], s = a.spd[d], v = a.vs[d];
      long long gn = a.gain[d];
      if (ag < 0) continue;
      const Terrain T = TT[ti];
      const CellQ* RT = a.cq + T.cell_base;
      const int ix = (int)p.x, iy = (int)p.y;
      const long long lc = (long long)ix * T.ny + iy;
      const long long c = T.cell_base + lc;
      a.cell[d] = c;
      // the five heights quad::_normal reads (0 outside the map)
      const bool xp = ix + 1 < T.nx, xm = ix > 0, yp = iy + 1 < T.ny, ym = iy > 0;
      // all loads issued together; a neighbour outside the map reads the
      // centre and is masked to height 0
      const long long q0 = RT[lc].hq;
      const int nhere = RT[lc].cnt[par];
      long long qxp = RT[xp ? lc + T.ny : lc].hq;
      long long qxm = RT[xm ? lc - T.ny : lc].hq;
      long long qyp = RT[yp ? lc + 1 : lc].hq;
      long long qym = RT[ym ? lc - 1 : lc].hq;
      const float4 r = __ldg(&a.rec[c]);
      const float ed = __ldg(&a.effd[c]);
      qxp = xp ? qxp : 0;
      qxm = xm ? qxm : 0;
      qyp = yp ? qyp : 0;
      qym = ym ? qym : 0;
      const float hp = shy_unq(q0);
      const float3 n = normal5(hp, shy_unq(qxp), shy_unq(qxm), shy_unq(qyp), shy_unq(qym), xp && yp, xm && ym,
                               xp && ym, xm && yp, P.map_scale);
      if ((float)ag > P.max_age || v.x < P.min_vol) {  // water.h:74-83
        const long long dep = shy_q32(v.y);
        add_i64(&a.cq[c].e, dep);
        a.own[d] = dep;
        gain_q += gn;
        a.age[d] = -2;
        a.ctr[d] = -1;
        continue;
      }
      ++n_steps;
      s.x = s.x + (P.gravity * n.x) / v.x;  // water.h:95
      s.y = s.y + (P.gravity * n.z) / v.x;
      if (len2(r.x, r.y) > 0.0f && len2(s.x, s.y) > 0.0f) {  // water.h:97-99
        const float rf = 1.0f / sqrtf(dot2(r.x, r.y, r.x, r.y));
        const float rs = 1.0f / sqrtf(dot2(s.x, s.y, s.x, s.y));
        const float k = (P.momentum_transfer * dot2(r.x * rf, r.y * rf, s.x * rs, s.y * rs)) / (v.x + r.z);
        s.x = s.x + k * r.x;
        s.y = s.y + k * r.y;
      }
      if (len2(s.x, s.y) > 0.0f) {  // water.h:108-109
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
      // the next cell's height and the drop's registration there travel
      // together; the first drop to arrive runs the cell's cascade
      int arrived_before = 1;
      long long qn = 0;
      if (!out) {
        qn = a.cq[c2].hq;
        arrived_before = atomicAdd(&a.cq[c2].cnt[par ^ 1], 1);
      }
      add_i64(&a.trk[c].td, shy_q32(v.x));  // water.h:115-117
      add_i64(&a.trk[c].tmx, shy_q32(v.x * s.x));
      add_i64(&a.trk[c].tmy, shy_q32(v.x * s.y));
      const float h2 = out ? __double2float_rn((double)hp - 0.002) : shy_unq(qn);  // water.h:120-124
      float ceq = r.w * (hp - h2);  // water.h:127-128
      if (ceq < 0.0f) ceq = 0.0f;
      const float edn = ed / (float)nhere;
      const float ex = edn * (ceq - v.y);  // water.h:129-132
      v.y += ex;
      const long long de = -shy_q32(ex);
      add_i64(&a.cq[c].e, de);
      a.own[d] = de;
      const float s0 = v.y;  // water.h:135-136, without the FP64 unit
      v.y = shy_evap_div(v.y, &ev);
      v.x = __ldg(&a.voltab[ag + 1]);
      gn += shy_q32(v.y - s0);  // exact difference (Sterbenz)
      if (out) {  // water.h:139-142
        ++n_oob;
        loss_q += shy_q32(v.y);
        gain_q += gn;
        a.age[d] = -2;
        a.ctr[d] = -1;
        continue;
      }
      a.ctr[d] = arrived_before == 0 ? c2 : -1;  // World::cascade(pos), water.h:151
      a.age[d] = ag + 1;
      a.pos[d] = p;
      a.spd[d] = s;
      a.vs[d] = v;
      a.gain[d] = gn;
    }
    lap(0);
    if (!grid_barrier(a.bar, passed)) { ok = false; break; }
    lap(1);

    // ---- phase C: World::cascade at each claimed cell ----
    // C1: each cascade computes the nine heights it works on; most move
    // nothing (no neighbour starts with excess) and are settled here.  The
    // steep ones go to a queue, which C2 works through one cell per warp after
    // a barrier, so that no warp carries more than its share of them.
    long long sq_c2 = 0;
    int sq_ti = 0, sq_ix = 0, sq_iy = 0;
    float sq_h0 = 0.0f, sq_v[8];
    for (long long d0 = tid - (threadIdx.x & 31); d0 < a.total_drops; d0 += G) {
      // warp-uniform loop, so that the warp can take queue slots together
      const int lane = threadIdx.x & 31;
      const long long d = d0 + lane;
      const long long c2 = d < a.total_drops ? a.ctr[d] : -1;
      const int ti = d < a.total_drops ? a.terr[d] : 0;
      bool steep = false;
      if (c2 >= 0) {
      const Terrain T = TT[ti];
      const int lc = (int)(c2 - T.cell_base);  // < 2^31 cells per terrain
      const int ix = lc / T.ny, iy = lc - ix * T.ny;
      // heights after phase A: fixed point plus the step's erosion.  All nine
      // loads are issued together: a neighbour outside the map reads the
      // centre instead and is masked out.
      longlong2 nv[8];
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        const bool in = !oob(ix + nb_dx(k), iy + nb_dy(k), T.nx, T.ny);
        nv[k] = hq_e(&a.cq[in ? c2 + (long long)nb_dx(k) * T.ny + nb_dy(k) : c2]);
      }
      const longlong2 v0 = hq_e(&a.cq[c2]);
      float sh[8];
#pragma unroll
      for (int k = 0; k < 8; ++k)
        sh[k] = oob(ix + nb_dx(k), iy + nb_dy(k), T.nx, T.ny) ? __int_as_float(0x7f800000)  // never used
                                                              : shy_unq(nv[k].x + nv[k].y);
      const float h0 = shy_unq(v0.x + v0.y);
      // the centre only changes through a transfer, so without any excess to
      // begin with the sequential loop moves nothing
      bool any = false;
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        const float diff = h0 - sh[k];
        const float dist = (nb_dx(k) != 0 && nb_dy(k) != 0) ? sqrtf(2.0f) : 1.0f;
        const float excess = sh[k] >= 0.1f ? fabsf(diff) - dist * P.max_diff : fabsf(diff);
        any |= (sh[k] < __int_as_float(0x7f800000)) && diff != 0.0f && excess > 0.0f;
      }
      a.cmask[d] = 0;
      steep = any;
      if (any) {
        // keep what the queue entry needs until the warp has its slots
        sq_c2 = c2; sq_ti = ti; sq_ix = ix; sq_iy = iy; sq_h0 = h0;
#pragma unroll
        for (int k = 0; k < 8; ++k) sq_v[k] = sh[k];
      }
      }
      const unsigned bal = __ballot_sync(0xffffffffu, steep);
      if (bal) {
        unsigned base = 0;
        if (lane == __ffs(bal) - 1) base = atomicAdd(&a.bar->steep, (unsigned)__popc(bal));
        base = __shfl_sync(0xffffffffu, base, __ffs(bal) - 1);
        if (steep) {
          SteepCell& q = a.steep[base + __popc(bal & ((1u << lane) - 1u))];
          q.c2 = sq_c2;
          q.d = (int)d;
          q.ti = sq_ti;
          q.ix = sq_ix;
          q.iy = sq_iy;
          q.h0 = sq_h0;
#pragma unroll
          for (int k = 0; k < 8; ++k) q.v[k] = sq_v[k];
        }
      }
    }
    lap(2);
    if (!grid_barrier(a.bar, passed)) { ok = false; break; }

    // C2: the steep cascades, each by one whole warp
    {
      const int lane = threadIdx.x & 31;
      const unsigned nsteep = *((volatile unsigned*)&a.bar->steep);
      const long long warp = tid >> 5, nwarps = G >> 5;
      for (long long i = warp; i < nsteep; i += nwarps) {
        const SteepCell& qc = a.steep[i];
        const long long sc2 = qc.c2;
        const int six = qc.ix, siy = qc.iy;
        const float sh0 = qc.h0;
        const Terrain T = TT[qc.ti];
        float v[8];
        int sk[8];
#pragma unroll
        for (int k = 0; k < 8; ++k) {
          v[k] = qc.v[k];
          sk[k] = k;
        }
        // cascade centres of this step in the 5 x 5 block (cells a drop moved
        // to): lane l looks at (dx, dy) = (l / 5 - 2, l % 5 - 2); bit l
        bool is_c = false;
        {
          const int dx = lane < 25 ? lane / 5 - 2 : 0, dy = lane < 25 ? lane % 5 - 2 : 0;
          const bool in = lane < 25 && !oob(six + dx, siy + dy, T.nx, T.ny);
          const int cv = a.cq[in ? sc2 + (long long)dx * T.ny + dy : sc2].cnt[par ^ 1];
          is_c = in && cv > 0;
        }
        const unsigned cen = __ballot_sync(0xffffffffu, is_c);
        // cascades whose 3 x 3 block holds cell (dx, dy): popcount of a window
        auto cover = [&](int dx, int dy) {
          const unsigned row = 7u << (dy + 1);  // 3 bits centred on dy
          const unsigned win = (row << (5 * (dx + 1))) | (row << (5 * (dx + 2))) | (row << (5 * (dx + 3)));
          return __popc(cen & win);
        };
        unsigned kv = 0;  // 4 bits per neighbour
#pragma unroll
        for (int k = 0; k < 8; ++k) kv |= (unsigned)cover(nb_dx(k), nb_dy(k)) << (4 * k);
        const int kc = cover(0, 0);
        sort8(v, sk);
        // the reference's sequential loop (every lane, same values)
        float hcv = sh0;
        float tr[8];
        int mask = 0;
#pragma unroll
        for (int j = 0; j < 8; ++j) {
          tr[j] = 0.0f;
          if (!(v[j] < __int_as_float(0x7f800000))) continue;
          const float diff = hcv - v[j];
          if (diff == 0.0f) continue;
          const int k = sk[j];
          const float dist = (nb_dx(k) != 0 && nb_dy(k) != 0) ? sqrtf(2.0f) : 1.0f;
          // h > 0.1 in double is h >= 0.1f in float (no float lies between)
          const float excess = v[j] >= 0.1f ? fabsf(diff) - dist * P.max_diff : fabsf(diff);
          if (excess <= 0.0f) continue;
          const int kn = (int)((kv >> (4 * k)) & 15u);
          const int kk = kc > kn ? kc : kn;
          float transfer = P.settling * excess / 2.0f;
          if (kk > 1) transfer = transfer / (float)kk;
          if (diff > 0.0f) {
            hcv -= transfer;
            tr[j] = transfer;
          } else {
            hcv += transfer;
            tr[j] = -transfer;
          }
          mask |= 1 << k;
        }
        if (mask) mask |= 256;
        // the fixed-point sums: lane j < 8 the j-th sorted neighbour, lane 8
        // the centre
        float t = 0.0f;
        int kt = 0;
#pragma unroll
        for (int j = 0; j < 8; ++j)
          if (lane == j) {
            t = tr[j];
            kt = sk[j];
          }
        if (lane < 8 && t != 0.0f)
          add_i64(&a.cq[sc2 + (long long)nb_dx(kt) * T.ny + nb_dy(kt)].q, shy_q32(t));
        if (lane == 8 && mask) add_i64(&a.cq[sc2].q, shy_q32(hcv - sh0));
        if (lane == 0) a.cmask[qc.d] = mask;
      }
    }
    lap(2);
    if (!grid_barrier(a.bar, passed)) { ok = false; break; }
    lap(3);

    // ---- phase D: apply, reset counts, retire ----
    if (tid == 0) a.bar->steep = 0;
    // Every drop adds its own erosion to its cell's fixed-point height; the
    // cascades add what they moved.  All integer additions, so the order
    // does not matter.
    unsigned long long retired = 0;
    for (long long d = tid; d < a.total_drops; d += G) {
      const int ag = a.age[d];
      const long long c = a.cell[d];
      const long long c2 = a.ctr[d];
      const long long own = a.own[d];
      const int ti = a.terr[d];
      const int m = c2 >= 0 ? a.cmask[d] : 0;
      if (ag == -1) continue;
      if (c >= 0) {
        if (own != 0) add_i64(&a.cq[c].hq, own);
        a.cq[c].e = 0;
        a.cq[c].cnt[par] = 0;
      }
      if (m) {  // the cells its cascade changed
        const Terrain T = TT[ti];
        for (int k = 0; k < 9; ++k) {
          if (!(m & (1 << (k == 8 ? 8 : k)))) continue;
          const long long x = k == 8 ? c2 : c2 + (long long)nb_dx(k) * T.ny + nb_dy(k);
          const long long q = (long long)atomicExch((unsigned long long*)&a.cq[x].q, 0ull);
          if (q != 0) add_i64(&a.cq[x].hq, q);
        }
      }
      if (ag == -2) {
        a.age[d] = -1;
        a.cell[d] = -1;
        ++retired;
      }
    }
    {
      const unsigned long long s = block_sum_u64(retired);
      if (threadIdx.x == 0 && s) atomicAdd(&a.bar->live, (unsigned long long)(-(long long)s));
    }
    lap(4);
    if (!grid_barrier(a.bar, passed)) { ok = false; break; }
  }
  lap(5);

  // counters
  {
    unsigned long long v;
    v = block_sum_u64(n_steps);   if (threadIdx.x == 0 && v) atomicAdd(&a.st->steps, v);
    v = block_sum_u64(n_oob);     if (threadIdx.x == 0 && v) atomicAdd(&a.st->oob, v);
    v = block_sum_u64(n_drops);   if (threadIdx.x == 0 && v) atomicAdd(&a.st->drops, v);
    v = block_sum_u64(n_skipped); if (threadIdx.x == 0 && v) atomicAdd(&a.st->skipped, v);
    v = block_sum_u64((unsigned long long)gain_q);
    if (threadIdx.x == 0 && v) atomicAdd((unsigned long long*)&a.st->gain_q, v);
    v = block_sum_u64((unsigned long long)loss_q);
    if (threadIdx.x == 0 && v) atomicAdd((unsigned long long*)&a.st->loss_q, v);
  }
  if (timer) {
    for (int i = 0; i < 6; ++i) a.bar->phase_ns[i] += ph[i];
    a.bar->iterations += (unsigned long long)step;
    if (ok && a.bar->live != 0) atomicCAS(&a.bar->error, 0, SHY_ERR_STATE);
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
    r.w = 1.0f + P.entrainment * shy_erff(0.4f * r.z);
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
    bar->steep = 0;
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

int batched_max_grid(shy_world* w, int block) {
  int per_sm = 0;
  if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, lockstep_kernel, block, 0) != cudaSuccess)
    return 0;
  return per_sm * w->sm_count;
}

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
  a.effd = w->effd;
  a.voltab = w->voltab;
  a.ev = shy_evap_make(w->P.evap_rate);
  a.trk = w->trk;
  a.pos = w->dpos;
  a.spd = w->dspd;
  a.vs = w->dvs;
  a.age = w->dage;
  a.gain = w->dgain;
  a.own = w->down;
  a.terr = w->dterr;
  a.cell = w->dcell;
  a.ctr = w->dctr;
  a.cmask = w->dcmask;
  a.steep = w->dsteep;
  a.P = w->P;
  a.st = w->stats;
  a.bar = w->bar;
  a.max_steps = (int)w->P.max_age + 3;

  int grid = w->batch_grid;
  const int maxg = batched_max_grid(w, kLockBlock);
  const int need = (a.total_drops + kLockBlock - 1) / kLockBlock;
  if (grid <= 0 || grid > maxg) grid = maxg;
  if (grid > need) grid = need < 1 ? 1 : need;
  void* args[] = {&a};
  int slot = -1;
  cudaError_t e = timing_begin(w, SHY_KERNEL_DROPS, &slot);
  if (e != cudaSuccess) return e;
  e = cudaLaunchCooperativeKernel((const void*)lockstep_kernel, dim3(grid), dim3(kLockBlock), args, 0,
                                  w->stream);
  if (e != cudaSuccess) return e;
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
  a.effd = b.effd;
  a.voltab = b.voltab;
  a.ev = shy_evap_make(b.P.evap_rate);
  a.trk = b.trk;
  a.pos = b.pos;
  a.spd = b.spd;
  a.vs = b.vs;
  a.age = b.age;
  a.gain = b.gain;
  a.own = b.own;
  a.terr = b.terr;
  a.cell = b.cell;
  a.ctr = b.ctr;
  a.cmask = b.cmask;
  a.steep = b.steep;
  a.P = b.P;
  a.st = b.st;
  a.bar = b.bar;
  a.max_steps = (int)b.P.max_age + 3;
  int per_sm = 0;
  cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, lockstep_kernel, kLockBlock, 0);
  if (e != cudaSuccess) return e;
  int grid = per_sm * b.sm_count;
  const int need = (b.total_drops + kLockBlock - 1) / kLockBlock;
  if (grid > need) grid = need < 1 ? 1 : need;
  void* args[] = {&a};
  e = cudaLaunchCooperativeKernel((const void*)lockstep_kernel, dim3(grid), dim3(kLockBlock), args, 0, stream);
  if (e != cudaSuccess) return e;
  cycle_end_kernel<<<cells_grid(b.cells), 256, 0, stream>>>(b.trk, b.rec, b.track_f, b.cq, b.h, b.cells, b.P,
                                                            b.bar, b.st);
  return cudaGetLastError();
}

cudaError_t launch_heights_to_fixed(shy_world* w) {
  heights_to_fixed_kernel<<<cells_grid(w->cells), 256, 0, w->stream>>>(w->h, w->cq, w->cells);
  return cudaGetLastError();
}

}  // namespace shy
