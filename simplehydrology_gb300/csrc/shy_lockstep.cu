// shy_lockstep.cu -- the batched erosion mode.
//
// One batched cycle is World::erode(drops) (source/world.h:54-88) with all
// drops of every terrain of the world descending at once, one drop per
// thread slot, in lock step.  Step t is three phases separated by grid-wide
// barriers:
//   A  each live drop takes one Drop::descend step (source/water.h:58-156)
//      against the heights after step t-1.  A drop sharing its cell with n-1
//      other live drops exchanges sediment at rate effD / n (n = 1 is the
//      reference).  Height change and the three tracks go to 32.32
//      fixed-point accumulators with integer atomics (one 32-byte sector per
//      cell).  The first drop to claim its new cell runs that cell's cascade.
//   C  World::cascade (source/world.h:90-168) at every claimed cell on the
//      heights as phase A left them; transfers go to fixed-point accumulators.
//      Where the 3 x 3 blocks of k cascades overlap, a pair's transfer is
//      divided by k (the larger count of its two cells), so overlapping
//      cascades together move what one would.
//   D  every changed cell is applied once (the first toucher claims it), the
//      per-cell drop counts move to the next step, finished drops retire.
// Integer sums make every result independent of thread timing: the same
// inputs give the same bits on every run, and oracle/hydro_oracle.cpp
// (Lockstep) restates the schedule on the CPU.
//
// The end-of-cycle kernel converts the tracks to float, applies the lrate
// blend (source/world.h:81-86) and rebuilds the per-cell records.
#include <cooperative_groups.h>

#include "shy_device.cuh"

namespace shy {

namespace {

const int kLockBlock = 256;
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
__device__ __forceinline__ int ld_relaxed_i32(const int* p) {
  int v;
  asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
  return v;
}

// Grid-wide barrier over a monotonically increasing arrival counter.  Every
// wait is bounded: past kBarrierLimitNs the waiter sets bar->abort and every
// later barrier returns false at once, so the kernel always ends.
__device__ bool grid_barrier(GridBar* bar) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    const unsigned long long nb = gridDim.x;
    __threadfence();
    const unsigned long long old = atomicAdd(&bar->arrive, 1ull);
    const unsigned long long target = (old / nb + 1) * nb;
    int ok = 1;
    const unsigned long long t0 = global_ns();
    unsigned sleep = 32;
    while (ld_acquire_u64(&bar->arrive) < target) {
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
      __nanosleep(sleep);
      if (sleep < 256) sleep <<= 1;
    }
    __threadfence();
    s_ok = ok;
  }
  __syncthreads();
  return s_ok != 0;
}

struct LockArgs {
  const Terrain* terrains;
  int n_terrains;
  int total_drops;
  long long cells;
  float* h;
  const float4* rec;
  const float* effd;
  Acc4* acc;
  long long* casc;
  int* cnt;
  int* cover;
  unsigned* stamp;
  float2* pos;
  float2* spd;
  float2* vs;
  int* age;
  double* gain;
  int* terr;
  long long* cell;
  long long* ctr;
  int* cmask;
  shy_params P;
  DevStats* st;
  GridBar* bar;
  int max_steps;
};

__device__ __forceinline__ void add_i64(long long* p, long long v) {
  atomicAdd((unsigned long long*)p, (unsigned long long)v);
}

__device__ __forceinline__ int find_terrain(const Terrain* T, int n, int d) {
  int lo = 0, hi = n - 1;
  while (lo < hi) {
    const int mid = (lo + hi + 1) >> 1;
    if (T[mid].drop_base <= d) lo = mid; else hi = mid - 1;
  }
  return lo;
}

// apply one cell's phase-A and phase-C sums, once per step (first claimer)
__device__ __forceinline__ void apply_cell(const LockArgs& a, long long x, unsigned atag) {
  if (atomicExch(&a.stamp[x], atag) == atag) return;
  const long long e = a.acc[x].e, q = a.casc[x];
  if (e == 0 && q == 0) return;
  a.h[x] = addq(addq(a.h[x], e), q);
  a.acc[x].e = 0;
  a.casc[x] = 0;
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

__global__ void __launch_bounds__(kLockBlock) lockstep_kernel(LockArgs a) {
  const long long G = (long long)gridDim.x * blockDim.x;
  const long long tid = (long long)blockIdx.x * blockDim.x + threadIdx.x;
  const shy_params& P = a.P;
  const unsigned long long cycle = a.bar->cycle;
  const unsigned long long tick0 = a.bar->tick;
  unsigned long long n_steps = 0, n_oob = 0, n_drops = 0, n_skipped = 0;
  long long gain_q = 0, loss_q = 0;

  // spawn (source/world.h:64-74)
  unsigned long long born = 0;
  for (long long d = tid; d < a.total_drops; d += G) {
    const int t = find_terrain(a.terrains, a.n_terrains, (int)d);
    const Terrain T = a.terrains[t];
    int x, y;
    shy_spawn_xy(T.seed, cycle, (unsigned)(d - T.drop_base), T.nx, T.ny, &x, &y);
    const long long c = T.cell_base + (long long)x * T.ny + y;
    a.terr[d] = t;
    a.cell[d] = -1;
    a.ctr[d] = -1;
    if ((double)a.h[c] < 0.1) {  // world.h:71
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
    a.gain[d] = 0.0;
    atomicAdd(&a.cnt[c], 1);
  }
  {
    const unsigned long long s = block_sum_u64(born);
    if (threadIdx.x == 0 && s) atomicAdd(&a.bar->live, s);
  }
  bool ok = grid_barrier(a.bar);

  int step = 0;
  for (; ok && step < a.max_steps; ++step) {
    if (*((volatile unsigned long long*)&a.bar->live) == 0) break;
    const int par = step & 1;
    int* cnt_now = a.cnt + par * a.cells;
    int* cnt_next = a.cnt + (par ^ 1) * a.cells;
    const unsigned ctag = (unsigned)(2ull * (tick0 + (unsigned long long)step));
    const unsigned atag = ctag + 1u;

    // ---- phase A: one descend step per live drop ----
    for (long long d = tid; d < a.total_drops; d += G) {
      const int ag = a.age[d];
      if (ag < 0) continue;
      const Terrain T = a.terrains[a.terr[d]];
      const float* hT = a.h + T.cell_base;
      float2 p = a.pos[d], s = a.spd[d], v = a.vs[d];
      double gn = a.gain[d];
      const int ix = (int)p.x, iy = (int)p.y;
      const long long c = T.cell_base + (long long)ix * T.ny + iy;
      a.cell[d] = c;
      const float3 n = normal_from(PlainHeights{hT, T.nx, T.ny}, ix, iy, T.nx, T.ny, P.map_scale);
      if ((float)ag > P.max_age || v.x < P.min_vol) {  // water.h:74-83
        add_i64(&a.acc[c].e, q32(v.y));
        gain_q += q64(gn);
        a.age[d] = -2;
        a.ctr[d] = -1;
        continue;
      }
      ++n_steps;
      const float4 r = __ldg(&a.rec[c]);
      const float ed = __ldg(&a.effd[c]);
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
      add_i64(&a.acc[c].td, q32(v.x));  // water.h:115-117
      add_i64(&a.acc[c].tmx, q32(v.x * s.x));
      add_i64(&a.acc[c].tmy, q32(v.x * s.y));
      const int jx = (int)p.x, jy = (int)p.y;
      const bool out = oob(jx, jy, T.nx, T.ny);
      const float hc = hT[(long long)ix * T.ny + iy];
      const float h2 = out ? __double2float_rn((double)hc - 0.002) : hT[(long long)jx * T.ny + jy];
      float ceq = r.w * (hc - h2);  // water.h:127-128
      if (ceq < 0.0f) ceq = 0.0f;
      const float edn = ed / (float)cnt_now[c];
      const float ex = edn * (ceq - v.y);  // water.h:129-132
      v.y += ex;
      add_i64(&a.acc[c].e, -q32(ex));
      const float s0 = v.y;  // water.h:135-136
      v.y = evap_div(v.y, P.evap_rate);
      v.x = evap_mul(v.x, P.evap_rate);
      gn += (double)v.y - (double)s0;
      if (out) {  // water.h:139-142
        ++n_oob;
        loss_q += q64((double)v.y);
        gain_q += q64(gn);
        a.age[d] = -2;
        a.ctr[d] = -1;
        continue;
      }
      const long long c2 = T.cell_base + (long long)jx * T.ny + jy;  // water.h:151
      if (atomicExch(&a.stamp[c2], ctag) != ctag) {
        a.ctr[d] = c2;
        // count the cascades whose 3 x 3 block holds each cell
        for (int dx = -1; dx <= 1; ++dx)
          for (int dy = -1; dy <= 1; ++dy)
            if (!oob(jx + dx, jy + dy, T.nx, T.ny)) atomicAdd(&a.cover[c2 + (long long)dx * T.ny + dy], 1);
      } else {
        a.ctr[d] = -1;
      }
      a.age[d] = ag + 1;
      a.pos[d] = p;
      a.spd[d] = s;
      a.vs[d] = v;
      a.gain[d] = gn;
    }
    if (!grid_barrier(a.bar)) { ok = false; break; }

    // ---- phase C: World::cascade at each claimed cell ----
    for (long long d = tid; d < a.total_drops; d += G) {
      const long long c2 = a.ctr[d];
      if (c2 < 0) continue;
      const Terrain T = a.terrains[a.terr[d]];
      const long long lc = c2 - T.cell_base;
      const int ix = (int)(lc / T.ny), iy = (int)(lc - (long long)ix * T.ny);
      int sk[8];
      float sh[8], sd[8];
      int num = 0;
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        const int x = ix + nb_dx(k), y = iy + nb_dy(k);
        if (oob(x, y, T.nx, T.ny)) continue;
        const long long nc = T.cell_base + (long long)x * T.ny + y;
        sk[num] = k;
        sh[num] = addq(a.h[nc], a.acc[nc].e);
        sd[num] = len2((float)nb_dx(k), (float)nb_dy(k));
        ++num;
      }
      for (int i = 1; i < num; ++i) {  // stable insertion sort by height
        const int vk = sk[i];
        const float vh = sh[i], vd = sd[i];
        int j = i;
        while (j > 0 && vh < sh[j - 1]) {
          sk[j] = sk[j - 1];
          sh[j] = sh[j - 1];
          sd[j] = sd[j - 1];
          --j;
        }
        sk[j] = vk;
        sh[j] = vh;
        sd[j] = vd;
      }
      const float h0 = addq(a.h[c2], a.acc[c2].e);
      const int kc = a.cover[c2];
      float hcv = h0;
      int mask = 256;
      for (int i = 0; i < num; ++i) {
        const float diff = hcv - sh[i];
        if (diff == 0.0f) continue;
        const float excess = (double)sh[i] > 0.1 ? fabsf(diff) - sd[i] * P.max_diff : fabsf(diff);
        if (excess <= 0.0f) continue;
        const int k = sk[i];
        const long long nc = c2 + (long long)nb_dx(k) * T.ny + nb_dy(k);
        // centres whose blocks overlap share the pair: divide by the larger
        // cover count (1 where cascades do not overlap: the reference)
        const int kn = a.cover[nc];
        const float transfer = P.settling * excess / 2.0f / (float)(kc > kn ? kc : kn);
        if (diff > 0.0f) {
          hcv -= transfer;
          add_i64(&a.casc[nc], q32(transfer));
        } else {
          hcv += transfer;
          add_i64(&a.casc[nc], -q32(transfer));
        }
        mask |= 1 << k;
      }
      add_i64(&a.casc[c2], q32(hcv - h0));
      a.cmask[d] = mask;
    }
    if (!grid_barrier(a.bar)) { ok = false; break; }

    // ---- phase D: apply, move counts, retire ----
    unsigned long long retired = 0;
    for (long long d = tid; d < a.total_drops; d += G) {
      const int ag = a.age[d];
      if (ag == -1) continue;
      const long long c = a.cell[d];
      if (c >= 0) {
        apply_cell(a, c, atag);
        cnt_now[c] = 0;
      }
      const long long c2 = a.ctr[d];
      if (c2 >= 0) {
        const Terrain T = a.terrains[a.terr[d]];
        const int m = a.cmask[d];
#pragma unroll
        for (int k = 0; k < 8; ++k)
          if (m & (1 << k)) apply_cell(a, c2 + (long long)nb_dx(k) * T.ny + nb_dy(k), atag);
        apply_cell(a, c2, atag);
        const long long lc = c2 - T.cell_base;
        const int ix = (int)(lc / T.ny), iy = (int)(lc - (long long)ix * T.ny);
        for (int dx = -1; dx <= 1; ++dx)
          for (int dy = -1; dy <= 1; ++dy)
            if (!oob(ix + dx, iy + dy, T.nx, T.ny)) a.cover[c2 + (long long)dx * T.ny + dy] = 0;
      }
      if (ag == -2) {
        a.age[d] = -1;
        a.cell[d] = -1;
        ++retired;
      } else {
        const Terrain T = a.terrains[a.terr[d]];
        const float2 p = a.pos[d];
        atomicAdd(&cnt_next[T.cell_base + (long long)(int)p.x * T.ny + (int)p.y], 1);
      }
    }
    {
      const unsigned long long s = block_sum_u64(retired);
      if (threadIdx.x == 0 && s) atomicAdd(&a.bar->live, (unsigned long long)(-(long long)s));
    }
    if (!grid_barrier(a.bar)) { ok = false; break; }
  }

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
  if (blockIdx.x == 0 && threadIdx.x == 0) {
    a.bar->tick = tick0 + (unsigned long long)step + 1ull;
    if (ok && a.bar->live != 0) atomicCAS(&a.bar->error, 0, SHY_ERR_STATE);
  }
}

// End of a batched cycle: tracks to float, lrate blend (source/world.h:81-86),
// records for the next cycle, accumulators cleared.
__global__ void cycle_end_kernel(Acc4* __restrict__ acc, float4* __restrict__ rec,
                                 float* __restrict__ track_f, long long cells, shy_params P,
                                 GridBar* bar, DevStats* st) {
  const float a = 1.0f - P.lrate, b = P.lrate;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < cells;
       i += (long long)gridDim.x * blockDim.x) {
    const Acc4 q = acc[i];
    const float fd = unq(q.td), fx = unq(q.tmx), fy = unq(q.tmy);
    track_f[i] = fd;
    track_f[cells + i] = fx;
    track_f[2 * cells + i] = fy;
    float4 r = rec[i];
    r.z = a * r.z + b * fd;
    r.x = a * r.x + b * fx;
    r.y = a * r.y + b * fy;
    r.w = 1.0f + P.entrainment * shy_erff(0.4f * r.z);
    rec[i] = r;
    Acc4 z;
    z.e = q.e;  // zero after a completed cycle; kept for a consistency check
    z.td = 0;
    z.tmx = 0;
    z.tmy = 0;
    acc[i] = z;
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
// which at least one cell was visited this cycle, from `hin` to `hout`.
__global__ void relax_kernel(const Terrain* __restrict__ terrains, int n_terrains,
                             const float* __restrict__ hin, float* __restrict__ hout,
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
    double sum = 0.0;
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
      const float excess = (double)lo > 0.1 ? fabsf(diff) - dist * P.max_diff : fabsf(diff);
      if (excess <= 0.0f) continue;
      const float transfer = P.cascade_weight * (P.settling * excess / 2.0f);
      sum += diff > 0.0f ? -(double)transfer : (double)transfer;
    }
    hout[i] = __double2float_rn((double)hc + sum);
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
  a.rec = w->rec;
  a.effd = w->effd;
  a.acc = w->acc;
  a.casc = w->casc;
  a.cnt = w->cnt;
  a.cover = w->cover;
  a.stamp = w->stamp;
  a.pos = w->dpos;
  a.spd = w->dspd;
  a.vs = w->dvs;
  a.age = w->dage;
  a.gain = w->dgain;
  a.terr = w->dterr;
  a.cell = w->dcell;
  a.ctr = w->dctr;
  a.cmask = w->dcmask;
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
  cycle_end_kernel<<<cells_grid(w->cells), 256, 0, w->stream>>>(w->acc, w->rec, w->track_f, w->cells,
                                                                w->P, w->bar, w->stats);
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if ((e = timing_end(w, slot)) != cudaSuccess) return e;

  for (int p = 0; p < w->P.cascade_passes; ++p) {
    if ((e = timing_begin(w, SHY_KERNEL_CASCADE, &slot)) != cudaSuccess) return e;
    relax_kernel<<<cells_grid(w->cells), 256, 0, w->stream>>>(w->dterrains, (int)w->terrains.size(),
                                                              w->h, w->relax, w->track_f, w->cells, w->P);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    e = cudaMemcpyAsync(w->h, w->relax, sizeof(float) * w->cells, cudaMemcpyDeviceToDevice, w->stream);
    if (e != cudaSuccess) return e;
    if ((e = timing_end(w, slot)) != cudaSuccess) return e;
  }
  return cudaSuccess;
}

}  // namespace shy
