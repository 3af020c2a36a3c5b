// shy_surrogate.cu -- device side of the learned warm-start surrogate: the
// convolutions of a small U-Net as BF16 implicit GEMMs on the tensor cores
// (tcgen05.mma, FP32 accumulators in tensor memory), their weight and input
// gradients, and the elementwise pieces of training and inference.
//
// Convolution forward (conv_fwd_kernel).  One CTA of 128 threads computes a
// tile of M = 128 output pixels (consecutive in (b, y, x) order) by N output
// channels (16..128).  K = taps x cin is walked one tap and one channel chunk
// (kc = 16, 32 or 64) at a time.  For each chunk the CTA stages A (the input
// pixels shifted by the tap, zero outside the image) and B (weights
// [cout][tap][cin]) in shared memory, in the no-swizzle K-major core-matrix
// layout: a core matrix is 8 rows x 16 bytes stored as 128 contiguous bytes;
// core matrices adjacent along K are 128 B apart (the descriptor's leading
// byte offset) and 8-row groups kc * 16 B apart (its stride byte offset).
// Stages are double-buffered: thread 0 issues kc / 16 MMAs of K = 16 on a
// stage and commits them to the stage's mbarrier, and the stage is filled
// again, two chunks later, once that barrier has completed.  So the loads of
// one chunk overlap the MMAs of the previous one.  The epilogue reads the
// accumulator with tcgen05.ld (warp w owns TMEM lanes 32w..32w+31, the tile's
// pixels 32w..32w+31), adds the bias and writes f32 and/or bf16 GELU output.
//
// Input gradient: the same kernel on the output gradient, with the weights
// rotated by 180 degrees and transposed (shy_sg_weight_prep).
//
// Weight gradient (conv_wgrad_kernel): a GEMM with M = 128 rows of
// (tap, cin), N = a cout tile and K = pixels in chunks of 64.  Both operands
// are K-major in shared memory but pixel-major in HBM, so the threads stage
// them transposed (a 16-byte load of 8 channels, 8 two-byte stores).  The
// pixel range is split over CTAs; each adds its partial sums to the f32
// weight gradient with atomics.
//
// Every wait on an mbarrier is bounded (2 s); a CTA that gives up records
// SHY_ERR_TIMEOUT, skips its epilogue and still frees its tensor memory.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <mutex>
#include <cuda_bf16.h>

#include "../../include/shy_surrogate.h"
#include "shy_internal.h"

namespace shy {

namespace {

constexpr int kTileM = 128;     // MMA M: pixels (forward) or weight rows (wgrad)
constexpr int kThreads = 128;   // one warpgroup: warp w reads TMEM lanes 32w..32w+31
constexpr int kWgradK = 64;     // pixels per weight-gradient chunk
constexpr unsigned long long kWaitLimitNs = 2000000000ull;
constexpr int kSmemPerSm = 233472;  // shared memory per SM (228 KiB)
constexpr int kSmemReservedPerCta = 1024;

__device__ int g_sg_status;

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ unsigned long long now_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}

__device__ __forceinline__ bool mbar_try(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
      "selp.u32 %0, 1, 0, p;\n\t}"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}

// Waits until the phase of `bar` with parity `parity` has completed; gives up
// after `limit_ns`.
__device__ bool mbar_wait(uint64_t* bar, uint32_t parity, unsigned long long limit_ns = kWaitLimitNs) {
  if (mbar_try(bar, parity)) return true;
  const unsigned long long t0 = now_ns();
  while (!mbar_try(bar, parity))
    if (now_ns() - t0 > limit_ns) return false;
  return true;
}

__device__ __forceinline__ void tc_fence_before() {
  asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
  asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}
// Makes this thread's shared-memory stores visible to the tensor cores.
__device__ __forceinline__ void fence_async_smem() {
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
}

// Warp-wide: allocate `cols` TMEM columns (a power of two >= 32); the base
// address lands in *slot.
__device__ __forceinline__ void tmem_alloc(uint32_t* slot, uint32_t cols) {
  asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                   smem_u32(slot)),
               "r"(cols)
               : "memory");
  asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
}
__device__ __forceinline__ void tmem_free(uint32_t base, uint32_t cols) {
  asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(base), "r"(cols)
               : "memory");
}

// Shared-memory matrix descriptor, no swizzle, K-major.
__device__ __forceinline__ uint64_t smem_desc(uint32_t addr, uint32_t lbo, uint32_t sbo) {
  return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)(lbo >> 4) << 16) |
         ((uint64_t)(sbo >> 4) << 32) | (1ull << 46);
}

// Instruction descriptor of kind::f16: F32 accumulator (bits 4-5 = 1), BF16
// A and B (bits 7-9, 10-12 = 1), both K-major, N >> 3 at bit 17, M >> 4 at
// bit 24, M = 128.
__host__ __device__ constexpr uint32_t idesc_bf16_m128(int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) |
         ((uint32_t)(kTileM >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t d, uint64_t a, uint64_t b, uint32_t idesc,
                                         uint32_t accumulate) {
  asm volatile(
      "{\n\t.reg .pred p;\n\t"
      "setp.ne.b32 p, %4, 0;\n\t"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d),
      "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
      : "memory");
}

// Arrives once on `bar` when every MMA this thread issued so far is done.
__device__ __forceinline__ void mma_commit(uint64_t* bar) {
  asm volatile(
      "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
          smem_u32(bar))
      : "memory");
}

// Warp-wide: 8 consecutive f32 columns of this warp's 32 TMEM lanes (one
// lane per thread); the wait is in the same statement so that no use of
// the registers can be scheduled before the load has landed.
__device__ __forceinline__ void tmem_ld8(uint32_t taddr, float v[8]) {
  uint32_t r0, r1, r2, r3, r4, r5, r6, r7;
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0, %1, %2, %3, %4, %5, %6, %7}, [%8];\n\t"
      "tcgen05.wait::ld.sync.aligned;"
      : "=r"(r0), "=r"(r1), "=r"(r2), "=r"(r3), "=r"(r4), "=r"(r5), "=r"(r6), "=r"(r7)
      : "r"(taddr)
      : "memory");
  v[0] = __uint_as_float(r0);
  v[1] = __uint_as_float(r1);
  v[2] = __uint_as_float(r2);
  v[3] = __uint_as_float(r3);
  v[4] = __uint_as_float(r4);
  v[5] = __uint_as_float(r5);
  v[6] = __uint_as_float(r6);
  v[7] = __uint_as_float(r7);
}

__device__ __forceinline__ float gelu(float z) {
  return 0.5f * z * (1.0f + erff(z * 0.70710678118654752f));
}
__device__ __forceinline__ float gelu_grad(float z) {
  const float cdf = 0.5f * (1.0f + erff(z * 0.70710678118654752f));
  const float pdf = 0.39894228040143268f * expf(-0.5f * z * z);
  return cdf + z * pdf;
}

__device__ __forceinline__ uint32_t pack_bf16(float lo, float hi) {
  const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
  return *reinterpret_cast<const uint32_t*>(&v);
}

__device__ __forceinline__ float bf16_lo(uint32_t w) { return __uint_as_float(w << 16); }
__device__ __forceinline__ float bf16_hi(uint32_t w) { return __uint_as_float(w & 0xFFFF0000u); }

// Epilogue of the convolutions: 8 accumulator columns of one pixel, plus
// bias, to f32 and/or bf16 (GELU'd) outputs.
template <class P>
__device__ __forceinline__ void store_out8(const P& p, long long q, int n, float v[8]) {
  if (p.bias)
    for (int j = 0; j < 8; ++j) v[j] += __ldg(p.bias + n + j);
  if (p.z) {
    float4* zp = reinterpret_cast<float4*>(p.z + q * p.zs + p.zo + n);
    zp[0] = make_float4(v[0], v[1], v[2], v[3]);
    zp[1] = make_float4(v[4], v[5], v[6], v[7]);
  }
  if (p.a) {
    if (p.act == SHY_SG_ACT_GELU)
      for (int j = 0; j < 8; ++j) v[j] = gelu(v[j]);
    uint4 o;
    o.x = pack_bf16(v[0], v[1]);
    o.y = pack_bf16(v[2], v[3]);
    o.z = pack_bf16(v[4], v[5]);
    o.w = pack_bf16(v[6], v[7]);
    *reinterpret_cast<uint4*>(p.a + q * p.as + p.ao + n) = o;
  }
}

// The epilogue of 8 columns of one pixel.  In input-gradient mode (p.gz
// set) the columns are the gradient of a GELU layer's output:
// dz = bf16(v * gelu'(z_prev)) goes to p.a.  Otherwise store_out8.
template <class P>
__device__ __forceinline__ void epilogue8(const P& p, bool valid, long long q, int n, float v[8]) {
  if (!valid) return;
  if (!p.gz) {
    store_out8(p, q, n, v);
    return;
  }
  float g[8];
  {
    const float4* zp = reinterpret_cast<const float4*>(p.gz + q * p.gzs + p.gzo + n);
    const float4 z0 = zp[0], z1 = zp[1];
    const float zv[8] = {z0.x, z0.y, z0.z, z0.w, z1.x, z1.y, z1.z, z1.w};
#pragma unroll
    for (int j = 0; j < 8; ++j) g[j] = __bfloat162float(__float2bfloat16_rn(v[j] * gelu_grad(zv[j])));
    uint4 o;
    o.x = pack_bf16(g[0], g[1]);
    o.y = pack_bf16(g[2], g[3]);
    o.z = pack_bf16(g[4], g[5]);
    o.w = pack_bf16(g[6], g[7]);
    *reinterpret_cast<uint4*>(p.a + q * p.as + p.ao + n) = o;
  }
}

struct ConvFwd {
  const __nv_bfloat16* x;
  const __nv_bfloat16* w;
  const float* bias;
  float* z;
  __nv_bfloat16* a;
  const float* gz;
  int batch, h, w_, cin, cout, ks;
  int xs, zs, zo, as, ao, act, gzs, gzo;
  int ntile, kc, tmem_cols;
};

__global__ void __launch_bounds__(kThreads) conv_fwd_kernel(const ConvFwd p) {
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ uint64_t bars[3];
  __shared__ uint32_t tmem_slot;
  const int tid = threadIdx.x, warp = tid >> 5;
  const long long hw = (long long)p.h * p.w_;
  const long long npix = (long long)p.batch * hw;
  const long long q = (long long)blockIdx.x * kTileM + tid;  // this thread's output pixel
  const bool valid = q < npix;
  int qb = 0, qy = 0, qx = 0;
  if (valid) {
    qb = (int)(q / hw);
    const long long r = q - (long long)qb * hw;
    qy = (int)(r / p.w_);
    qx = (int)(r - (long long)qy * p.w_);
  }
  const int n0 = blockIdx.y * p.ntile;
  const uint32_t sbo = (uint32_t)p.kc * 16;
  const uint32_t a_bytes = (uint32_t)kTileM * p.kc * 2, b_bytes = (uint32_t)p.ntile * p.kc * 2;
  const uint32_t stage_bytes = a_bytes + b_bytes;

  if (warp == 0) tmem_alloc(&tmem_slot, p.tmem_cols);
  if (tid == 0) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    mbar_init(&bars[2], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;

  const int taps = p.ks * p.ks, half = p.ks >> 1;
  const int nchunk = p.cin / p.kc;
  const int iters = taps * nchunk;
  const int vecs = p.kc >> 3;
  const long long wrow = (long long)taps * p.cin;
  const uint32_t idesc = idesc_bf16_m128(p.ntile);
  bool failed = false;
  for (int it = 0; it < iters; ++it) {
    const int s = it & 1;
    uint8_t* sa = smem + s * stage_bytes;
    uint8_t* sb = sa + a_bytes;
    int fail = 0;
    if (it >= 2 && !mbar_wait(&bars[s], (uint32_t)((it >> 1) - 1) & 1u)) fail = 1;
    const int tap = it / nchunk, c0 = (it - tap * nchunk) * p.kc;
    const int dy = tap / p.ks - half, dx = tap % p.ks - half;
    {
      const int yy = qy + dy, xx = qx + dx;
      const bool in = valid && yy >= 0 && yy < p.h && xx >= 0 && xx < p.w_;
      const uint4* src =
          reinterpret_cast<const uint4*>(p.x + (((long long)qb * p.h + yy) * p.w_ + xx) * p.xs + c0);
      uint8_t* dst = sa + (tid >> 3) * sbo + (tid & 7) * 16;
      for (int j = 0; j < vecs; ++j) {
        const uint4 v = in ? __ldg(src + j) : make_uint4(0u, 0u, 0u, 0u);
        *reinterpret_cast<uint4*>(dst + j * 128) = v;
      }
    }
    if (tid < p.ntile) {
      const uint4* src =
          reinterpret_cast<const uint4*>(p.w + (long long)(n0 + tid) * wrow + (long long)tap * p.cin + c0);
      uint8_t* dst = sb + (tid >> 3) * sbo + (tid & 7) * 16;
      for (int j = 0; j < vecs; ++j) *reinterpret_cast<uint4*>(dst + j * 128) = __ldg(src + j);
    }
    fence_async_smem();
    if (__syncthreads_or(fail)) {
      failed = true;
      break;
    }
    if (tid == 0) {
      tc_fence_after();
      const uint32_t a0 = smem_u32(sa), b0 = smem_u32(sb);
      for (int kk = 0; kk < (p.kc >> 4); ++kk)
        mma_bf16(tmem, smem_desc(a0 + kk * 256, 128, sbo), smem_desc(b0 + kk * 256, 128, sbo), idesc,
                 (it | kk) != 0);
      mma_commit(&bars[s]);
    }
  }
  if (tid == 0) mma_commit(&bars[2]);
  const bool done = mbar_wait(&bars[2], 0);
  const bool ok = __syncthreads_and(done && !failed) != 0;
  if (ok) {
    tc_fence_after();
    const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16);
    for (int nc = 0; nc < p.ntile; nc += 8) {
      float v[8];
      tmem_ld8(lane_base + (uint32_t)nc, v);
      epilogue8(p, valid, q, n0 + nc, v);
    }
  } else if (tid == 0) {
    atomicCAS(&g_sg_status, 0, SHY_ERR_TIMEOUT);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tmem_free(tmem, p.tmem_cols);
  }
}

// ---------------------------------------------------------------------------
// Convolution forward with TMA staging (conv_tma_kernel).
//
// The same GEMM as conv_fwd_kernel, but the tile is 8 x 16 pixels of one
// image and its operands arrive by TMA: A is a box of kc channels x 16 x 8
// pixels of the input at the tap's offset (the tensor map's zero fill gives
// the padding at the image border), B a box of kc x ntile weights.  Each
// box lands as rows of kc * 2 bytes, swizzled by the TMA in the pattern the
// MMA's descriptor names (128-, 64- or 32-byte swizzle for kc = 64, 32, 16;
// 8-row groups 8 * kc * 2 bytes apart).  Thread 0 runs a pipeline of 2..8
// pipeline: loads run stages - 1 chunks ahead of the MMAs, each stage's
// "full" barrier completes on the loads' byte count and its "empty" barrier
// on the commit of the MMAs that read it.  All 128 threads then read the
// accumulator for the epilogue.
constexpr int kMaxStages = 8;
constexpr int kTileH = 8, kTileW = 16;

struct ConvTma {
  const float* bias;
  float* z;
  __nv_bfloat16* a;
  const float* gz;  // input-gradient mode: the previous layer's pre-activation (else NULL)
  int batch, h, w_, cin, cout, ks;
  int zs, zo, as, ao, act, gzs, gzo;
  int ntile, kc, tmem_cols, tiles_w, tiles_h, stages, mt;  // mt: 128-pixel sub-tiles (1 or 2)
  int tap_rows;  // taps per stage: 3 (one column of a 3x3 kernel, one taller input box) or 1
  uint32_t a_bytes, b_bytes, stage_bytes, layout;
  uint32_t a_box, b_box;  // bytes of the input box and of one weight box (b_bytes: all weight boxes)
  unsigned long long stall_ns;  // test hook: first wait on a barrier nothing arrives at, this long
};

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void tma_load_4d(uint32_t dst, const CUtensorMap* map, int c0, int c1, int c2, int c3,
                                            uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.4d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
      "[%6];" ::"r"(dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(c2), "r"(c3), "r"(smem_u32(bar))
      : "memory");
}

__device__ __forceinline__ void tma_load_2d(uint32_t dst, const CUtensorMap* map, int c0, int c1, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          dst),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(c0), "r"(c1), "r"(smem_u32(bar))
      : "memory");
}

// Shared-memory matrix descriptor, K-major, swizzled: `layout` 2, 4 or 6
// (128-, 64-, 32-byte swizzle), `sbo` the distance between 8-row groups.
__device__ __forceinline__ uint64_t smem_desc_sw(uint32_t addr, uint32_t sbo, uint32_t layout) {
  return (uint64_t)((addr & 0x3FFFFu) >> 4) | (1ull << 16) | ((uint64_t)(sbo >> 4) << 32) | (1ull << 46) |
         ((uint64_t)layout << 61);
}

// Shared-memory matrix descriptor, MN-major, swizzled: `lbo` the distance
// between blocks of one swizzle width along M (or N), `sbo` between 8-row
// groups along K.
__device__ __forceinline__ uint64_t smem_desc_mn(uint32_t addr, uint32_t lbo, uint32_t sbo, uint32_t layout) {
  return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)(lbo >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) |
         (1ull << 46) | ((uint64_t)layout << 61);
}

__global__ void __launch_bounds__(kThreads) conv_tma_kernel(const __grid_constant__ CUtensorMap map_x,
                                                           const __grid_constant__ CUtensorMap map_w,
                                                           const ConvTma p) {
  extern __shared__ uint8_t smem_raw[];
  __shared__ uint64_t full[kMaxStages], empty[kMaxStages], done, never;
  __shared__ uint32_t tmem_slot;
  __shared__ int s_fail;
  const uint32_t base = (smem_u32(smem_raw) + 1023u) & ~1023u;
  const int tid = threadIdx.x, warp = tid >> 5;
  int t = blockIdx.x;
  const int tx = t % p.tiles_w;
  t /= p.tiles_w;
  const int ty = t % p.tiles_h, b = t / p.tiles_h;
  const int x0 = tx * kTileW, y0 = ty * kTileH * p.mt;
  const int n0 = blockIdx.y * p.ntile;

  if (warp == 0) tmem_alloc(&tmem_slot, p.tmem_cols);
  if (tid == 0) {
    for (int s = 0; s < p.stages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(&done, 1);
    mbar_init(&never, 1);  // nothing arrives here: the bounded-wait test hook waits on it
    s_fail = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;
  const uint32_t sub_bytes = (uint32_t)kTileM * p.kc * 2;  // one 128-pixel sub-tile of A

  if (tid == 0) {
    const int taps = p.ks * p.ks, half = p.ks >> 1;
    const int nchunk = p.cin / p.kc, iters = (taps / p.tap_rows) * nchunk;
    const uint32_t idesc = idesc_bf16_m128(p.ntile);
    const uint32_t sbo = 16u * p.kc;
    const int S = p.stages;
    // iteration it: channel chunk it % nchunk of tap group it / nchunk; with
    // tap_rows = 3 a group is one column kx of the 3x3 kernel: one input box
    // two rows taller than the tile, and the weights of taps (0, kx), (1, kx),
    // (2, kx)
    auto issue = [&](int it) {
      const int s = it % S;
      const int grp = it / nchunk, c0 = (it - grp * nchunk) * p.kc;
      const uint32_t sa = base + s * p.stage_bytes;
      mbar_expect_tx(&full[s], p.a_box + p.b_bytes);
      if (p.tap_rows == 3) {
        tma_load_4d(sa, &map_x, c0, x0 + grp - 1, y0 - 1, b, &full[s]);
        for (int r = 0; r < 3; ++r)
          tma_load_2d(sa + p.a_bytes + r * p.b_box, &map_w, (r * 3 + grp) * p.cin + c0, n0, &full[s]);
      } else {
        const int dy = grp / p.ks - half, dx = grp % p.ks - half;
        tma_load_4d(sa, &map_x, c0, x0 + dx, y0 + dy, b, &full[s]);
        tma_load_2d(sa + p.a_bytes, &map_w, grp * p.cin + c0, n0, &full[s]);
      }
    };
    int issued = 0, consumed = 0;
    // the test hook: a wait that runs out before anything is issued
    bool fail = p.stall_ns != 0 && !mbar_wait(&never, 0, p.stall_ns);
    for (; !fail && issued < S - 1 && issued < iters; ++issued) issue(issued);
    for (int it = 0; !fail && it < iters; ++it) {
      const int s = it % S;
      if (!mbar_wait(&full[s], (uint32_t)(it / S) & 1u)) {
        fail = true;
        break;
      }
      consumed = it + 1;
      tc_fence_after();
      const uint32_t sa = base + s * p.stage_bytes, sb = sa + p.a_bytes;
      // each 128-pixel sub-tile has its own accumulator (ntile columns apart)
      // and shares the stage's weights; tap row r of a column group reads the
      // input box from row r of the tile (16 pixel rows, two swizzle atoms,
      // further on)
      for (int kk = 0; kk < (p.kc >> 4); ++kk)
        for (int r = 0; r < p.tap_rows; ++r)
          for (int u = 0; u < p.mt; ++u)
            mma_bf16(tmem + (uint32_t)(u * p.ntile),
                     smem_desc_sw(sa + u * sub_bytes + r * 16u * 2u * p.kc + kk * 32, sbo, p.layout),
                     smem_desc_sw(sb + r * p.b_box + kk * 32, sbo, p.layout), idesc, (it | kk | r) != 0);
      mma_commit(&empty[s]);
      if (issued < iters) {
        const int s2 = issued % S;
        if (issued >= S && !mbar_wait(&empty[s2], (uint32_t)(issued / S - 1) & 1u)) {
          fail = true;
          break;
        }
        issue(issued);
        ++issued;
      }
    }
    // after a failure, wait (bounded) for loads still landing in this CTA's memory
    for (int it = consumed; it < issued; ++it) mbar_wait(&full[it % S], (uint32_t)(it / S) & 1u);
    mma_commit(&done);
    if (fail) s_fail = 1;
  }
  const bool fin = mbar_wait(&done, 0);
  const bool ok = __syncthreads_and(fin) != 0 && s_fail == 0;
  if (ok) {
    tc_fence_after();
    for (int u = 0; u < p.mt; ++u) {
      const int y = y0 + u * kTileH + (tid >> 4), x = x0 + (tid & 15);
      const bool valid = y < p.h && x < p.w_;
      const long long q = ((long long)b * p.h + y) * p.w_ + x;
      const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)(u * p.ntile);
      for (int nc = 0; nc < p.ntile; nc += 8) {
        float v[8];
        tmem_ld8(lane_base + (uint32_t)nc, v);
        epilogue8(p, valid, q, n0 + nc, v);
      }
    }
  } else if (tid == 0) {
    atomicCAS(&g_sg_status, 0, SHY_ERR_TIMEOUT);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tmem_free(tmem, p.tmem_cols);
  }
}

// ---------------------------------------------------------------------------
// Persistent, warp-specialised convolution (conv_ws_kernel).
//
// The GEMM of conv_tma_kernel with one CTA per SM walking the tiles
// t = blockIdx.x, + gridDim.x, ...  Warp 4 (one lane) issues the TMA loads
// into a ring of stages that runs on from tile to tile; warp 5 (one lane)
// issues the MMAs into one of two accumulators in tensor memory, alternating
// by tile; warps 0-3 read the other accumulator back and store it, so a
// tile's epilogue runs under the next tile's loads and MMAs.  Barriers:
// full / empty per stage (TMA bytes / MMA commit), acc_full per accumulator
// (MMA commit), acc_empty per accumulator (the 128 epilogue threads).  Every
// wait is bounded; a role that gives up raises an abort flag the others poll,
// and the CTA still waits for its own loads and frees its tensor memory.
constexpr int kWsThreads = 192;

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
  asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// mbar_wait that also gives up when *abort is raised, and raises it on timeout.
__device__ bool mbar_wait_abort(uint64_t* bar, uint32_t parity, volatile int* abort) {
  if (mbar_try(bar, parity)) return true;
  const unsigned long long t0 = now_ns();
  while (!mbar_try(bar, parity)) {
    if (*abort) return false;
    if (now_ns() - t0 > kWaitLimitNs) {
      *abort = 1;
      return false;
    }
  }
  return true;
}

__global__ void __launch_bounds__(kWsThreads, 1) conv_ws_kernel(const __grid_constant__ CUtensorMap map_x,
                                                               const __grid_constant__ CUtensorMap map_w,
                                                               const ConvTma p) {
  extern __shared__ uint8_t smem_raw[];
  __shared__ uint64_t full[kMaxStages], empty[kMaxStages], accf[2], acce[2], done;
  __shared__ uint32_t tmem_slot;
  __shared__ int s_abort, s_issued, s_consumed;
  const uint32_t base = (smem_u32(smem_raw) + 1023u) & ~1023u;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int n_tiles = p.cout / p.ntile;
  const int total = p.batch * p.tiles_h * p.tiles_w * n_tiles;
  const int S = p.stages;
  volatile int* abort = &s_abort;

  if (warp == 0) tmem_alloc(&tmem_slot, p.tmem_cols);
  if (tid == 0) {
    for (int s = 0; s < S; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    for (int a = 0; a < 2; ++a) {
      mbar_init(&accf[a], 1);
      mbar_init(&acce[a], 128);
    }
    mbar_init(&done, 1);
    s_abort = 0;
    s_issued = 0;
    s_consumed = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;
  const int taps = p.ks * p.ks, half = p.ks >> 1;
  const int nchunk = p.cin / p.kc, iters = taps * nchunk;
  const uint32_t acc_cols = (uint32_t)(p.mt * p.ntile);
  const uint32_t sub_bytes = (uint32_t)kTileM * p.kc * 2;
  // tile t: output-channel tile t % n_tiles of pixel tile t / n_tiles
  auto decode = [&](int t, int& b, int& x0, int& y0, int& n0) {
    n0 = (t % n_tiles) * p.ntile;
    int r = t / n_tiles;
    x0 = (r % p.tiles_w) * kTileW;
    r /= p.tiles_w;
    y0 = (r % p.tiles_h) * kTileH * p.mt;
    b = r / p.tiles_h;
  };

  if (warp == 4) {
    if (lane == 0) {
      int g = 0;
      for (int t = blockIdx.x; t < total && !*abort; t += gridDim.x) {
        int b, x0, y0, n0;
        decode(t, b, x0, y0, n0);
        bool ok = true;
        for (int it = 0; it < iters; ++it) {
          const int s = g % S;
          if (g >= S && !mbar_wait_abort(&empty[s], (uint32_t)(g / S - 1) & 1u, abort)) {
            ok = false;
            break;
          }
          const int tap = it / nchunk, c0 = (it - tap * nchunk) * p.kc;
          const uint32_t sa = base + s * p.stage_bytes;
          mbar_expect_tx(&full[s], p.a_box + p.b_bytes);
          tma_load_4d(sa, &map_x, c0, x0 + tap % p.ks - half, y0 + tap / p.ks - half, b, &full[s]);
          tma_load_2d(sa + p.a_bytes, &map_w, tap * p.cin + c0, n0, &full[s]);
          ++g;
        }
        if (!ok) break;
      }
      s_issued = g;
    }
  } else if (warp == 5) {
    if (lane == 0) {
      const uint32_t idesc = idesc_bf16_m128(p.ntile);
      const uint32_t sbo = 16u * p.kc;
      int g = 0, j = 0;
      for (int t = blockIdx.x; t < total && !*abort; t += gridDim.x, ++j) {
        const int a = j & 1;
        if (j >= 2 && !mbar_wait_abort(&acce[a], (uint32_t)(j / 2 - 1) & 1u, abort)) break;
        tc_fence_after();
        const uint32_t d0 = tmem + (uint32_t)a * acc_cols;
        bool ok = true;
        for (int it = 0; it < iters; ++it) {
          const int s = g % S;
          if (!mbar_wait_abort(&full[s], (uint32_t)(g / S) & 1u, abort)) {
            ok = false;
            break;
          }
          tc_fence_after();
          const uint32_t sa = base + s * p.stage_bytes, sb = sa + p.a_bytes;
          for (int kk = 0; kk < (p.kc >> 4); ++kk)
            for (int u = 0; u < p.mt; ++u)
              mma_bf16(d0 + (uint32_t)(u * p.ntile), smem_desc_sw(sa + u * sub_bytes + kk * 32, sbo, p.layout),
                       smem_desc_sw(sb + kk * 32, sbo, p.layout), idesc, (it | kk) != 0);
          mma_commit(&empty[s]);
          ++g;
        }
        if (!ok) break;
        mma_commit(&accf[a]);
      }
      s_consumed = g;
      mma_commit(&done);
    }
  } else {
    // epilogue: warp w reads TMEM lanes 32w..32w+31, the tile rows of its threads
    int j = 0;
    for (int t = blockIdx.x; t < total; t += gridDim.x, ++j) {
      const int a = j & 1;
      if (!__all_sync(0xFFFFFFFFu, mbar_wait_abort(&accf[a], (uint32_t)(j / 2) & 1u, abort))) break;
      tc_fence_after();
      int b, x0, y0, n0;
      decode(t, b, x0, y0, n0);
      for (int u = 0; u < p.mt; ++u) {
        const int y = y0 + u * kTileH + (tid >> 4), x = x0 + (tid & 15);
        const bool valid = y < p.h && x < p.w_;
        const long long q = ((long long)b * p.h + y) * p.w_ + x;
        const uint32_t lane_base =
            tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)a * acc_cols + (uint32_t)(u * p.ntile);
        for (int nc = 0; nc < p.ntile; nc += 8) {
          float v[8];
          tmem_ld8(lane_base + (uint32_t)nc, v);
          epilogue8(p, valid, q, n0 + nc, v);
        }
      }
      tc_fence_before();
      mbar_arrive(&acce[a]);
    }
  }
  __syncthreads();
  // loads issued but never consumed (after an abort): wait for them to land
  if (tid == 128)
    for (int g = s_consumed; g < s_issued; ++g) mbar_wait(&full[g % S], (uint32_t)(g / S) & 1u);
  const bool fin = mbar_wait(&done, 0);
  if (tid == 0 && (!fin || s_abort)) atomicCAS(&g_sg_status, 0, SHY_ERR_TIMEOUT);
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tmem_free(tmem, p.tmem_cols);
  }
}

// ---------------------------------------------------------------------------
// Weight gradient with TMA staging (wgrad_tma_kernel).
//
// D[m = (tap, ci)][n = co] += sum over pixels k of X[k + tap][ci] * dZ[k][co]:
// M = 128 weight rows, N = a cout tile, K = pixels, one tile of 16 x 4 or
// 16 x 8 pixels per pipeline stage.  Both operands keep their channel index
// contiguous, so the MMA reads them MN-major.  A is 128 / kcm boxes of kcm
// input channels x 16 x 8 pixels at one tap's offset (box i holds weight
// rows m0 + i * kcm .., all of one tap); B is ntile / kcn boxes of kcn
// channels of dZ.  A box lands as one row of kcm * 2 bytes per pixel,
// swizzled to that row width, so its 8-row groups (the swizzle atoms) are
// 16 * kcm bytes apart (the descriptor's stride byte offset) and consecutive
// boxes, the next kcm channels along M (or N), a box's size apart (its
// leading byte offset).  Each CTA sums a range of pixel tiles in tensor memory and
// adds the result to dw with atomics.
struct WgradTma {
  float* dw;
  int batch, h, w_, cin, cout, ks;
  int ntile, kcm, kcn, tmem_cols, tiles_w, tiles_h, stages, box_h;
  long long tiles_per_split;
  uint32_t a_bytes, b_bytes, stage_bytes, la, lb;
};

__global__ void __launch_bounds__(kThreads) wgrad_tma_kernel(const __grid_constant__ CUtensorMap map_x,
                                                            const __grid_constant__ CUtensorMap map_dz,
                                                            const WgradTma p) {
  extern __shared__ uint8_t smem_raw[];
  __shared__ uint64_t full[kMaxStages], empty[kMaxStages], done;
  __shared__ uint32_t tmem_slot;
  __shared__ int s_fail;
  const uint32_t base = (smem_u32(smem_raw) + 1023u) & ~1023u;
  const int tid = threadIdx.x, warp = tid >> 5;
  const int taps = p.ks * p.ks, half = p.ks >> 1;
  const int rows = taps * p.cin;
  const int m0 = blockIdx.x * kTileM, n0 = blockIdx.y * p.ntile;
  const long long ntiles = (long long)p.batch * p.tiles_h * p.tiles_w;
  const long long t_begin = (long long)blockIdx.z * p.tiles_per_split;
  const long long t_end = min(t_begin + p.tiles_per_split, ntiles);
  const int iters = (int)max(0ll, t_end - t_begin);

  if (warp == 0) tmem_alloc(&tmem_slot, p.tmem_cols);
  if (tid == 0) {
    for (int s = 0; s < p.stages; ++s) {
      mbar_init(&full[s], 1);
      mbar_init(&empty[s], 1);
    }
    mbar_init(&done, 1);
    s_fail = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;

  if (tid == 0) {
    const int S = p.stages;
    // MN-major operands: bits 15 and 16 of the instruction descriptor
    const uint32_t idesc = idesc_bf16_m128(p.ntile) | (1u << 15) | (1u << 16);
    const int na = kTileM / p.kcm, nb = p.ntile / p.kcn;
    int na_live = 0;  // boxes of A inside the weight rows (the rest of the tile's rows are never stored)
    for (int i = 0; i < na; ++i) na_live += (m0 + i * p.kcm < rows);
    const uint32_t box_a = 32u * p.box_h * p.kcm, box_b = 32u * p.box_h * p.kcn;  // bytes of one box
    const uint32_t tx_bytes = (uint32_t)na_live * box_a + (uint32_t)nb * box_b;
    auto issue = [&](int it) {
      const int s = it % S;
      long long t = t_begin + it;
      const int tx = (int)(t % p.tiles_w);
      t /= p.tiles_w;
      const int ty = (int)(t % p.tiles_h), b = (int)(t / p.tiles_h);
      const int x0 = tx * kTileW, y0 = ty * p.box_h;
      const uint32_t sa = base + s * p.stage_bytes, sb = sa + p.a_bytes;
      mbar_expect_tx(&full[s], tx_bytes);
      for (int i = 0; i < na; ++i) {
        const int r = m0 + i * p.kcm;
        if (r >= rows) break;
        const int tap = r / p.cin, c0 = r - tap * p.cin;
        tma_load_4d(sa + i * box_a, &map_x, c0, x0 + tap % p.ks - half, y0 + tap / p.ks - half, b,
                    &full[s]);
      }
      for (int j = 0; j < nb; ++j) tma_load_4d(sb + j * box_b, &map_dz, n0 + j * p.kcn, x0, y0, b, &full[s]);
    };
    int issued = 0, consumed = 0;
    bool fail = false;
    for (; issued < S - 1 && issued < iters; ++issued) issue(issued);
    for (int it = 0; it < iters; ++it) {
      const int s = it % S;
      if (!mbar_wait(&full[s], (uint32_t)(it / S) & 1u)) {
        fail = true;
        break;
      }
      consumed = it + 1;
      tc_fence_after();
      const uint32_t sa = base + s * p.stage_bytes, sb = sa + p.a_bytes;
      for (int kk = 0; kk < p.box_h; ++kk)  // 16 pixels (one tile row) per MMA
        mma_bf16(tmem, smem_desc_mn(sa + kk * 32u * p.kcm, box_a, 16u * p.kcm, p.la),
                 smem_desc_mn(sb + kk * 32u * p.kcn, box_b, 16u * p.kcn, p.lb), idesc, (it | kk) != 0);
      mma_commit(&empty[s]);
      if (issued < iters) {
        const int s2 = issued % S;
        if (issued >= S && !mbar_wait(&empty[s2], (uint32_t)(issued / S - 1) & 1u)) {
          fail = true;
          break;
        }
        issue(issued);
        ++issued;
      }
    }
    for (int it = consumed; it < issued; ++it) mbar_wait(&full[it % S], (uint32_t)(it / S) & 1u);
    mma_commit(&done);
    if (fail) s_fail = 1;
  }
  const bool fin = mbar_wait(&done, 0);
  const bool ok = __syncthreads_and(fin) != 0 && s_fail == 0;
  if (ok && iters > 0) {
    tc_fence_after();
    const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16);
    const int r = m0 + tid;
    for (int nc = 0; nc < p.ntile; nc += 8) {
      float v[8];
      tmem_ld8(lane_base + (uint32_t)nc, v);
      if (r >= rows) continue;
      for (int j = 0; j < 8; ++j) atomicAdd(p.dw + (long long)(n0 + nc + j) * rows + r, v[j]);
    }
  } else if (!ok && tid == 0) {
    atomicCAS(&g_sg_status, 0, SHY_ERR_TIMEOUT);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tmem_free(tmem, p.tmem_cols);
  }
}

struct ConvWgrad {
  const __nv_bfloat16* x;
  const __nv_bfloat16* dz;
  float* dw;
  int batch, h, w_, cin, cout, ks;
  int xs, dzs;
  int ntile, tmem_cols;
  long long chunks_per_split;
};

// Stores the 8 bf16 of `v` down 8 consecutive rows of a K-major core-matrix
// group: row e at byte e * 16 from `dst`.
__device__ __forceinline__ void scatter8(uint8_t* dst, const uint4 v) {
  const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
  for (int e = 0; e < 4; ++e) {
    *reinterpret_cast<uint16_t*>(dst + (2 * e) * 16) = (uint16_t)(w[e] & 0xFFFFu);
    *reinterpret_cast<uint16_t*>(dst + (2 * e + 1) * 16) = (uint16_t)(w[e] >> 16);
  }
}

__global__ void __launch_bounds__(kThreads) conv_wgrad_kernel(const ConvWgrad p) {
  extern __shared__ __align__(1024) uint8_t smem[];
  __shared__ uint64_t bars[3];
  __shared__ uint32_t tmem_slot;
  const int tid = threadIdx.x, warp = tid >> 5;
  const long long hw = (long long)p.h * p.w_;
  const long long npix = (long long)p.batch * hw;
  const int taps = p.ks * p.ks, half = p.ks >> 1;
  const int rows = taps * p.cin;  // weight rows (tap, cin)
  const int m0 = blockIdx.x * kTileM;
  const int n0 = blockIdx.y * p.ntile;
  const long long nchunks = (npix + kWgradK - 1) / kWgradK;
  const long long c_begin = (long long)blockIdx.z * p.chunks_per_split;
  const long long c_end = min(c_begin + p.chunks_per_split, nchunks);
  const int iters = (int)max(0ll, c_end - c_begin);
  const uint32_t sbo = (uint32_t)kWgradK * 16;
  const uint32_t a_bytes = (uint32_t)kTileM * kWgradK * 2, b_bytes = (uint32_t)p.ntile * kWgradK * 2;
  const uint32_t stage_bytes = a_bytes + b_bytes;

  if (warp == 0) tmem_alloc(&tmem_slot, p.tmem_cols);
  if (tid == 0) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    mbar_init(&bars[2], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  tc_fence_before();
  __syncthreads();
  tc_fence_after();
  const uint32_t tmem = tmem_slot;
  const uint32_t idesc = idesc_bf16_m128(p.ntile);
  const int b_items = p.ntile * (kWgradK / 8);  // (8-channel group, pixel) pairs of B
  bool failed = false;
  for (int it = 0; it < iters; ++it) {
    const int s = it & 1;
    uint8_t* sa = smem + s * stage_bytes;
    uint8_t* sb = sa + a_bytes;
    int fail = 0;
    if (it >= 2 && !mbar_wait(&bars[s], (uint32_t)((it >> 1) - 1) & 1u)) fail = 1;
    const long long q0 = (c_begin + it) * kWgradK;
    // A: 16 groups of 8 weight rows x 64 pixels
    for (int i = tid; i < (kTileM / 8) * kWgradK; i += kThreads) {
      const int pix = i & (kWgradK - 1), grp = i / kWgradK;
      const int r0 = m0 + grp * 8;
      uint4 v = make_uint4(0u, 0u, 0u, 0u);
      const long long q = q0 + pix;
      if (r0 < rows && q < npix) {
        const int tap = r0 / p.cin, ci = r0 - tap * p.cin;
        const int qb = (int)(q / hw);
        const long long r = q - (long long)qb * hw;
        const int qy = (int)(r / p.w_), qx = (int)(r - (long long)(r / p.w_) * p.w_);
        const int yy = qy + tap / p.ks - half, xx = qx + tap % p.ks - half;
        if (yy >= 0 && yy < p.h && xx >= 0 && xx < p.w_)
          v = __ldg(reinterpret_cast<const uint4*>(
              p.x + (((long long)qb * p.h + yy) * p.w_ + xx) * p.xs + ci));
      }
      scatter8(sa + grp * sbo + (pix >> 3) * 128 + (pix & 7) * 2, v);
    }
    // B: ntile / 8 groups of 8 output channels x 64 pixels
    for (int i = tid; i < b_items; i += kThreads) {
      const int pix = i & (kWgradK - 1), grp = i / kWgradK;
      const long long q = q0 + pix;
      uint4 v = make_uint4(0u, 0u, 0u, 0u);
      if (q < npix) v = __ldg(reinterpret_cast<const uint4*>(p.dz + q * p.dzs + n0 + grp * 8));
      scatter8(sb + grp * sbo + (pix >> 3) * 128 + (pix & 7) * 2, v);
    }
    fence_async_smem();
    if (__syncthreads_or(fail)) {
      failed = true;
      break;
    }
    if (tid == 0) {
      tc_fence_after();
      const uint32_t a0 = smem_u32(sa), b0 = smem_u32(sb);
      for (int kk = 0; kk < kWgradK / 16; ++kk)
        mma_bf16(tmem, smem_desc(a0 + kk * 256, 128, sbo), smem_desc(b0 + kk * 256, 128, sbo), idesc,
                 (it | kk) != 0);
      mma_commit(&bars[s]);
    }
  }
  if (tid == 0) mma_commit(&bars[2]);
  const bool done = mbar_wait(&bars[2], 0);
  const bool ok = __syncthreads_and(done && !failed) != 0;
  if (ok && iters > 0) {
    tc_fence_after();
    const uint32_t lane_base = tmem + ((uint32_t)(warp * 32) << 16);
    const int r = m0 + tid;
    for (int nc = 0; nc < p.ntile; nc += 8) {
      float v[8];
      tmem_ld8(lane_base + (uint32_t)nc, v);
      if (r >= rows) continue;
      for (int j = 0; j < 8; ++j) atomicAdd(p.dw + (long long)(n0 + nc + j) * rows + r, v[j]);
    }
  } else if (!ok && tid == 0) {
    atomicCAS(&g_sg_status, 0, SHY_ERR_TIMEOUT);
  }
  tc_fence_before();
  __syncthreads();
  if (warp == 0) {
    tc_fence_after();
    tmem_free(tmem, p.tmem_cols);
  }
}

// Per-channel sums for channel counts dividing 256: with 256-thread blocks
// and a grid stride that is a multiple of 256, every element a thread visits
// has channel threadIdx.x % channels.  The block adds its threads' sums in
// shared memory and makes one atomic addition per channel.
__device__ __forceinline__ void flush_channel_sums(float acc, int channels, float* db) {
  __shared__ float red[256];
  red[threadIdx.x] = acc;
  __syncthreads();
  if ((int)threadIdx.x < channels) {
    float s = 0.0f;
    for (int t = threadIdx.x; t < (int)blockDim.x; t += channels) s += red[t];
    atomicAdd(db + threadIdx.x, s);
  }
}

__global__ void __launch_bounds__(256) bias_grad_kernel(const __nv_bfloat16* __restrict__ dz, int dzs,
                                                        long long npix, int channels, float* __restrict__ db) {
  const long long n = npix * channels;
  float acc = 0.0f;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const long long q = i / channels;
    acc += __bfloat162float(dz[q * dzs + (i - q * channels)]);
  }
  flush_channel_sums(acc, channels, db);
}

// any channel count: one thread per channel over a range of pixels
__global__ void bias_grad_any_kernel(const __nv_bfloat16* __restrict__ dz, int dzs, long long npix, int channels,
                                     long long per_block, float* __restrict__ db) {
  const long long q0 = (long long)blockIdx.x * per_block;
  const long long q1 = min(q0 + per_block, npix);
  for (int c = threadIdx.x; c < channels; c += blockDim.x) {
    float s = 0.0f;
    for (long long q = q0; q < q1; ++q) s += __bfloat162float(dz[q * dzs + c]);
    atomicAdd(db + c, s);
  }
}

// One thread per (pixel, 8 channels): two 16-byte loads each of da and z,
// one 16-byte store of dz.  Channel groups per pixel (channels / 8) divide
// 256, so with a grid stride that is a multiple of 256 each thread keeps one
// channel group and its 8 bias sums; the block adds them in shared memory.
__global__ void __launch_bounds__(256) gelu_backward_kernel(int n8, int groups, const float* __restrict__ da,
                                                            int das, int dao, const float* __restrict__ z, int zs,
                                                            int zo, __nv_bfloat16* __restrict__ dz,
                                                            float* __restrict__ db) {
  float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n8; i += gridDim.x * blockDim.x) {
    const int q = i / groups, c = (i - q * groups) * 8;
    const float4* ap = reinterpret_cast<const float4*>(da + (long long)q * das + dao + c);
    const float4* zp = reinterpret_cast<const float4*>(z + (long long)q * zs + zo + c);
    const float4 a0 = ap[0], a1 = ap[1], z0 = zp[0], z1 = zp[1];
    const float av[8] = {a0.x, a0.y, a0.z, a0.w, a1.x, a1.y, a1.z, a1.w};
    const float zv[8] = {z0.x, z0.y, z0.z, z0.w, z1.x, z1.y, z1.z, z1.w};
    float g[8];
#pragma unroll
    for (int e = 0; e < 8; ++e) {
      g[e] = __bfloat162float(__float2bfloat16_rn(av[e] * gelu_grad(zv[e])));
      acc[e] += g[e];
    }
    uint4 o;
    o.x = pack_bf16(g[0], g[1]);
    o.y = pack_bf16(g[2], g[3]);
    o.z = pack_bf16(g[4], g[5]);
    o.w = pack_bf16(g[6], g[7]);
    *reinterpret_cast<uint4*>(dz + (long long)i * 8) = o;
  }
  if (!db) return;
  __shared__ float red[8][256];
#pragma unroll
  for (int e = 0; e < 8; ++e) red[e][threadIdx.x] = acc[e];
  __syncthreads();
  const int channels = groups * 8;
  if ((int)threadIdx.x < channels) {
    const int gi = threadIdx.x >> 3, e = threadIdx.x & 7;
    float sum = 0.0f;
    for (int t = gi; t < (int)blockDim.x; t += groups) sum += red[e][t];
    atomicAdd(db + threadIdx.x, sum);
  }
}

// one thread per (pooled pixel, 8-channel vector)
__global__ void pool_fwd_kernel(int batch, int h, int w, int channels, const __nv_bfloat16* __restrict__ x,
                                int xs, int xo, __nv_bfloat16* __restrict__ y, int ys, int yo) {
  const int ho = h >> 1, wo = w >> 1, nv = channels >> 3;
  const long long n = (long long)batch * ho * wo * nv;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const int v = (int)(i % nv);
    const long long qo = i / nv;
    const int ox = (int)(qo % wo);
    const long long t = qo / wo;
    const int oy = (int)(t % ho), b = (int)(t / ho);
    float acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int dy = 0; dy < 2; ++dy)
      for (int dx = 0; dx < 2; ++dx) {
        const long long qi = ((long long)b * h + 2 * oy + dy) * w + 2 * ox + dx;
        const uint4 u = __ldg(reinterpret_cast<const uint4*>(x + qi * xs + xo + 8 * v));
        const uint32_t ws[4] = {u.x, u.y, u.z, u.w};
        for (int e = 0; e < 4; ++e) {
          acc[2 * e] += bf16_lo(ws[e]);
          acc[2 * e + 1] += bf16_hi(ws[e]);
        }
      }
    uint4 o;
    o.x = pack_bf16(0.25f * acc[0], 0.25f * acc[1]);
    o.y = pack_bf16(0.25f * acc[2], 0.25f * acc[3]);
    o.z = pack_bf16(0.25f * acc[4], 0.25f * acc[5]);
    o.w = pack_bf16(0.25f * acc[6], 0.25f * acc[7]);
    *reinterpret_cast<uint4*>(y + qo * ys + yo + 8 * v) = o;
  }
}

// one thread per (input pixel, channel)
__global__ void pool_bwd_kernel(int batch, int h, int w, int channels, const float* __restrict__ dy, int dys,
                                int dyo, float* __restrict__ dx, int dxs, int dxo) {
  const long long n = (long long)batch * h * w * channels;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const int c = (int)(i % channels);
    const long long qi = i / channels;
    const int x = (int)(qi % w);
    const long long t = qi / w;
    const int y = (int)(t % h), b = (int)(t / h);
    const long long qo = ((long long)b * (h >> 1) + (y >> 1)) * (w >> 1) + (x >> 1);
    dx[qi * dxs + dxo + c] += 0.25f * dy[qo * dys + dyo + c];
  }
}

// one thread per (fine pixel, 8-channel vector); h, w: the coarse grid
__global__ void up_fwd_kernel(int batch, int h, int w, int channels, const __nv_bfloat16* __restrict__ x,
                              int xs, int xo, __nv_bfloat16* __restrict__ y, int ys, int yo) {
  const int hf = 2 * h, wf = 2 * w, nv = channels >> 3;
  const long long n = (long long)batch * hf * wf * nv;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const int v = (int)(i % nv);
    const long long qf = i / nv;
    const int fx = (int)(qf % wf);
    const long long t = qf / wf;
    const int fy = (int)(t % hf), b = (int)(t / hf);
    const long long qc = ((long long)b * h + (fy >> 1)) * w + (fx >> 1);
    *reinterpret_cast<uint4*>(y + qf * ys + yo + 8 * v) =
        __ldg(reinterpret_cast<const uint4*>(x + qc * xs + xo + 8 * v));
  }
}

// one thread per (coarse pixel, channel)
__global__ void up_bwd_kernel(int batch, int h, int w, int channels, const float* __restrict__ dy, int dys,
                              int dyo, float* __restrict__ dx, int dxs, int dxo) {
  const long long n = (long long)batch * h * w * channels;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const int c = (int)(i % channels);
    const long long qc = i / channels;
    const int x = (int)(qc % w);
    const long long t = qc / w;
    const int y = (int)(t % h), b = (int)(t / h);
    float s = 0.0f;
    for (int ddy = 0; ddy < 2; ++ddy)
      for (int ddx = 0; ddx < 2; ++ddx) {
        const long long qf = ((long long)b * 2 * h + 2 * y + ddy) * (2 * w) + 2 * x + ddx;
        s += dy[qf * dys + dyo + c];
      }
    dx[qc * dxs + dxo + c] += s;
  }
}

__global__ void weight_prep_kernel(int cout, int taps, int cin, const float* __restrict__ w,
                                   __nv_bfloat16* __restrict__ wb, __nv_bfloat16* __restrict__ wf) {
  const long long n = (long long)cout * taps * cin;
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const int ci = (int)(i % cin);
    const long long t = i / cin;
    const int tap = (int)(t % taps), co = (int)(t / taps);
    const __nv_bfloat16 v = __float2bfloat16_rn(w[i]);
    wb[i] = v;
    if (wf) wf[((long long)ci * taps + (taps - 1 - tap)) * cout + co] = v;
  }
}

__global__ void adamw_kernel(long long n, float* __restrict__ p, const float* __restrict__ g,
                             float* __restrict__ m, float* __restrict__ v, const shy_sg_adamw_args a) {
  for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
       i += (long long)gridDim.x * blockDim.x) {
    const float gi = g[i];
    const float mi = a.beta1 * m[i] + (1.0f - a.beta1) * gi;
    const float vi = a.beta2 * v[i] + (1.0f - a.beta2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float step = (mi / a.bc1) / (sqrtf(vi / a.bc2) + a.eps);
    p[i] -= a.lr * (step + a.weight_decay * p[i]);
  }
}

__global__ void features_kernel(int batch, int h, int w, const float* __restrict__ hm, const shy_sg_norm nm,
                                __nv_bfloat16* __restrict__ x) {
  const long long n = (long long)batch * h * w;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    const int c = (int)(q % w);
    const long long t = q / w;
    const int r = (int)(t % h), b = (int)(t / h);
    const float* img = hm + (long long)b * h * w;
    const int r0 = max(r - 1, 0), r1 = min(r + 1, h - 1);
    const int c0 = max(c - 1, 0), c1 = min(c + 1, w - 1);
    const float gr = (img[(long long)r1 * w + c] - img[(long long)r0 * w + c]) / (float)max(r1 - r0, 1);
    const float gc = (img[(long long)r * w + c1] - img[(long long)r * w + c0]) / (float)max(c1 - c0, 1);
    const float hv = (img[(long long)r * w + c] - nm.height_mean) * nm.height_scale;
    uint4* dst = reinterpret_cast<uint4*>(x + q * 16);
    dst[0] = make_uint4(pack_bf16(hv, gr * nm.slope_scale), pack_bf16(gc * nm.slope_scale, 0.0f), 0u, 0u);
    dst[1] = make_uint4(0u, 0u, 0u, 0u);
  }
}

__global__ void loss_kernel(long long n, const float* __restrict__ z, int zs, const float* __restrict__ t,
                            float w0, float w1, float w2, float scale, __nv_bfloat16* __restrict__ dz,
                            double* __restrict__ loss) {
  __shared__ double part[32];
  double acc = 0.0;
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    const float e0 = z[q * zs] - t[3 * q], e1 = z[q * zs + 1] - t[3 * q + 1], e2 = z[q * zs + 2] - t[3 * q + 2];
    acc += (double)(w0 * e0 * e0) + (double)(w1 * e1 * e1) + (double)(w2 * e2 * e2);
    uint4* dst = reinterpret_cast<uint4*>(dz + q * 16);
    dst[0] = make_uint4(pack_bf16(2.0f * w0 * e0 * scale, 2.0f * w1 * e1 * scale),
                        pack_bf16(2.0f * w2 * e2 * scale, 0.0f), 0u, 0u);
    dst[1] = make_uint4(0u, 0u, 0u, 0u);
  }
  for (int o = 16; o > 0; o >>= 1) acc += __shfl_xor_sync(0xFFFFFFFFu, acc, o);
  if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = acc;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) s += part[i];
    atomicAdd(loss, s * (double)scale);
  }
}

__global__ void decode_kernel(long long n, const float* __restrict__ z, int zs, const shy_sg_norm nm,
                              float* __restrict__ d, float* __restrict__ mx, float* __restrict__ my) {
  for (long long q = blockIdx.x * (long long)blockDim.x + threadIdx.x; q < n;
       q += (long long)gridDim.x * blockDim.x) {
    d[q] = fmaxf(0.0f, expm1f(z[q * zs] * nm.out_scale[0] + nm.out_mean[0]));
    mx[q] = z[q * zs + 1] * nm.out_scale[1] + nm.out_mean[1];
    my[q] = z[q * zs + 2] * nm.out_scale[2] + nm.out_mean[2];
  }
}

int grid_for(long long n, int block = 256) {
  const long long g = (n + block - 1) / block;
  return (int)std::max(1ll, std::min(g, 152ll * 32));
}

bool aligned16(const void* p) { return ((uintptr_t)p & 15u) == 0; }

int launch_status(const char* what) {
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    set_error("%s: %s", what, cudaGetErrorString(e));
    return SHY_ERR_CUDA;
  }
  return SHY_OK;
}

// Output-channel tile: the largest of 128, 96, 64, 32, 16 dividing cout.
int pick_ntile(int cout) {
  for (int t : {128, 96, 64, 32, 16})
    if (cout % t == 0) return t;
  return 0;
}

int pow2_cols(int n) {
  int c = 32;
  while (c < n) c <<= 1;
  return c;
}

// Dynamic shared memory for a tensor-core CTA: its stages, raised where
// needed so that the CTAs resident on one SM never ask for more than the
// 512 TMEM columns together.
int smem_for(int stage_bytes, int tmem_cols) {
  const int need = 2 * stage_bytes;
  const int max_ctas = 512 / tmem_cols;
  const int floor_bytes = kSmemPerSm / (max_ctas + 1) - kSmemReservedPerCta + 1024;
  return std::max(need, floor_bytes);
}

int g_conv_path = SHY_SG_CONV_TMA;
int g_conv_stages = 0;  // 0: chosen per convolution
int g_conv_pixels = 0;  // pixels per tile, 128 or 256; 0: chosen per convolution
int g_conv_tap_rows = 3;  // 3x3 taps per stage on the TMA path: 3 (a kernel column) or 1
int g_wgrad_pixels = 0, g_wgrad_stages = 0;  // 0: chosen per convolution

// cuTensorMapEncodeTiled from the driver, looked up once per process through
// the runtime (a function-local static: initialised once, thread-safe).
PFN_cuTensorMapEncodeTiled_v12000 lookup_encode_tiled() {
  void* f = nullptr;
  cudaDriverEntryPointQueryResult q;
  if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &f, 12000, cudaEnableDefault, &q) ==
          cudaSuccess &&
      q == cudaDriverEntryPointSuccess)
    return reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(f);
  cudaGetLastError();
  return nullptr;
}
PFN_cuTensorMapEncodeTiled_v12000 encode_tiled() {
  static const PFN_cuTensorMapEncodeTiled_v12000 fn = lookup_encode_tiled();
  return fn;
}

CUtensorMapSwizzle swizzle_for(int kc) {
  return kc == 64 ? CU_TENSOR_MAP_SWIZZLE_128B : kc == 32 ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_32B;
}

// An NHWC bf16 activation tensor (channels, width, height, batch) with a
// box of kc channels x 16 x 8 pixels x 1 image, swizzled to the box's row
// width, zero fill outside.
bool encode_act_map(CUtensorMap* m, const void* ptr, int channels, int width, int height, int batch, int stride,
                    int kc, int box_h = kTileH) {
  auto fn = encode_tiled();
  if (!fn) return false;
  const cuuint64_t row = (cuuint64_t)stride * 2;
  const cuuint64_t g[4] = {(cuuint64_t)channels, (cuuint64_t)width, (cuuint64_t)height, (cuuint64_t)batch};
  const cuuint64_t st[3] = {row, row * width, row * width * height};
  const cuuint32_t box[4] = {(cuuint32_t)kc, (cuuint32_t)kTileW, (cuuint32_t)box_h, 1};
  const cuuint32_t e[4] = {1, 1, 1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 4, const_cast<void*>(ptr), g, st, box, e,
            CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle_for(kc), CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

// Tensor maps of one convolution: the input (encode_act_map) and the
// weights as (taps * cin, cout) with a box of kc x ntile.
bool encode_conv_maps(const shy_sg_conv_desc* d, const void* x, int xs, const void* w, int kc, int ntile, int mt,
                      int tap_rows, CUtensorMap* mx, CUtensorMap* mw) {
  auto fn = encode_tiled();
  if (!fn || !encode_act_map(mx, x, d->cin, d->width, d->height, d->batch, xs, kc, kTileH * mt + tap_rows - 1))
    return false;
  const cuuint64_t k = (cuuint64_t)d->ksize * d->ksize * d->cin;
  const cuuint64_t gw[2] = {k, (cuuint64_t)d->cout};
  const cuuint64_t sw2[1] = {k * 2};
  const cuuint32_t bw[2] = {(cuuint32_t)kc, (cuuint32_t)ntile};
  const cuuint32_t e[2] = {1, 1};
  return fn(mw, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(w), gw, sw2, bw, e,
            CU_TENSOR_MAP_INTERLEAVE_NONE, swizzle_for(kc), CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

bool check_conv_desc(const shy_sg_conv_desc* d, const char* fn) {
  if (!d) {
    set_error("%s: null descriptor", fn);
    return false;
  }
  if (d->batch <= 0 || d->height <= 0 || d->width <= 0 || d->cin <= 0 || d->cout <= 0 ||
      d->cin % 16 || d->cout % 16 || (d->ksize != 1 && d->ksize != 3) ||
      (d->stages != 0 && (d->stages < 2 || d->stages > kMaxStages))) {
    set_error("%s: bad shape %dx%dx%d cin %d cout %d ksize %d", fn, d->batch, d->height, d->width, d->cin,
              d->cout, d->ksize);
    return false;
  }
  const long long npix = (long long)d->batch * d->height * d->width;
  if (npix > (1ll << 40) / 128) {
    set_error("%s: too many pixels", fn);
    return false;
  }
  return true;
}

}  // namespace

}  // namespace shy

using namespace shy;

namespace {

// Launch set-up of the current device, done once per device under a lock:
// the dynamic shared-memory limits of the convolution kernels (an attribute
// of a kernel on one device) and the SM count that sizes persistent and
// split grids.
struct DeviceSetup {
  bool done;
  int sms;
};
const int kMaxDevices = 64;
std::mutex g_setup_mu;
DeviceSetup g_setup[kMaxDevices] = {};

const int kConvSmem = 200 * 1024;      // conv_tma, conv_fwd, wgrad kernels
const int kWsSmem = 227 * 1024 - 1024;  // the persistent convolution

int device_sms() {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    cudaGetLastError();
    return 152;
  }
  std::lock_guard<std::mutex> lock(g_setup_mu);
  DeviceSetup& d = g_setup[dev];
  if (!d.done) {
    cudaFuncSetAttribute(conv_tma_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kConvSmem);
    cudaFuncSetAttribute(conv_ws_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kWsSmem);
    cudaFuncSetAttribute(conv_fwd_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kConvSmem);
    cudaFuncSetAttribute(wgrad_tma_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kConvSmem);
    cudaFuncSetAttribute(conv_wgrad_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, kConvSmem);
    int sms = 0;
    if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || sms < 1) sms = 152;
    d.sms = sms;
    d.done = true;
  }
  return d.sms;
}

// Both convolution entry points: a forward (gz NULL) or an input gradient
// through a GELU (gz the previous layer's pre-activation, output bf16 to a).
int conv_launch(const char* fn, const shy_sg_conv_desc* d, const void* x, int32_t x_stride, const void* w,
                const float* bias, float* z, int32_t z_stride, int32_t z_offset, void* a, int32_t a_stride,
                int32_t a_offset, int32_t act, const float* gz, int32_t gz_stride, int32_t gz_offset,
                void* stream) {
  if (!check_conv_desc(d, fn)) return SHY_ERR_INVALID_ARG;
  if (!x || !w || (!z && !a) || !aligned16(x) || !aligned16(w) || x_stride < d->cin || x_stride % 8) {
    set_error("%s: bad input or weight pointer or stride", fn);
    return SHY_ERR_INVALID_ARG;
  }
  if (z && (!aligned16(z) || z_stride % 4 || z_offset % 4 || z_offset < 0 || z_offset + d->cout > z_stride)) {
    set_error("%s: bad f32 output layout", fn);
    return SHY_ERR_INVALID_ARG;
  }
  if (a && (!aligned16(a) || a_stride % 8 || a_offset % 8 || a_offset < 0 || a_offset + d->cout > a_stride)) {
    set_error("%s: bad bf16 output layout", fn);
    return SHY_ERR_INVALID_ARG;
  }
  if (act != SHY_SG_ACT_NONE && act != SHY_SG_ACT_GELU) {
    set_error("%s: unknown activation %d", fn, act);
    return SHY_ERR_INVALID_ARG;
  }
  const int ntile = pick_ntile(d->cout);
  CUtensorMap mx, mw;
  // tile: the call's own choice, else the process-wide one, else 128 pixels
  if (d->tile != 0 && d->tile != 128 && d->tile != 256 && d->tile != 512) {
    set_error("%s: tile %d (0, 128, 256 or 512 pixels)", fn, d->tile);
    return SHY_ERR_INVALID_ARG;
  }
  const int pix = d->tile ? d->tile : g_conv_pixels;
  const int mt = pix ? pix / kTileM : 1;
  const bool tma_path = g_conv_path == SHY_SG_CONV_TMA || g_conv_path == SHY_SG_CONV_PERSISTENT;
  // 512-pixel tiles: four accumulators of up to 128 columns (all of TMEM at
  // N = 128, one CTA per SM); each weight chunk then feeds 512 pixels.  With
  // three taps per stage they take 32-channel chunks, so that two or three
  // stages fit in shared memory; with one tap per stage 64-channel chunks
  // (128-byte box rows) fit two stages.  The persistent path double-buffers
  // its accumulators and cannot hold four; the staged path has its own tile
  // and ignores this one.
  if (mt == 4 && g_conv_path == SHY_SG_CONV_PERSISTENT) {
    set_error("%s: 512-pixel tiles are for the TMA path (one CTA per tile)", fn);
    return SHY_ERR_INVALID_ARG;
  }
  if (d->tap_rows != 0 && d->tap_rows != 1 && d->tap_rows != 3) {
    set_error("%s: tap_rows %d (0, 1 or 3)", fn, d->tap_rows);
    return SHY_ERR_INVALID_ARG;
  }
  const int rows_want = d->tap_rows ? d->tap_rows : g_conv_tap_rows;
  const int tap_rows = (g_conv_path == SHY_SG_CONV_TMA && d->ksize == 3 && rows_want == 3) ? 3 : 1;
  const int kc = (d->cin % 64 == 0 && (mt < 4 || tap_rows == 1)) ? 64 : d->cin % 32 == 0 ? 32 : 16;
  // (3x3 on the one-CTA-per-tile TMA path: one input box per kernel column)
  if (tma_path && encode_conv_maps(d, x, x_stride, w, kc, ntile, mt, tap_rows, &mx, &mw)) {
    ConvTma p{};
    p.bias = bias;
    p.z = z;
    p.a = static_cast<__nv_bfloat16*>(a);
    p.gz = gz;
    p.gzs = gz_stride;
    p.gzo = gz_offset;
    p.batch = d->batch;
    p.h = d->height;
    p.w_ = d->width;
    p.cin = d->cin;
    p.cout = d->cout;
    p.ks = d->ksize;
    p.zs = z_stride;
    p.zo = z_offset;
    p.as = a_stride;
    p.ao = a_offset;
    p.act = act;
    p.ntile = ntile;
    p.kc = kc;
    p.mt = mt;
    p.tmem_cols = pow2_cols(ntile * mt);
    p.tiles_w = (d->width + kTileW - 1) / kTileW;
    p.tiles_h = (d->height + kTileH * mt - 1) / (kTileH * mt);
    p.tap_rows = tap_rows;
    p.stall_ns = debug_stall_ns();
    p.a_box = (uint32_t)kTileW * (kTileH * mt + tap_rows - 1) * kc * 2;
    p.a_bytes = (p.a_box + 1023u) & ~1023u;
    p.b_box = ((uint32_t)ntile * kc * 2 + 1023u) & ~1023u;
    p.b_bytes = (uint32_t)tap_rows * ntile * kc * 2;
    p.stage_bytes = p.a_bytes + tap_rows * p.b_box;
    p.layout = kc == 64 ? 2u : kc == 32 ? 4u : 6u;
    // automatic depth: 3 stages (two CTAs an SM) for long 64-channel K loops,
    // else 2 (measured at the training shapes: 543 vs 476 TFLOP/s on the
    // 384 -> 128 layer, 269 vs 242 on 96 -> 32)
    const int iters = d->ksize * d->ksize / tap_rows * (d->cin / kc);
    const int st = d->stages ? d->stages : g_conv_stages;
    const int want = st ? st : (kc == 64 && iters >= 16 && mt == 1 ? 3 : 2);
    p.stages = std::max(2, std::min(want, (200 * 1024 - 1024) / (int)p.stage_bytes));
    const int smem = smem_for((p.stages * (int)p.stage_bytes + 1024) / 2, p.tmem_cols);
    const int sms = device_sms();
    const long long tiles = (long long)d->batch * p.tiles_h * p.tiles_w;
    if (g_conv_path == SHY_SG_CONV_PERSISTENT) {
      // one CTA per SM, two accumulators, the deepest ring that fits
      p.tmem_cols = pow2_cols(2 * ntile * mt);
      const int max_smem = kWsSmem;
      p.stages = d->stages ? d->stages : std::min(6, (max_smem - 1024) / (int)p.stage_bytes);
      p.stages = std::max(2, std::min(p.stages, (max_smem - 1024) / (int)p.stage_bytes));
      const int ws_smem = std::max(p.stages * (int)p.stage_bytes + 1024, 120 * 1024);
      const long long work = tiles * (d->cout / ntile);
      const unsigned grid = (unsigned)std::max(1ll, std::min(work, (long long)std::max(sms, 1)));
      conv_ws_kernel<<<grid, kWsThreads, ws_smem, static_cast<cudaStream_t>(stream)>>>(mx, mw, p);
      return launch_status(fn);
    }
    dim3 grid((unsigned)tiles, (unsigned)(d->cout / ntile));
    conv_tma_kernel<<<grid, kThreads, smem, static_cast<cudaStream_t>(stream)>>>(mx, mw, p);
    return launch_status(fn);
  }
  if (tma_path && !encode_tiled()) {
    set_error("%s: cuTensorMapEncodeTiled is not available", fn);
    return SHY_ERR_CUDA;
  }
  if (tma_path) {
    set_error("%s: tensor map encoding failed", fn);
    return SHY_ERR_INVALID_ARG;
  }
  ConvFwd p{};
  p.x = static_cast<const __nv_bfloat16*>(x);
  p.w = static_cast<const __nv_bfloat16*>(w);
  p.bias = bias;
  p.z = z;
  p.a = static_cast<__nv_bfloat16*>(a);
  p.gz = gz;
  p.gzs = gz_stride;
  p.gzo = gz_offset;
  p.batch = d->batch;
  p.h = d->height;
  p.w_ = d->width;
  p.cin = d->cin;
  p.cout = d->cout;
  p.ks = d->ksize;
  p.xs = x_stride;
  p.zs = z_stride;
  p.zo = z_offset;
  p.as = a_stride;
  p.ao = a_offset;
  p.act = act;
  p.ntile = pick_ntile(d->cout);
  p.kc = d->cin % 64 == 0 ? 64 : d->cin % 32 == 0 ? 32 : 16;
  p.tmem_cols = pow2_cols(p.ntile);
  const int stage = (kTileM + p.ntile) * p.kc * 2;
  const int smem = smem_for(stage, p.tmem_cols);
  device_sms();
  const long long npix = (long long)d->batch * d->height * d->width;
  dim3 grid((unsigned)((npix + kTileM - 1) / kTileM), (unsigned)(d->cout / p.ntile));
  conv_fwd_kernel<<<grid, kThreads, smem, static_cast<cudaStream_t>(stream)>>>(p);
  return launch_status(fn);
}

}  // namespace

extern "C" int shy_sg_conv_forward(const shy_sg_conv_desc* d, const void* x, int32_t x_stride, const void* w,
                                   const float* bias, float* z, int32_t z_stride, int32_t z_offset, void* a,
                                   int32_t a_stride, int32_t a_offset, int32_t act, void* stream) {
  return conv_launch("shy_sg_conv_forward", d, x, x_stride, w, bias, z, z_stride, z_offset, a, a_stride, a_offset,
                     act, nullptr, 0, 0, stream);
}

extern "C" int shy_sg_conv_input_grad(const shy_sg_conv_desc* d, const void* dz, int32_t dz_stride,
                                      const void* w_flip, const float* z_prev, int32_t zp_stride,
                                      int32_t zp_offset, void* dz_prev, void* stream) {
  static const char* fn = "shy_sg_conv_input_grad";
  if (!d || !z_prev || !dz_prev || !aligned16(z_prev) || zp_stride % 4 || zp_offset % 4 || zp_offset < 0 ||
      zp_offset + d->cout > zp_stride) {
    set_error("%s: bad pre-activation or output (16-byte aligned, stride and offset multiples of 4)", fn);
    return SHY_ERR_INVALID_ARG;
  }
  return conv_launch(fn, d, dz, dz_stride, w_flip, nullptr, nullptr, 0, 0, dz_prev, d->cout, 0, SHY_SG_ACT_NONE,
                     z_prev, zp_stride, zp_offset, stream);
}

extern "C" int shy_sg_conv_wgrad(const shy_sg_conv_desc* d, const void* x, int32_t x_stride, const void* dz,
                                 int32_t dz_stride, float* dw, void* stream) {
  static const char* fn = "shy_sg_conv_wgrad";
  if (!check_conv_desc(d, fn)) return SHY_ERR_INVALID_ARG;
  if (!x || !dz || !dw || !aligned16(x) || !aligned16(dz) || x_stride < d->cin || x_stride % 8 ||
      dz_stride < d->cout || dz_stride % 8) {
    set_error("%s: bad pointer or stride", fn);
    return SHY_ERR_INVALID_ARG;
  }
  const int ntile = pick_ntile(d->cout);
  const int rows = d->ksize * d->ksize * d->cin;
  if (g_conv_path == SHY_SG_CONV_TMA || g_conv_path == SHY_SG_CONV_PERSISTENT) {
    WgradTma q{};
    q.kcm = d->cin % 64 == 0 ? 64 : d->cin % 32 == 0 ? 32 : 16;
    q.kcn = ntile % 64 == 0 ? 64 : ntile % 32 == 0 ? 32 : 16;
    CUtensorMap mx, mdz;
    // automatic tile: 64-pixel stages where few (M, N) tiles share a small
    // image (measured at the training shapes: 0.32 against 0.47 ms on the
    // 192 -> 64 layer at 128^2), else 128
    const long long npix = (long long)d->batch * d->width * d->height;
    const int ctas_mn = ((rows + kTileM - 1) / kTileM) * (d->cout / ntile);
    if (d->tile != 0 && d->tile != 64 && d->tile != 128) {
      set_error("%s: tile %d (0, 64 or 128 pixels)", fn, d->tile);
      return SHY_ERR_INVALID_ARG;
    }
    const int pix = d->tile ? d->tile : g_wgrad_pixels;
    const int pixels = pix ? pix : (npix < (1ll << 19) && ctas_mn < 16 ? 64 : 128);
    q.box_h = pixels / kTileW;
    if (!encode_act_map(&mx, x, d->cin, d->width, d->height, d->batch, x_stride, q.kcm, q.box_h) ||
        !encode_act_map(&mdz, dz, d->cout, d->width, d->height, d->batch, dz_stride, q.kcn, q.box_h)) {
      set_error("%s: tensor map encoding failed", fn);
      return encode_tiled() ? SHY_ERR_INVALID_ARG : SHY_ERR_CUDA;
    }
    q.dw = dw;
    q.batch = d->batch;
    q.h = d->height;
    q.w_ = d->width;
    q.cin = d->cin;
    q.cout = d->cout;
    q.ks = d->ksize;
    q.ntile = ntile;
    q.tmem_cols = pow2_cols(ntile);
    q.tiles_w = (d->width + kTileW - 1) / kTileW;
    q.tiles_h = (d->height + q.box_h - 1) / q.box_h;
    q.a_bytes = 32u * q.box_h * kTileM;           // 128 / kcm boxes of 32 * box_h * kcm bytes
    q.b_bytes = 32u * q.box_h * ntile;
    q.stage_bytes = q.a_bytes + ((q.b_bytes + 1023u) & ~1023u);
    q.la = q.kcm == 64 ? 2u : q.kcm == 32 ? 4u : 6u;
    q.lb = q.kcn == 64 ? 2u : q.kcn == 32 ? 4u : 6u;
    const int st = d->stages ? d->stages : g_wgrad_stages;
    q.stages = std::max(2, std::min(st ? st : 2, (200 * 1024 - 1024 - 16384) / (int)q.stage_bytes));
    // 16 KiB beyond the last stage: the MMAs' operand reads stay inside the
    // allocation for either order of the descriptor's two strides
    const int smem = smem_for((q.stages * (int)q.stage_bytes + 1024 + 16384) / 2, q.tmem_cols);
    const long long tiles = (long long)d->batch * q.tiles_h * q.tiles_w;
    const long long sms = device_sms();
    long long splits = std::max(1ll, std::min(tiles, (2ll * sms + ctas_mn - 1) / ctas_mn));
    q.tiles_per_split = (tiles + splits - 1) / splits;
    splits = (tiles + q.tiles_per_split - 1) / q.tiles_per_split;
    dim3 grid((unsigned)((rows + kTileM - 1) / kTileM), (unsigned)(d->cout / ntile), (unsigned)splits);
    wgrad_tma_kernel<<<grid, kThreads, smem, static_cast<cudaStream_t>(stream)>>>(mx, mdz, q);
    return launch_status(fn);
  }
  ConvWgrad p{};
  p.x = static_cast<const __nv_bfloat16*>(x);
  p.dz = static_cast<const __nv_bfloat16*>(dz);
  p.dw = dw;
  p.batch = d->batch;
  p.h = d->height;
  p.w_ = d->width;
  p.cin = d->cin;
  p.cout = d->cout;
  p.ks = d->ksize;
  p.xs = x_stride;
  p.dzs = dz_stride;
  p.ntile = pick_ntile(d->cout);
  p.tmem_cols = pow2_cols(p.ntile);
  const long long npix = (long long)d->batch * d->height * d->width;
  const long long nchunks = (npix + kWgradK - 1) / kWgradK;
  const int tiles = ((rows + kTileM - 1) / kTileM) * (d->cout / p.ntile);
  const long long sms = device_sms();
  long long splits = std::max(1ll, std::min(nchunks, (4ll * sms + tiles - 1) / tiles));
  p.chunks_per_split = (nchunks + splits - 1) / splits;
  splits = (nchunks + p.chunks_per_split - 1) / p.chunks_per_split;
  const int stage = (kTileM + p.ntile) * kWgradK * 2;
  const int smem = smem_for(stage, p.tmem_cols);
  dim3 grid((unsigned)((rows + kTileM - 1) / kTileM), (unsigned)(d->cout / p.ntile), (unsigned)splits);
  conv_wgrad_kernel<<<grid, kThreads, smem, static_cast<cudaStream_t>(stream)>>>(p);
  return launch_status(fn);
}

extern "C" int shy_sg_bias_grad(int64_t pixels, int32_t channels, const void* dz, int32_t dz_stride, float* db,
                                void* stream) {
  if (pixels <= 0 || channels <= 0 || !dz || !db || dz_stride < channels) {
    set_error("shy_sg_bias_grad: bad arguments");
    return SHY_ERR_INVALID_ARG;
  }
  const auto st = static_cast<cudaStream_t>(stream);
  const __nv_bfloat16* g = static_cast<const __nv_bfloat16*>(dz);
  if (channels <= 256 && 256 % channels == 0) {
    bias_grad_kernel<<<grid_for(pixels * channels), 256, 0, st>>>(g, dz_stride, pixels, channels, db);
  } else {
    const long long sms4 = 4ll * device_sms();
    const long long per = std::max(64ll, (long long)(pixels + sms4 - 1) / sms4);
    bias_grad_any_kernel<<<(int)((pixels + per - 1) / per), 128, 0, st>>>(g, dz_stride, pixels, channels, per, db);
  }
  return launch_status("shy_sg_bias_grad");
}

extern "C" int shy_sg_gelu_backward(int64_t pixels, int32_t channels, const float* da, int32_t da_stride,
                                    int32_t da_offset, const float* z, int32_t z_stride, int32_t z_offset,
                                    void* dz, float* db, void* stream) {
  if (pixels <= 0 || channels <= 0 || channels % 8 || channels > 2048 || 256 % (channels / 8) || !da || !z ||
      !dz || !aligned16(da) || !aligned16(z) || !aligned16(dz) || da_stride % 4 || da_offset % 4 ||
      z_stride % 4 || z_offset % 4 || da_offset < 0 || z_offset < 0 || da_offset + channels > da_stride ||
      z_offset + channels > z_stride || pixels * (channels / 8) >= (1ll << 31)) {
    set_error("shy_sg_gelu_backward: bad arguments (channels a multiple of 8 with channels / 8 dividing 256; "
              "16-byte aligned tensors, strides and offsets multiples of 4)");
    return SHY_ERR_INVALID_ARG;
  }
  const long long n8 = pixels * (channels / 8);
  gelu_backward_kernel<<<grid_for(n8), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      (int)n8, channels / 8, da, da_stride, da_offset, z, z_stride, z_offset, static_cast<__nv_bfloat16*>(dz), db);
  return launch_status("shy_sg_gelu_backward");
}

namespace {
bool check_resample(int batch, int h, int w, int c, bool need_even, const char* fn) {
  if (batch <= 0 || h <= 0 || w <= 0 || c <= 0 || (need_even && ((h | w) & 1))) {
    shy::set_error("%s: bad shape %dx%dx%d c %d", fn, batch, h, w, c);
    return false;
  }
  return true;
}
bool check_vec(const void* p, int stride, int off, int c, const char* fn) {
  if (!p || !aligned16(p) || stride % 8 || off % 8 || c % 8 || off < 0 || off + c > stride) {
    shy::set_error("%s: bf16 tensors need 16-byte alignment, strides, offsets and channels in multiples of 8",
                   fn);
    return false;
  }
  return true;
}
bool check_scalar(const void* p, int stride, int off, int c, const char* fn) {
  if (!p || off < 0 || off + c > stride) {
    shy::set_error("%s: bad f32 tensor layout", fn);
    return false;
  }
  return true;
}
}  // namespace

extern "C" int shy_sg_pool_forward(int32_t batch, int32_t height, int32_t width, int32_t channels, const void* x,
                                   int32_t x_stride, int32_t x_offset, void* y, int32_t y_stride,
                                   int32_t y_offset, void* stream) {
  static const char* fn = "shy_sg_pool_forward";
  if (!check_resample(batch, height, width, channels, true, fn) ||
      !check_vec(x, x_stride, x_offset, channels, fn) || !check_vec(y, y_stride, y_offset, channels, fn))
    return SHY_ERR_INVALID_ARG;
  const long long n = (long long)batch * (height / 2) * (width / 2) * (channels / 8);
  pool_fwd_kernel<<<grid_for(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      batch, height, width, channels, static_cast<const __nv_bfloat16*>(x), x_stride, x_offset,
      static_cast<__nv_bfloat16*>(y), y_stride, y_offset);
  return launch_status(fn);
}

extern "C" int shy_sg_pool_backward(int32_t batch, int32_t height, int32_t width, int32_t channels,
                                    const float* dy, int32_t dy_stride, int32_t dy_offset, float* dx,
                                    int32_t dx_stride, int32_t dx_offset, void* stream) {
  static const char* fn = "shy_sg_pool_backward";
  if (!check_resample(batch, height, width, channels, true, fn) ||
      !check_scalar(dy, dy_stride, dy_offset, channels, fn) || !check_scalar(dx, dx_stride, dx_offset, channels, fn))
    return SHY_ERR_INVALID_ARG;
  const long long n = (long long)batch * height * width * channels;
  pool_bwd_kernel<<<grid_for(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      batch, height, width, channels, dy, dy_stride, dy_offset, dx, dx_stride, dx_offset);
  return launch_status(fn);
}

extern "C" int shy_sg_upsample_forward(int32_t batch, int32_t height, int32_t width, int32_t channels,
                                       const void* x, int32_t x_stride, int32_t x_offset, void* y, int32_t y_stride,
                                       int32_t y_offset, void* stream) {
  static const char* fn = "shy_sg_upsample_forward";
  if (!check_resample(batch, height, width, channels, false, fn) ||
      !check_vec(x, x_stride, x_offset, channels, fn) || !check_vec(y, y_stride, y_offset, channels, fn))
    return SHY_ERR_INVALID_ARG;
  const long long n = (long long)batch * (2 * height) * (2 * width) * (channels / 8);
  up_fwd_kernel<<<grid_for(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      batch, height, width, channels, static_cast<const __nv_bfloat16*>(x), x_stride, x_offset,
      static_cast<__nv_bfloat16*>(y), y_stride, y_offset);
  return launch_status(fn);
}

extern "C" int shy_sg_upsample_backward(int32_t batch, int32_t height, int32_t width, int32_t channels,
                                        const float* dy, int32_t dy_stride, int32_t dy_offset, float* dx,
                                        int32_t dx_stride, int32_t dx_offset, void* stream) {
  static const char* fn = "shy_sg_upsample_backward";
  if (!check_resample(batch, height, width, channels, false, fn) ||
      !check_scalar(dy, dy_stride, dy_offset, channels, fn) || !check_scalar(dx, dx_stride, dx_offset, channels, fn))
    return SHY_ERR_INVALID_ARG;
  const long long n = (long long)batch * height * width * channels;
  up_bwd_kernel<<<grid_for(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      batch, height, width, channels, dy, dy_stride, dy_offset, dx, dx_stride, dx_offset);
  return launch_status(fn);
}

extern "C" int shy_sg_weight_prep(int32_t cout, int32_t ksize, int32_t cin, const float* w, void* w_bf16,
                                  void* w_flip, void* stream) {
  if (cout <= 0 || cin <= 0 || (ksize != 1 && ksize != 3) || !w || !w_bf16) {
    set_error("shy_sg_weight_prep: bad arguments");
    return SHY_ERR_INVALID_ARG;
  }
  const long long n = (long long)cout * ksize * ksize * cin;
  weight_prep_kernel<<<grid_for(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      cout, ksize * ksize, cin, w, static_cast<__nv_bfloat16*>(w_bf16), static_cast<__nv_bfloat16*>(w_flip));
  return launch_status("shy_sg_weight_prep");
}

extern "C" int shy_sg_adamw(int64_t n, float* p, const float* g, float* m, float* v, const shy_sg_adamw_args* a,
                            void* stream) {
  if (n <= 0 || !p || !g || !m || !v || !a || !(a->bc1 > 0.0f) || !(a->bc2 > 0.0f)) {
    set_error("shy_sg_adamw: bad arguments");
    return SHY_ERR_INVALID_ARG;
  }
  adamw_kernel<<<grid_for(n), 256, 0, static_cast<cudaStream_t>(stream)>>>(n, p, g, m, v, *a);
  return launch_status("shy_sg_adamw");
}

extern "C" int shy_sg_features(int32_t batch, int32_t height, int32_t width, const float* h, const shy_sg_norm* n,
                               void* x, void* stream) {
  if (batch <= 0 || height <= 0 || width <= 0 || !h || !n || !x || !aligned16(x)) {
    set_error("shy_sg_features: bad arguments");
    return SHY_ERR_INVALID_ARG;
  }
  const long long npix = (long long)batch * height * width;
  features_kernel<<<grid_for(npix), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      batch, height, width, h, *n, static_cast<__nv_bfloat16*>(x));
  return launch_status("shy_sg_features");
}

extern "C" int shy_sg_loss(int64_t pixels, const float* z, int32_t z_stride, const float* target,
                           const float weights[3], void* dz, double* loss, void* stream) {
  if (pixels <= 0 || !z || z_stride < 3 || !target || !weights || !dz || !aligned16(dz) || !loss) {
    set_error("shy_sg_loss: bad arguments");
    return SHY_ERR_INVALID_ARG;
  }
  const float scale = (float)(1.0 / (3.0 * (double)pixels));
  loss_kernel<<<grid_for(pixels), 256, 0, static_cast<cudaStream_t>(stream)>>>(
      pixels, z, z_stride, target, weights[0], weights[1], weights[2], scale, static_cast<__nv_bfloat16*>(dz),
      loss);
  return launch_status("shy_sg_loss");
}

extern "C" int shy_sg_decode(int64_t pixels, const float* z, int32_t z_stride, const shy_sg_norm* n,
                             float* discharge, float* momentumx, float* momentumy, void* stream) {
  if (pixels <= 0 || !z || z_stride < 3 || !n || !discharge || !momentumx || !momentumy) {
    set_error("shy_sg_decode: bad arguments");
    return SHY_ERR_INVALID_ARG;
  }
  decode_kernel<<<grid_for(pixels), 256, 0, static_cast<cudaStream_t>(stream)>>>(pixels, z, z_stride, *n,
                                                                                 discharge, momentumx, momentumy);
  return launch_status("shy_sg_decode");
}

extern "C" int shy_sg_set_conv_path(int32_t path) {
  if (path != SHY_SG_CONV_TMA && path != SHY_SG_CONV_STAGED && path != SHY_SG_CONV_PERSISTENT) {
    set_error("shy_sg_set_conv_path: unknown path %d", path);
    return SHY_ERR_INVALID_ARG;
  }
  g_conv_path = path;
  return SHY_OK;
}

extern "C" int shy_sg_set_conv_tile(int32_t pixels, int32_t stages) {
  if ((pixels != 0 && pixels != 128 && pixels != 256 && pixels != 512) ||
      (stages != 0 && (stages < 2 || stages > kMaxStages))) {
    set_error("shy_sg_set_conv_tile: %d pixels (0, 128, 256 or 512), %d stages (0 or 2..%d)", pixels, stages,
              kMaxStages);
    return SHY_ERR_INVALID_ARG;
  }
  g_conv_pixels = pixels;
  g_conv_stages = stages;
  return SHY_OK;
}

extern "C" int shy_sg_set_wgrad_tile(int32_t pixels, int32_t stages) {
  if ((pixels != 0 && pixels != 64 && pixels != 128) || (stages != 0 && (stages < 2 || stages > kMaxStages))) {
    set_error("shy_sg_set_wgrad_tile: %d pixels (0, 64 or 128), %d stages (0 or 2..%d)", pixels, stages,
              kMaxStages);
    return SHY_ERR_INVALID_ARG;
  }
  g_wgrad_pixels = pixels;
  g_wgrad_stages = stages;
  return SHY_OK;
}

extern "C" int shy_sg_set_conv_tap_rows(int32_t rows) {
  if (rows != 1 && rows != 3) {
    set_error("shy_sg_set_conv_tap_rows: %d (1 or 3)", rows);
    return SHY_ERR_INVALID_ARG;
  }
  g_conv_tap_rows = rows;
  return SHY_OK;
}

extern "C" int shy_sg_status(void) {
  if (cudaDeviceSynchronize() != cudaSuccess) {
    set_error("shy_sg_status: %s", cudaGetErrorString(cudaGetLastError()));
    return SHY_ERR_CUDA;
  }
  int st = 0;
  const int zero = 0;
  if (cudaMemcpyFromSymbol(&st, g_sg_status, sizeof(int)) != cudaSuccess ||
      cudaMemcpyToSymbol(g_sg_status, &zero, sizeof(int)) != cudaSuccess) {
    set_error("shy_sg_status: %s", cudaGetErrorString(cudaGetLastError()));
    return SHY_ERR_CUDA;
  }
  if (st != 0) {
    set_error("surrogate tensor-core kernel gave up waiting on its MMAs");
    return st;
  }
  return SHY_OK;
}
