// shy_probe.cu -- L2 peaks of this device, measured by the library itself.
//
// The batched erosion kernel keeps a 1024^2 terrain's cell state in L2, so
// its roofline is the L2's, not HBM's.  shy_measure_l2 measures the figures
// that roofline needs on the device at hand:
//   read_gbs                   streaming 16-byte loads that bypass L1, over a
//                              buffer a quarter of the L2 (at most 32 MiB)
//   random_sector_reads_per_s  8-byte loads, each to a different 32-byte
//                              sector picked at random in that buffer (the
//                              access pattern of a drop-step's cell loads)
//   red_per_s                  64-bit integer atomic additions without return
//                              to random addresses of an 8 MiB table (the
//                              drop-step's scatter)
// Each is timed with CUDA events after one untimed pass that brings the
// buffer into L2.
#include "shy_device.cuh"

namespace shy {

namespace {

__device__ __forceinline__ unsigned long long mix64(unsigned long long z) {
  z += 0x9E3779B97F4A7C15ull;
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

__global__ void stream_read_kernel(const uint4* __restrict__ buf, long long n, int passes,
                                   unsigned* __restrict__ sink) {
  unsigned acc = 0;
  const long long G = (long long)gridDim.x * blockDim.x;
  for (int p = 0; p < passes; ++p)
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += G) {
      const uint4 v = __ldcg(buf + i);
      acc ^= v.x ^ v.y ^ v.z ^ v.w;
    }
  if (acc == 0x9E3779B9u) sink[0] = acc;  // keeps the loads
}

// kLoads independent loads in flight per thread and round
__global__ void random_sector_kernel(const unsigned long long* __restrict__ buf, long long sectors, int rounds,
                                     unsigned long long* __restrict__ sink) {
  const int kLoads = 8;
  const unsigned long long t = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
  unsigned long long acc = 0;
  for (int r = 0; r < rounds; ++r) {
    unsigned long long v[kLoads];
#pragma unroll
    for (int k = 0; k < kLoads; ++k) {
      const unsigned long long s = mix64(t * 0x100000001B3ull + (unsigned long long)(r * kLoads + k)) % sectors;
      v[k] = __ldcg(buf + s * 4);  // one 8-byte word of sector s
    }
#pragma unroll
    for (int k = 0; k < kLoads; ++k) acc += v[k];
  }
  if (acc == 0x9E3779B97F4A7C15ull) sink[0] = acc;
}

__global__ void random_red_kernel(unsigned long long* __restrict__ table, long long n, int per_thread) {
  const unsigned long long t = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
  for (int k = 0; k < per_thread; ++k) {
    const unsigned long long s = mix64(t * 0x100000001B3ull + (unsigned long long)k) % (unsigned long long)n;
    atomicAdd(table + s, 1ull);
  }
}

struct ProbeBuffers {
  void* buf = nullptr;
  void* table = nullptr;
  void* sink = nullptr;
  cudaStream_t stream = nullptr;
  cudaEvent_t a = nullptr, b = nullptr;
  ~ProbeBuffers() {
    if (stream) cudaStreamSynchronize(stream);
    if (buf) cudaFree(buf);
    if (table) cudaFree(table);
    if (sink) cudaFree(sink);
    if (a) cudaEventDestroy(a);
    if (b) cudaEventDestroy(b);
    if (stream) cudaStreamDestroy(stream);
  }
};

// milliseconds of `launch` (enqueued on pb.stream) between two events
template <class F>
cudaError_t timed(ProbeBuffers& pb, F launch, float* ms) {
  cudaError_t e;
  if ((e = cudaEventRecord(pb.a, pb.stream)) != cudaSuccess) return e;
  launch();
  if ((e = cudaGetLastError()) != cudaSuccess) return e;
  if ((e = cudaEventRecord(pb.b, pb.stream)) != cudaSuccess) return e;
  if ((e = cudaEventSynchronize(pb.b)) != cudaSuccess) return e;
  return cudaEventElapsedTime(ms, pb.a, pb.b);
}

int measure(int device, shy_l2_probe* out) {
  int sms = 0, l2 = 0;
  SHY_CHECK_CUDA(cudaSetDevice(device), "select device");
  SHY_CHECK_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, device), "query SMs");
  SHY_CHECK_CUDA(cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, device), "query L2 size");
  long long bytes = (long long)l2 / 4;
  if (bytes > (32ll << 20)) bytes = 32ll << 20;
  bytes &= ~255ll;
  if (bytes < (1 << 20)) bytes = 1 << 20;
  const long long table_n = (8ll << 20) / 8;
  ProbeBuffers pb;
  SHY_CHECK_CUDA(cudaStreamCreateWithFlags(&pb.stream, cudaStreamNonBlocking), "create stream");
  SHY_CHECK_CUDA(cudaEventCreate(&pb.a), "create event");
  SHY_CHECK_CUDA(cudaEventCreate(&pb.b), "create event");
  SHY_CHECK_CUDA(cudaMalloc(&pb.buf, (size_t)bytes), "allocate probe buffer");
  SHY_CHECK_CUDA(cudaMalloc(&pb.table, (size_t)table_n * 8), "allocate probe table");
  SHY_CHECK_CUDA(cudaMalloc(&pb.sink, 64), "allocate probe sink");
  SHY_CHECK_CUDA(cudaMemsetAsync(pb.buf, 1, (size_t)bytes, pb.stream), "fill probe buffer");
  SHY_CHECK_CUDA(cudaMemsetAsync(pb.table, 0, (size_t)table_n * 8, pb.stream), "clear probe table");

  const int grid = sms * 8, block = 256;
  const long long n16 = bytes / 16;
  const int passes = 20;
  float ms = 0.0f;
  auto stream_run = [&](int p) {
    stream_read_kernel<<<grid, block, 0, pb.stream>>>((const uint4*)pb.buf, n16, p, (unsigned*)pb.sink);
  };
  SHY_CHECK_CUDA(timed(pb, [&] { stream_run(1); }, &ms), "L2 read probe");
  SHY_CHECK_CUDA(timed(pb, [&] { stream_run(passes); }, &ms), "L2 read probe");
  out->read_gbs = (double)bytes * passes / (ms * 1e-3) / 1e9;

  const long long sectors = bytes / 32;
  const int rounds = 64;
  auto sector_run = [&](int r) {
    random_sector_kernel<<<grid, block, 0, pb.stream>>>((const unsigned long long*)pb.buf, sectors, r,
                                                         (unsigned long long*)pb.sink);
  };
  SHY_CHECK_CUDA(timed(pb, [&] { sector_run(4); }, &ms), "L2 sector probe");
  SHY_CHECK_CUDA(timed(pb, [&] { sector_run(rounds); }, &ms), "L2 sector probe");
  out->random_sector_reads_per_s = (double)grid * block * rounds * 8 / (ms * 1e-3);

  const int per_thread = 64;
  auto red_run = [&](int k) {
    random_red_kernel<<<grid, block, 0, pb.stream>>>((unsigned long long*)pb.table, table_n, k);
  };
  SHY_CHECK_CUDA(timed(pb, [&] { red_run(4); }, &ms), "L2 atomic probe");
  SHY_CHECK_CUDA(timed(pb, [&] { red_run(per_thread); }, &ms), "L2 atomic probe");
  out->red_per_s = (double)grid * block * per_thread / (ms * 1e-3);
  out->l2_bytes = (uint64_t)l2;
  out->buffer_bytes = (uint64_t)bytes;
  return SHY_OK;
}

// Every float with |v| < 2^31 (and no NaN or infinity): the hardware
// float -> 32.32 conversion against the integer restatement.
__global__ void check_q32_kernel(unsigned long long* bad) {
  unsigned long long n = 0;
  for (unsigned long long u = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; u < (1ull << 32);
       u += (unsigned long long)gridDim.x * blockDim.x) {
    const float v = __uint_as_float((unsigned)u);
    if (!(fabsf(v) < 2147483648.0f)) continue;
    n += shy_q32_dev(v) != shy_q32(v);
  }
  if (n) atomicAdd(bad, n);
}

// 32.32 -> float: every q with |q| < 2^26, every power of two with its
// neighbours, and 2^30 values spread over the whole int64 range.
__global__ void check_unq_kernel(unsigned long long* bad) {
  unsigned long long n = 0;
  const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  const unsigned long long tid = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x;
  auto test = [&](long long q) { n += __float_as_uint(shy_unq_dev(q)) != __float_as_uint(shy_unq(q)); };
  for (unsigned long long i = tid; i < (1ull << 27); i += stride) test((long long)i - (1ll << 26));
  for (unsigned long long i = tid; i < 63 * 64; i += stride) {
    const long long p = 1ll << (i / 64);
    const long long d = (long long)(i % 64) - 32;
    test(p + d);
    test(-(p + d));
  }
  for (unsigned long long i = tid; i < (1ull << 30); i += stride) {
    unsigned long long z = (i + 1) * 0x9E3779B97F4A7C15ull;  // SplitMix64 finaliser
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    test((long long)(z >> (i & 63)));  // magnitudes of every size, both signs
    test((long long)(0ull - (z >> (i & 63))));
  }
  if (n) atomicAdd(bad, n);
}

// Every float: the float-float erf against the FP64 evaluation whose
// rounding it reproduces (NaN inputs must give NaN).
__global__ void check_erf_kernel(unsigned long long* bad) {
  unsigned long long n = 0;
  for (unsigned long long u = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; u < (1ull << 32);
       u += (unsigned long long)gridDim.x * blockDim.x) {
    const float v = __uint_as_float((unsigned)u);
    const float a = shy_erff_ff(v), b = shy_erff(v);
    n += (a == a || b == b) && __float_as_uint(a) != __float_as_uint(b);
  }
  if (n) atomicAdd(bad, n);
}

// Every float: the float edge height h - 0.002 against the double expression.
__global__ void check_edge_kernel(unsigned long long* bad) {
  unsigned long long n = 0;
  for (unsigned long long u = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; u < (1ull << 32);
       u += (unsigned long long)gridDim.x * blockDim.x) {
    const float v = __uint_as_float((unsigned)u);
    const float a = shy_minus_0002(v), b = (float)((double)v - 0.002);
    n += (a == a || b == b) && __float_as_uint(a) != __float_as_uint(b);
  }
  if (n) atomicAdd(bad, n);
}

// Every positive float: the float evaporation division against the integer
// restatement, and the float volume evaporation against the double
// expression, for the evaporation constant `E`.
__global__ void check_evap_kernel(shy_evap E, unsigned long long* bad) {
  unsigned long long n = 0;
  for (unsigned long long u = blockIdx.x * (unsigned long long)blockDim.x + threadIdx.x; u < 0x7F800000ull;
       u += (unsigned long long)gridDim.x * blockDim.x) {
    const float v = __uint_as_float((unsigned)u);
    n += __float_as_uint(shy_evap_div_ff(v, &E)) != __float_as_uint(shy_evap_div(v, &E));
    n += __float_as_uint(shy_evap_mul_ff(v, &E)) != __float_as_uint((float)((double)v * E.c));
  }
  if (n) atomicAdd(bad, n);
}

}  // namespace

}  // namespace shy

using namespace shy;

extern "C" int shy_check_conversions(uint64_t* mismatches) {
  if (!mismatches) {
    set_error("shy_check_conversions: null output");
    return SHY_ERR_INVALID_ARG;
  }
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
    cudaGetLastError();
    set_error("shy_check_conversions: no CUDA device");
    return SHY_ERR_NO_DEVICE;
  }
  unsigned long long* bad = nullptr;
  SHY_CHECK_CUDA(cudaMalloc((void**)&bad, 5 * sizeof(unsigned long long)), "allocate check counters");
  cudaError_t e = cudaMemset(bad, 0, 5 * sizeof(unsigned long long));
  if (e == cudaSuccess) {
    shy_params P;
    shy_params_default(&P);
    check_q32_kernel<<<4096, 256>>>(bad);
    check_unq_kernel<<<4096, 256>>>(bad + 1);
    check_erf_kernel<<<4096, 256>>>(bad + 2);
    // the default evaporation rate and three others
    const float rates[4] = {P.evap_rate, 0.0005f, 0.01f, 0.1f};
    for (float r : rates) check_evap_kernel<<<4096, 256>>>(shy_evap_make(r), bad + 3);
    check_edge_kernel<<<4096, 256>>>(bad + 4);
    e = cudaGetLastError();
  }
  unsigned long long h[5] = {0, 0, 0, 0, 0};
  if (e == cudaSuccess) e = cudaMemcpy(h, bad, sizeof(h), cudaMemcpyDeviceToHost);
  cudaFree(bad);
  if (e != cudaSuccess) {
    set_error("shy_check_conversions: %s", cudaGetErrorString(e));
    return e == cudaErrorMemoryAllocation ? SHY_ERR_OUT_OF_MEMORY : SHY_ERR_CUDA;
  }
  mismatches[0] = h[0];
  mismatches[1] = h[1];
  mismatches[2] = h[2];
  mismatches[3] = h[3];
  mismatches[4] = h[4];
  return SHY_OK;
}

extern "C" int shy_measure_l2(int device, shy_l2_probe* out) {
  if (!out) {
    set_error("shy_measure_l2: null output");
    return SHY_ERR_INVALID_ARG;
  }
  int n = 0;
  if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
    cudaGetLastError();
    set_error("shy_measure_l2: no CUDA device");
    return SHY_ERR_NO_DEVICE;
  }
  if (device < 0 || device >= n) {
    set_error("shy_measure_l2: device %d out of range (%d devices)", device, n);
    return SHY_ERR_INVALID_ARG;
  }
  int prev = 0;
  cudaGetDevice(&prev);
  const int rc = measure(device, out);
  cudaSetDevice(prev);
  return rc;
}
