// A C++ host using the surrogate's C ABI (include/shy_surrogate.h) with no
// Python: one 3x3 convolution forward and its weight gradient on the GPU,
// checked against loops on the host.  Prints "ok <max relative error>".
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <string.h>

#include <cmath>
#include <random>
#include <vector>

#include "shy_surrogate.h"

static uint16_t to_bf16(float f) {  // round to nearest even
  uint32_t u;
  memcpy(&u, &f, 4);
  u += 0x7FFFu + ((u >> 16) & 1u);
  return (uint16_t)(u >> 16);
}
static float from_bf16(uint16_t h) {
  uint32_t u = (uint32_t)h << 16;
  float f;
  memcpy(&f, &u, 4);
  return f;
}

int main() {
  const int B = 1, H = 24, W = 20, CI = 32, CO = 64, K = 3, T = K * K;
  const int P = B * H * W;
  std::mt19937 rng(7);
  std::normal_distribution<float> nd(0.0f, 1.0f);
  std::vector<uint16_t> x(P * CI), w(CO * T * CI), dz(P * CO);
  std::vector<float> bias(CO);
  for (auto& v : x) v = to_bf16(nd(rng));
  for (auto& v : w) v = to_bf16(nd(rng) * 0.1f);
  for (auto& v : dz) v = to_bf16(nd(rng));
  for (auto& v : bias) v = nd(rng);

  void *dx, *dw, *ddz;
  float *dbias, *dzout, *dgw;
  if (cudaMalloc(&dx, x.size() * 2) || cudaMalloc(&dw, w.size() * 2) || cudaMalloc(&ddz, dz.size() * 2) ||
      cudaMalloc((void**)&dbias, CO * 4) || cudaMalloc((void**)&dzout, (size_t)P * CO * 4) ||
      cudaMalloc((void**)&dgw, w.size() * 4)) {
    fprintf(stderr, "cudaMalloc failed\n");
    return 2;
  }
  cudaMemcpy(dx, x.data(), x.size() * 2, cudaMemcpyHostToDevice);
  cudaMemcpy(dw, w.data(), w.size() * 2, cudaMemcpyHostToDevice);
  cudaMemcpy(ddz, dz.data(), dz.size() * 2, cudaMemcpyHostToDevice);
  cudaMemcpy(dbias, bias.data(), CO * 4, cudaMemcpyHostToDevice);
  cudaMemset(dgw, 0, w.size() * 4);

  shy_sg_conv_desc d = {B, H, W, CI, CO, K};
  if (shy_sg_conv_forward(&d, dx, CI, dw, dbias, dzout, CO, 0, nullptr, 0, 0, SHY_SG_ACT_NONE, nullptr) != SHY_OK ||
      shy_sg_conv_wgrad(&d, dx, CI, ddz, CO, dgw, nullptr) != SHY_OK || shy_sg_status() != SHY_OK) {
    fprintf(stderr, "%s\n", shy_last_error());
    return 1;
  }
  std::vector<float> z((size_t)P * CO), gw(w.size());
  cudaMemcpy(z.data(), dzout, z.size() * 4, cudaMemcpyDeviceToHost);
  cudaMemcpy(gw.data(), dgw, gw.size() * 4, cudaMemcpyDeviceToHost);

  double worst = 0.0;
  std::vector<double> gref(w.size(), 0.0), gabs(w.size(), 0.0);
  for (int y = 0; y < H; ++y)
    for (int xx = 0; xx < W; ++xx)
      for (int o = 0; o < CO; ++o) {
        double s = bias[o], a = std::fabs(bias[o]);
        for (int t = 0; t < T; ++t) {
          const int yy = y + t / K - 1, xs = xx + t % K - 1;
          if (yy < 0 || yy >= H || xs < 0 || xs >= W) continue;
          for (int c = 0; c < CI; ++c) {
            const double p = (double)from_bf16(w[(o * T + t) * CI + c]) * from_bf16(x[(yy * W + xs) * CI + c]);
            s += p;
            a += std::fabs(p);
            const double g = (double)from_bf16(dz[(y * W + xx) * CO + o]) * from_bf16(x[(yy * W + xs) * CI + c]);
            gref[(o * T + t) * CI + c] += g;
            gabs[(o * T + t) * CI + c] += std::fabs(g);
          }
        }
        const double err = std::fabs(z[(y * W + xx) * CO + o] - s);
        if (err > 1e-5 * a + 1e-6) {
          fprintf(stderr, "forward mismatch at %d %d %d: %g vs %g\n", y, xx, o, z[(y * W + xx) * CO + o], s);
          return 1;
        }
        worst = std::fmax(worst, err / (a + 1e-30));
      }
  for (size_t i = 0; i < gw.size(); ++i) {
    const double err = std::fabs(gw[i] - gref[i]);
    if (err > 1e-5 * gabs[i] + 1e-6) {
      fprintf(stderr, "weight gradient mismatch at %zu: %g vs %g\n", i, gw[i], gref[i]);
      return 1;
    }
    worst = std::fmax(worst, err / (gabs[i] + 1e-30));
  }
  printf("ok %.3g\n", worst);
  cudaFree(dx);
  cudaFree(dw);
  cudaFree(ddz);
  cudaFree(dbias);
  cudaFree(dzout);
  cudaFree(dgw);
  return 0;
}
