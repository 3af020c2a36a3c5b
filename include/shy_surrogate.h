/* shy_surrogate.h -- device kernels of the learned warm-start surrogate.
 *
 * The reference has no counterpart: its track maps start at zero and fill
 * through the lrate blend of World::erode (source/world.h:83-85).  The
 * surrogate predicts converged log-discharge and momentum maps from the
 * heightmap with a small convolutional U-Net and writes them into a world
 * before plain cycles continue (shy_world_set_field).  This header exposes
 * the network's building blocks: 3x3 and 1x1 convolutions as BF16 implicit
 * GEMMs on the tensor cores (tcgen05, FP32 accumulation in tensor memory),
 * their weight and input gradients, and the elementwise pieces of forward
 * and backward passes and of AdamW training.
 *
 * Tensors are NHWC.  Element (b, y, x, c) of a tensor with pixel stride s
 * and channel offset o lives at ((b*H + y)*W + x)*s + o + c.  bf16 tensors
 * read or written 8 channels at a time need 16-byte aligned base pointers
 * and strides and offsets that are multiples of 8.  f32 tensors written 8
 * channels at a time need 16-byte alignment and multiples of 4.
 *
 * Every pointer is a device pointer.  Every call is asynchronous on
 * `stream`, a cudaStream_t or NULL for the legacy default stream.  Every
 * call returns SHY_OK or a negative status and leaves a message in
 * shy_last_error(). */
#ifndef SHY_SURROGATE_H
#define SHY_SURROGATE_H

#include <stdint.h>

#include "shy.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Shape of one convolution: input and output share batch x height x width
 * (zero padding keeps the size); ksize is 1 or 3; cin and cout are
 * multiples of 16.  tile, stages and tap_rows tune the TMA pipeline for
 * this call (0: the process-wide setting, see shy_sg_set_conv_tile,
 * shy_sg_set_wgrad_tile and shy_sg_set_conv_tap_rows): pixels per tile
 * (forward 128, 256 or 512 -- 512 on the SHY_SG_CONV_TMA path only --,
 * weight gradient 64 or 128), stages (2..8), and taps
 * per stage of a 3x3 forward or input gradient (1 or 3). */
typedef struct shy_sg_conv_desc {
  int32_t batch, height, width;
  int32_t cin, cout, ksize;
  int32_t tile, stages, tap_rows;
} shy_sg_conv_desc;

#define SHY_SG_ACT_NONE 0
#define SHY_SG_ACT_GELU 1 /* 0.5 z (1 + erf(z / sqrt 2)) */

/* How the convolutions stage their operands (process-wide):
 * SHY_SG_CONV_TMA         tensor-memory-accelerator copies into a 2- to
 *                         8-stage pipeline, one CTA per tile (the default);
 * SHY_SG_CONV_STAGED      loads by the CTA's threads into two stages;
 * SHY_SG_CONV_PERSISTENT  the TMA pipeline in a persistent CTA per SM with
 *                         separate load, MMA and epilogue warps and two
 *                         accumulators, so one tile's epilogue runs under
 *                         the next tile's main loop (forward and input
 *                         gradient; the weight gradient runs as with TMA). */
#define SHY_SG_CONV_TMA 0
#define SHY_SG_CONV_STAGED 1
#define SHY_SG_CONV_PERSISTENT 2
int shy_sg_set_conv_path(int32_t path);
/* Tile and depth of the TMA pipeline (process-wide): pixels per tile (128,
 * or 256 / 512 with two / four accumulators sharing each weight chunk; 512
 * uses 32-channel chunks and all of the SM's tensor memory) and stages
 * (2..8, one channel chunk each); 0 for either (the default) chooses per
 * convolution.  Deeper pipelines keep more loads in flight; shallower ones
 * fit more CTAs on an SM. */
int shy_sg_set_conv_tile(int32_t pixels, int32_t stages);
/* Taps per pipeline stage of a 3x3 convolution on SHY_SG_CONV_TMA
 * (process-wide): 3 (the default: one input box two rows taller than the
 * tile serves a whole kernel column) or 1 (one box per tap). */
int shy_sg_set_conv_tap_rows(int32_t rows);
/* Pipeline of the TMA weight gradient (process-wide): pixels per stage (64
 * or 128, a tile of 16 x 4 or 16 x 8) and stages (2..8); 0 for either (the
 * default) chooses per convolution. */
int shy_sg_set_wgrad_tile(int32_t pixels, int32_t stages);

/* z = conv(x, w) + bias (bias may be NULL); written as f32 to `z` (may be
 * NULL) and as act(z) in bf16 to `a` (may be NULL).  x: bf16, pixel stride
 * x_stride.  w: bf16 [cout][ksize*ksize][cin] (tap = ky*ksize + kx).  The
 * input gradient of a convolution is this call on the output gradient with
 * the weights that shy_sg_weight_prep rotates by 180 degrees and
 * transposes, and cin and cout swapped. */
int shy_sg_conv_forward(const shy_sg_conv_desc* d, const void* x, int32_t x_stride,
                        const void* w, const float* bias, float* z, int32_t z_stride,
                        int32_t z_offset, void* a, int32_t a_stride, int32_t a_offset,
                        int32_t act, void* stream);

/* The input gradient of a convolution whose input is a GELU layer's output,
 * fused with that layer's backward pass: with d the input-gradient
 * convolution (cin = the forward's cout, cout = the forward's cin) and
 * w_flip from shy_sg_weight_prep,
 *   dz_prev[pixel][c] = bf16(conv(dz, w_flip)[pixel][c] * gelu'(z_prev[pixel][c]))
 * (bf16, pixel stride d->cout).  z_prev is f32 with its own stride and
 * offset (16-byte aligned, multiples of 4).  The GELU layer's bias gradient
 * is shy_sg_bias_grad of dz_prev. */
int shy_sg_conv_input_grad(const shy_sg_conv_desc* d, const void* dz, int32_t dz_stride,
                           const void* w_flip, const float* z_prev, int32_t zp_stride,
                           int32_t zp_offset, void* dz_prev, void* stream);

/* dw[cout][tap][cin] += sum over pixels of dz[pixel][cout] * x[pixel + tap][cin]
 * (x zero outside the image).  x, dz: bf16; dw: f32, accumulated with
 * atomics, so the summation order varies from run to run. */
int shy_sg_conv_wgrad(const shy_sg_conv_desc* d, const void* x, int32_t x_stride,
                      const void* dz, int32_t dz_stride, float* dw, void* stream);

/* db[c] += sum over pixels of dz[pixel][c]; dz bf16. */
int shy_sg_bias_grad(int64_t pixels, int32_t channels, const void* dz, int32_t dz_stride,
                     float* db, void* stream);

/* dz[pixel][c] = bf16(da * gelu'(z)); da, z: f32 with their own stride and
 * offset (16-byte aligned, multiples of 4); dz: bf16, pixel stride
 * `channels`, a multiple of 8 with channels / 8 dividing 256.  If db is not
 * NULL, db[c] += the sum of dz[.][c] over pixels as well: the bias gradient
 * of the convolution whose output gradient dz is. */
int shy_sg_gelu_backward(int64_t pixels, int32_t channels, const float* da, int32_t da_stride,
                         int32_t da_offset, const float* z, int32_t z_stride, int32_t z_offset,
                         void* dz, float* db, void* stream);

/* 2 x 2 average pooling, bf16 -> bf16.  height, width: the input's (even). */
int shy_sg_pool_forward(int32_t batch, int32_t height, int32_t width, int32_t channels,
                        const void* x, int32_t x_stride, int32_t x_offset, void* y,
                        int32_t y_stride, int32_t y_offset, void* stream);
/* dx += 0.25 * dy of the pooled pixel; f32.  height, width: the input's. */
int shy_sg_pool_backward(int32_t batch, int32_t height, int32_t width, int32_t channels,
                         const float* dy, int32_t dy_stride, int32_t dy_offset, float* dx,
                         int32_t dx_stride, int32_t dx_offset, void* stream);
/* Nearest-neighbour 2x upsampling, bf16 -> bf16.  height, width: the
 * input's (the coarse grid). */
int shy_sg_upsample_forward(int32_t batch, int32_t height, int32_t width, int32_t channels,
                            const void* x, int32_t x_stride, int32_t x_offset, void* y,
                            int32_t y_stride, int32_t y_offset, void* stream);
/* dx += sum of dy over the four fine pixels; f32.  height, width: coarse. */
int shy_sg_upsample_backward(int32_t batch, int32_t height, int32_t width, int32_t channels,
                             const float* dy, int32_t dy_stride, int32_t dy_offset, float* dx,
                             int32_t dx_stride, int32_t dx_offset, void* stream);

/* From the f32 master weights w[cout][tap][cin]: w_bf16 (same layout) and,
 * if w_flip is not NULL, w_flip[cin][taps-1-tap][cout] in bf16, the
 * weights of the input-gradient convolution. */
int shy_sg_weight_prep(int32_t cout, int32_t ksize, int32_t cin, const float* w, void* w_bf16,
                       void* w_flip, void* stream);

/* One AdamW step over n parameters (decoupled weight decay):
 *   m = b1 m + (1-b1) g;  v = b2 v + (1-b2) g^2
 *   p -= lr * ((m / bc1) / (sqrt(v / bc2) + eps) + wd * p)
 * with bc1 = 1 - b1^t and bc2 = 1 - b2^t given by the caller. */
typedef struct shy_sg_adamw_args {
  float lr, beta1, beta2, eps, weight_decay, bc1, bc2;
} shy_sg_adamw_args;
int shy_sg_adamw(int64_t n, float* p, const float* g, float* m, float* v,
                 const shy_sg_adamw_args* a, void* stream);

/* Input and output scaling of the network. */
typedef struct shy_sg_norm {
  float height_mean, height_scale; /* channel 0: (h - mean) * scale */
  float slope_scale;               /* channels 1, 2: central differences * scale */
  float out_mean[3], out_scale[3]; /* log1p(discharge), momentum x, momentum y */
} shy_sg_norm;

/* Network input from heightmaps h[batch][height][width] (f32, a world's
 * x-major map is an image with height = nx, width = ny): bf16, 16 channels
 * per pixel: normalised height, the two central differences (one-sided at
 * the border), zeros. */
int shy_sg_features(int32_t batch, int32_t height, int32_t width, const float* h,
                    const shy_sg_norm* n, void* x, void* stream);

/* Mean squared error of the first three channels of z (f32, pixel stride
 * z_stride) against target[pixel][3] (f32, normalised), channel c weighted
 * by weights[c]: loss += sum w_c (z_c - t_c)^2 / (3 * pixels) (a device
 * double), and dz (bf16, 16 channels per pixel) = its gradient, zero in
 * channels 3..15. */
int shy_sg_loss(int64_t pixels, const float* z, int32_t z_stride, const float* target,
                const float weights[3], void* dz, double* loss, void* stream);

/* Network output to maps: discharge = max(0, expm1(z0 * s0 + m0)),
 * momentum x = z1 * s1 + m1, momentum y = z2 * s2 + m2. */
int shy_sg_decode(int64_t pixels, const float* z, int32_t z_stride, const shy_sg_norm* n,
                  float* discharge, float* momentumx, float* momentumy, void* stream);

/* Synchronises the device and returns (and clears) the status of the
 * surrogate kernels' bounded waits: SHY_OK, or SHY_ERR_TIMEOUT if a
 * tensor-core kernel gave up waiting on its MMAs. */
int shy_sg_status(void);

#ifdef __cplusplus
}
#endif

#endif /* SHY_SURROGATE_H */
