/* asuna_denoise.h — C ABI of the learned denoiser.
 *
 * Replaces the reference's denoise step, DenoiserOptix::denoiseImageBuffer
 * (src/tracer/denoiser.cpp:143-224, driven by Tracer::denoise at
 * src/tracer/tracer.cpp:531-573): radiance with albedo (multi_channel[0],
 * "diffuse") and normal (multi_channel[1]) guides in, denoised radiance out.
 * The reference calls the closed OptiX AOV denoiser; here a U-Net with
 * hand-written BF16 tensor-core kernels (FP32 accumulation) takes its place,
 * trained on low/high sample-count pairs the renderer produces.
 *
 * Network: levels L (default 5) with channels c[0..L-1] (default
 * 32/48/64/96/128).  Encoder level l: two 3x3 conv + ReLU, then 2x2 average
 * pooling; decoder level l: nearest x2 upsampling, concatenation with the
 * encoder output of level l, two 3x3 conv + ReLU; a 3x3 head gives a residual
 * added to log1p(radiance).  Input channels (padded to 16): log1p(radiance),
 * albedo, normal, log2(1 + filter-weight sum) / 16.  Activations NHWC bf16; images are padded to multiples of
 * 2^(L-1) internally.
 *
 * Parameter layout (asuna_denoiser_get_params / set_params / get_grads): for
 * each convolution in order (encoder 0..L-1 conv1, conv2; decoder L-2..0
 * conv1, conv2; head), its weights [cout][3*3][cin] then its bias [cout], as
 * float32.  cin of encoder conv1 of level 0 is 16; the head has cout 16, of
 * which outputs 0..2 are used.
 *
 * Images passed as `const float*` are DEVICE pointers to n images of h x w
 * RGBA32F pixels, contiguous (the layout of a film image).  All calls are
 * asynchronous on the context's stream unless they return host values.
 */
#ifndef ASUNA_DENOISE_H
#define ASUNA_DENOISE_H

#include <stdint.h>

#include "asuna_rt.h"

#ifdef __cplusplus
extern "C" {
#endif

#define ASUNA_DENOISER_MAX_LEVELS 6

/* Training losses (asuna_denoiser_opts.loss). */
enum {
  ASUNA_DENOISER_LOSS_L1_LOG = 0, /* mean |log1p(out) - log1p(target)| */
  ASUNA_DENOISER_LOSS_RELMSE = 1  /* mean (out - target)^2 / (out + 0.01)^2, the
                                     denominator held fixed: unbiased with noisy targets */
};

typedef struct asuna_denoiser_opts {
  uint32_t levels;                               /* 2..6, default 5 */
  uint32_t channels[ASUNA_DENOISER_MAX_LEVELS];  /* multiples of 16 */
  uint64_t seed;                                 /* He-normal initialisation */
  uint64_t max_pixels;                           /* n*h*w of the largest call (padded) */
  uint32_t training;                             /* 1: allocate gradient and Adam state */
  uint32_t tensor_memory;                        /* 1: forward and input-gradient convolutions on tcgen05
                                                    (TMEM accumulators, TMA; the faster path); 0: mma.sync */
  uint32_t loss;                                 /* ASUNA_DENOISER_LOSS_*, used by asuna_denoiser_loss_grad */
} asuna_denoiser_opts;

typedef struct asuna_denoiser asuna_denoiser;

int asuna_denoiser_create(asuna_ctx* ctx, const asuna_denoiser_opts* opts, asuna_denoiser** out);
int asuna_denoiser_destroy(asuna_denoiser* d);
uint64_t asuna_denoiser_num_params(const asuna_denoiser* d);
int asuna_denoiser_get_params(asuna_denoiser* d, float* host, uint64_t n);
int asuna_denoiser_set_params(asuna_denoiser* d, const float* host, uint64_t n);
int asuna_denoiser_get_grads(asuna_denoiser* d, float* host, uint64_t n);

/* Forward pass: out = expm1(log1p(radiance) + head), clamped at 0 (RGBA, alpha 1).
 * `weight` is the film's filter-weight sum image (image 8; NULL = unknown):
 * it tells the network how many samples the radiance holds.  `noise`
 * (RGBA, NULL = unknown) estimates, per pixel and channel, the standard
 * deviation of `radiance`: where it is known (two independent half renders
 * give it) the network sees how much noise there is at each pixel. */
int asuna_denoiser_forward(asuna_denoiser* d, const float* radiance, const float* albedo, const float* normal,
                           const float* weight, const float* noise, uint32_t n, uint32_t h, uint32_t w, float* out);
/* Zeroes the gradients, runs forward, the loss chosen at creation against
 * `target` (mean over valid pixels and 3 channels) and the backward pass.
 * *loss (host) receives the loss; the call synchronises the stream. */
int asuna_denoiser_loss_grad(asuna_denoiser* d, const float* radiance, const float* albedo, const float* normal,
                             const float* weight, const float* noise, const float* target, uint32_t n, uint32_t h,
                             uint32_t w, float* loss);
/* One Adam step (bias-corrected) on the gradients of the last loss_grad. */
int asuna_denoiser_adam(asuna_denoiser* d, float lr, float beta1, float beta2, float eps);

/* Denoises image 0 of `film` (radiance) with guides `albedo_image` and
 * `normal_image` (film image indices 1..7; -1 = none) into `out` (device,
 * film-sized RGBA32F).  Stands in for DenoiserOptix::denoiseImageBuffer. */
int asuna_denoise(asuna_ctx* ctx, asuna_denoiser* d, asuna_film* film, int albedo_image, int normal_image,
                  float* out);

/* Error estimate of the denoised image from two independent half renders
 * `a` and `b` of the same shot (disjoint frames, equal counts; their
 * difference also gives the network its per-pixel noise input): with D the
 * denoised a,  err_denoised^2 = mean((D - b)^2) - mean((a - b)^2) / 2  and
 * err_plain^2 = mean((a - b)^2) / 4  estimate the RMSE of D and of the plain
 * average of a and b against the converged image (means over pixels and RGB).
 * The caller takes the plain path when err_denoised exceeds its threshold or
 * err_plain.  Writes D into `out` (device, film-sized RGBA32F). */
int asuna_denoise_estimate(asuna_ctx* ctx, asuna_denoiser* d, asuna_film* a, asuna_film* b, int albedo_image,
                           int normal_image, float* out, double* err_denoised, double* err_plain);
/* Denoises all samples of the two half renders (radiance (a + b) / 2, weight
 * a + b, guides of a) into `out` and estimates the RMSE of that output:
 * with D_a, D_b the denoised halves, var = mean((D_a - D_b)^2) / 2 is the
 * output variance of a half, and doubling the samples is taken to halve it
 * and keep the bias, so err_denoised^2 = err^2(D_a) - var / 2 (err(D_a) as in
 * asuna_denoise_estimate).  err_plain estimates the plain average of a, b. */
int asuna_denoise_combined(asuna_ctx* ctx, asuna_denoiser* d, asuna_film* a, asuna_film* b, int albedo_image,
                           int normal_image, float* out, double* err_denoised, double* err_plain);
/* Blends the all-sample denoise with the plain average of the two half
 * renders: out = w D(a + b) + (1 - w) (a + b) / 2 (rgb), with w in [0, 1]
 * chosen to minimise the estimated RMSE against the converged image.  The
 * estimate judges the half blend w D_a + (1 - w) a by b (its error^2 is the
 * mean square difference less the variance of b, mean((a - b)^2) / 2) and
 * takes a quarter of the halves' blend difference, mean((X_a - X_b)^2) / 4,
 * off for doubling the samples; both are quadratic in w.  w = 0 is the plain
 * average (err_plain); *err_out is the estimate at the chosen *weight. */
int asuna_denoise_blended(asuna_ctx* ctx, asuna_denoiser* d, asuna_film* a, asuna_film* b, int albedo_image,
                          int normal_image, float* out, double* err_out, double* err_plain, double* weight);

/* Device-side building blocks (raw device pointers, NHWC bf16, the context
 * stream as `stream`); exported for kernel-level tests.  cin % 16 == 0 and
 * cout % 8 == 0 for the convolutions. */
int asuna_nn_conv3x3(void* stream, const void* in, int n, int h, int w, int cin, const void* weight, const float* bias,
                     int cout, int relu, const void* mask, void* out, int out_f32);
int asuna_nn_conv3x3_wgrad(void* stream, const void* dz, const void* x, int n, int h, int w, int cin, int cout,
                           float* dweight);
int asuna_nn_bias_grad(void* stream, const void* dz, int pixels, int c, float* dbias);
int asuna_nn_flip_weights(void* stream, const void* w, void* wt, int cout, int cin);
int asuna_nn_avgpool2(void* stream, const void* in, void* out, int n, int h, int w, int c);
int asuna_nn_avgpool2_bwd(void* stream, const void* dout, void* din, int n, int h, int w, int c, int accumulate);
int asuna_nn_upsample2(void* stream, const void* in, void* out, int n, int h, int w, int c, int ctot, int coff);
int asuna_nn_upsample2_bwd(void* stream, const void* dout, void* din, int n, int h, int w, int c, int ctot, int coff);
int asuna_nn_copy_channels(void* stream, const void* src, int csrc, int soff, void* dst, int cdst, int doff, int c,
                           uint64_t pixels, int accumulate);
int asuna_nn_relu_mask(void* stream, void* grad, const void* y, uint64_t count);
/* The same convolution on the fifth-generation tensor cores: tcgen05.mma
 * with the accumulator in tensor memory, TMA-staged operands, weights in
 * the layout asuna_nn_weights_tc makes ([cout/nt][cin/16][9][2][nt][8],
 * nt = the output channels one CTA computes: the widest multiple of 16
 * dividing cout whose weight stages fit shared memory, e.g. 224 -> 112);
 * cin % 16 == 0, cout % 16 == 0, 16-byte aligned operands.
 * A CTA whose bounded waits expire writes nothing and sets the flag that
 * asuna_nn_tc_status reports (and clears). */
int asuna_nn_weights_tc(void* stream, const void* w, void* wtc, int cout, int cin);
int asuna_nn_conv3x3_tc(void* stream, const void* in, int n, int h, int w, int cin, const void* weight_tc,
                        const float* bias, int cout, int relu, const void* mask, void* out, int out_f32);
int asuna_nn_tc_status(int* expired);
int asuna_nn_f32_to_bf16(void* stream, const float* a, void* b, uint64_t n);

#ifdef __cplusplus
}
#endif
#endif /* ASUNA_DENOISE_H */
