/* Kernels of the learned preconditioner for batched CG on the ADRT normal
 * equations: a 4-level convolutional encoder-decoder (32/64/128/256
 * channels, 3x3 kernels) that maps back-projected data A^T b to a starting
 * image for CG.
 *
 * The reference has no learned component; its reconstruction recipe is CG on
 * the normal equations with a zero start (docs/examples.cginverse.md:40-67).
 * These entry points have no reference counterpart.
 *
 * Conventions: activations are bf16 NHWC (batch, h, w, c) contiguous; images
 * f32 (batch, h, w); tensor-core weights bf16 [9][c_out][c_in] with tap
 * 3 * dy + dx over the zero-padded 3 x 3 window; gradients f32.  Pointers are
 * device pointers, `stream` a cudaStream_t (NULL = legacy default stream).
 * Every function returns an adrt_gb300 status code (adrt_gb300.h).
 */
#ifndef ADRT_GB300_NET_H
#define ADRT_GB300_NET_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* 3 x 3 convolution on the tcgen05 tensor cores (bf16 in, f32 accumulate,
 * bf16 out).  c_in, c_out in {32, 64, 128, 256}; h * w a multiple of 128 and
 * w a multiple of 128 or a divisor of 128; 16-byte aligned buffers.
 * Epilogue per output: v = acc + bias[co] (bias may be NULL) + addend
 * (NHWC like out, may be NULL); if relu, v = max(v, 0); if mask (NHWC like
 * out, may be NULL) is not positive, v = 0.
 * Forward: x = layer input, w = weights.  Input gradient: x = output
 * gradient (c_out channels of the layer), w = wt[8 - t][ci][co], and the
 * result has the layer's c_in channels. */
int adrtnet_conv3x3(const void *x, int c_in, const void *w, int c_out, const float *bias, const void *addend,
                    const void *mask, int relu, void *out, int64_t batch, int64_t h, int64_t w_, void *stream);

/* Weight gradient of a 3 x 3 convolution, accumulated (+=) into f32
 * dw[9][c_out][c_in]: dw[t][co][ci] += sum_p x[p + d_t][ci] * dy[p][co].
 * h * w a multiple of 64 and w a multiple of 64 or a divisor of 64. */
int adrtnet_conv3x3_wgrad(const void *x, int c_in, const void *dy, int c_out, float *dw, int64_t batch, int64_t h,
                          int64_t w_, void *stream);

/* Reads and clears the error word of the tensor-core kernels' bounded
 * waits: ADRT_GB300_ERR_TIMEOUT if a wait gave up since the last call. */
int adrtnet_status(void *stream);

/* First layer, 1 -> 32 channels: out = relu(b + sum_t w[t][co] u[p + d_t]);
 * w f32 [9][32], b f32 [32], u f32 image, out bf16 NHWC. */
int adrtnet_conv_in(const float *u, const float *w, const float *b, void *out, int64_t batch, int64_t h, int64_t w_,
                    void *stream);
/* Its weight and bias gradients, accumulated: g = gradient at the
 * pre-activation (bf16 NHWC, 32 channels). */
int adrtnet_conv_in_wgrad(const float *u, const void *g, float *dw, float *db, int64_t batch, int64_t h, int64_t w_,
                          void *stream);

/* Last layer, 32 -> 1 channel: out = b + sum_t sum_ci w[t][ci] f[p + d_t][ci]. */
int adrtnet_conv_out(const void *f, const float *w, const float *b, float *out, int64_t batch, int64_t h,
                     int64_t w_, void *stream);
/* Its backward: dx = input gradient masked by f > 0 (bf16 NHWC), dw and db
 * accumulated (+=). */
int adrtnet_conv_out_bwd(const float *g, const float *w, const void *f, void *dx, float *dw, float *db,
                         int64_t batch, int64_t h, int64_t w_, void *stream);

/* 2 x 2 average pooling (h, w even; c a multiple of 8) and its backward
 * out = (skip + g_low / 4) * (mask > 0) at full resolution (skip, mask may be NULL). */
int adrtnet_pool2(const void *x, void *out, int64_t batch, int64_t h, int64_t w_, int c, void *stream);
int adrtnet_pool2_bwd(const void *g_low, const void *skip, const void *mask, void *out, int64_t batch, int64_t h,
                      int64_t w_, int c, void *stream);

/* Nearest 2x upsampling of (batch, h, w, c) and its backward: out (low
 * resolution h x w) = (sum of each 2 x 2 block of g_high) * (mask > 0). */
int adrtnet_up2(const void *x, void *out, int64_t batch, int64_t h, int64_t w_, int c, void *stream);
int adrtnet_up2_bwd(const void *g_high, const void *mask, void *out, int64_t batch, int64_t h, int64_t w_, int c,
                    void *stream);

/* db[c] += sum over npix pixels of g[p][c] (bf16 NHWC, c a multiple of 32). */
int adrtnet_bias_grad(const void *g, float *db, int64_t npix, int c, void *stream);

/* Training loss, two steps: d = scale * out - target; then, with e = K d
 * for a symmetric positive semi-definite K the caller applies (e may be
 * NULL), loss += (alpha d.d + mu d.e) / n (loss may be NULL) and
 * g = 2 scale (alpha d + mu e) / n, the gradient with respect to out. */
int adrtnet_diff(const float *out, const float *target, float scale, float *d, int64_t n, void *stream);
int adrtnet_loss_grad(const float *d, const float *e, float alpha, float mu, float scale, float *g, float *loss,
                      int64_t n, void *stream);

/* A run of the flat f32 parameter vector.  Conv segments hold weights
 * [9][c_out][c_in]; the Adam kernel also writes their bf16 copies at
 * wbuf + w_offset (same layout) and wbuf + wt_offset ([9][c_in][c_out],
 * tap-flipped: the input-gradient weights). */
enum { ADRTNET_SEG_PLAIN = 0, ADRTNET_SEG_CONV = 1 };
typedef struct {
  int64_t offset;
  int64_t count;
  int32_t kind;
  int32_t c_in;
  int32_t c_out;
  int32_t pad_;
  int64_t w_offset;
  int64_t wt_offset;
} AdrtnetSegment;

/* Fused Adam step over n parameters (segments sorted by offset, device
 * array): m, v, p updated with bias correction for the step count *step
 * (device int64, >= 1), then the bf16 copies refreshed.  update = 0 only
 * refreshes the bf16 copies (g, m, v, step may then be NULL). */
int adrtnet_adam(float *p, const float *g, float *m, float *v, const AdrtnetSegment *segs, int nseg, int64_t n,
                 float lr, float beta1, float beta2, float eps, const int64_t *step, int update, void *wbuf,
                 void *stream);

#ifdef __cplusplus
}
#endif

#endif
