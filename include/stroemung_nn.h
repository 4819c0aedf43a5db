/*
 * stroemung_nn.h — C ABI of the learned pressure warm start (BF16 network on
 * the tcgen05 tensor cores).  No counterpart in the reference: the learned
 * warm start is an extension of this project.
 */
#ifndef STROEMUNG_NN_H
#define STROEMUNG_NN_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

enum {
    STRM_NN_OK = 0,
    STRM_NN_ERR_INVALID = 6,
    STRM_NN_ERR_CUDA = 5,
    STRM_NN_ERR_TIMEOUT = 4
};

/* The three tensor-core contractions (strm_nn_gemm_bf16, strm_nn_conv3x3,
 * strm_nn_conv3x3_wgrad) wait for their kernel and return STRM_NN_ERR_TIMEOUT
 * when a bounded wait inside it gave up.  strm_nn_set_sync(0) makes them
 * return right after the launch (process-wide; 1 restores waiting); a
 * timeout is then reported by strm_nn_status, which waits for `stream` and
 * returns STRM_NN_ERR_TIMEOUT once any such wait on this device has given
 * up (the flag stays set). */
int strm_nn_set_sync(int sync);
/* Staging of the forward convolution's operands (strm_nn_conv3x3): 1 (the
 * default) stages them with TMA for layers whose input channels are a
 * multiple of 32 and whose image width is a multiple of 128 (one tensor-map
 * box per tap and channel slice); 0 gathers every layer's im2col rows with
 * 16-byte copies.  The results agree within BF16-input / FP32-accumulation
 * rounding (the K sums are split differently). */
int strm_nn_set_conv_tma(int use);
/* Launch shape of the TMA-staged forward: tiles_per_cta n >= 1 gives each
 * CTA n of the layer's 128-pixel tiles, ctas_per_sm of them sharing an SM's
 * shared memory; 0 (the default) takes four while the layer fills every
 * CTA slot of the GPU that often, else two, else one.  ctas_per_sm 0 (the
 * default) takes as many as hold a two-stage ring each, at most 8 and what
 * TMEM allows; each CTA has a ring of `stages` operand stages (0: as many
 * as its share of the SM's shared memory holds; else 2..32).  rows = 1 (the
 * default) loads, for up to 128 output channels, one 130-pixel box per
 * kernel row and 32-channel slice and feeds the three taps of that row from
 * it; 0 loads one 128-pixel box per tap and 32- or 64-channel slice (as
 * 256-channel tiles always do).  Process-wide; for a given `rows` results
 * do not depend on it (the two `rows` modes add the K terms in different
 * orders).  STRM_NN_ERR_INVALID for values out of range (tiles_per_cta
 * 0..64). */
int strm_nn_tune_conv_tma(int ctas_per_sm, int stages, int tiles_per_cta, int rows);
int strm_nn_status(void *stream);

/* d[m x n] (FP32, row-major) = a[m x k] * b[n x k]^T with a, b BF16 row-major
 * device arrays; m, n multiples of 128, k a multiple of 64.  tcgen05.mma with
 * TMEM accumulators, on `stream` (a cudaStream_t); waits for the kernel
 * unless strm_nn_set_sync(0). */
int strm_nn_gemm_bf16(const void *a, const void *b, float *d, int m, int n, int k,
                      void *stream);

/* Activations are BF16 NHWC device tensors: pixel q = (b*h + y)*w + x at
 * base + q*cs, channels contiguous (cs = pixel stride in elements, >= the
 * channel count; channel slices of one buffer form a concatenation).  All
 * calls are asynchronous on `stream` unless stated. */

/* 3x3 "same" convolution (implicit GEMM on tcgen05): y = act(conv(x, w) +
 * bias).  cin_p: input channels padded to a multiple of 8; w: BF16
 * [cout][kp] with K = tap*cin_p + channel (tap = (dy+1)*3 + (dx+1)), kp =
 * roundup(9*cin_p, 64), zero padded; cout in {16, 32, 64, 128, 256}; bias
 * FP32 [cout] or NULL; relu 0/1; output BF16 at y (pixel stride cs_out), or
 * FP32 at y32 when y32 is not NULL.  Waits for the kernel unless
 * strm_nn_set_sync(0) (see above). */
int strm_nn_conv3x3(const void *x, int cs_in, int cin_p, const void *w, int kp,
                    const float *bias, void *y, float *y32, int cs_out, int cout, int batch,
                    int h, int width, int relu, void *stream);

/* Weight gradient of that convolution, accumulated (+=) into FP32
 * dw[cout][kp]: dw += sum_q g[q] (x) im2col(x)[q], with g = dy masked by the
 * forward ReLU output yact (y > 0) when yact is not NULL (yact uses the
 * forward pixel stride cs_out).  Waits for the kernel unless
 * strm_nn_set_sync(0). */
/* strm_nn_conv3x3 with ReLU (relu = 1) and BF16 output, followed by the 1x1
 * FP32 head of strm_nn_head in the same kernel: q[p] = bh[0] + sum_c wh[c] *
 * y[p][c] over the BF16 outputs, in channel order — the same bits as the two
 * calls.  y may be NULL: the activations are then not stored (cs_out is
 * ignored), as a prediction that no backward follows needs. */
int strm_nn_conv3x3_head(const void *x, int cs_in, int cin_p, const void *w, int kp,
                         const float *bias, void *y, int cs_out, int cout, int batch, int h,
                         int width, const float *wh, const float *bh, float *q, void *stream);
int strm_nn_conv3x3_wgrad(const void *x, int cs_in, int cin_p, int kp, const void *dy,
                          int cs_dy, const void *yact, int cs_out, float *dw, int cout,
                          int batch, int h, int width, void *stream);

int strm_nn_avgpool(const void *in, int cs_in, void *out, int cs_out, int batch, int h,
                    int width, int c, void *stream);
int strm_nn_avgpool_bwd(const void *gout, int cs_out, void *gin, int cs_in, int batch, int h,
                        int width, int c, int accumulate, void *stream);
/* h, width: the upsampled (output) size. */
int strm_nn_upsample(const void *in, int cs_in, void *out, int cs_out, int batch, int h,
                     int width, int c, void *stream);
int strm_nn_upsample_bwd(const void *gout, int cs_out, void *gin, int cs_in, int batch, int h,
                         int width, int c, void *stream);
int strm_nn_relu_mask(const void *g, int cs_g, const void *y, int cs_y, void *out, int cs_out,
                      long long npix, int c, void *stream);
int strm_nn_bias_grad(const void *g, int cs_g, const void *y, int cs_y, float *db,
                      long long npix, int c, void *stream);
/* wt[ci][t][co] = w[co][8 - t][ci]: weights of the data gradient. */
int strm_nn_flip_weights(const void *w, int cout, int cin_p, int kp, void *wt, int cout_p,
                         int kp_t, void *stream);
/* 1x1 output head in FP32 and its adjoint. */
int strm_nn_head(const void *act, int cs, int c, const float *wh, const float *bh, float *out,
                 long long npix, void *stream);
int strm_nn_head_bwd(const void *act, int cs, int c, const float *wh, const float *gout,
                     void *gact, int cs_g, float *dwh, float *dbh, long long npix,
                     void *stream);
/* Network input from solver planes [batch][nx][ny] (ring included): FP32
 * rhs and previous pressure, u8 flags (kind | edge << 3).  Writes the
 * per-sample scale smax (max |rhs| on fluid cells), pmean (mean previous
 * pressure on fluid cells) and the 8-channel BF16 input [batch][nx-2][ny-2].
 * work2 holds 2*batch floats. */
int strm_nn_prepare_input(const float *rhs, const uint8_t *flags, const float *pprev,
                          float *smax, float *pmean, float *work2, float dx2, void *xin,
                          int batch, int nx, int ny, void *stream);
/* Relative Poisson residual of the prediction p = p_prev + smax*dx2*q on
 * fluid interior cells (boundary values by the solver's copy rule):
 * sum_r2[b] = sum r^2, sum_b2[b] = sum rhs^2; pfull and r are [batch][nx][ny]
 * work planes. */
int strm_nn_residual_loss(const float *pprev, const float *q, const uint8_t *flags,
                          const float *rhs, const float *smax, float dx2, float rdx2,
                          float rdy2, float *pfull, float *r, float *sum_r2, float *sum_b2,
                          int batch, int nx, int ny, void *stream);
/* Gradient of mean_b(sum_r2 / sum_b2) with respect to q ([batch][nx-2][ny-2]). */
int strm_nn_residual_loss_grad(const float *r, const uint8_t *flags, const float *sum_b2,
                               const float *smax, float dx2, float rdx2, float rdy2,
                               float *gp, float *gq, int batch, int nx, int ny, void *stream);
/* Error loss against target pressures (converged solutions), full planes
 * [batch][nx][ny] as for the residual loss, q [batch][nx-2][ny-2]: on fluid
 * interior cells e = p_prev + s dx^2 q - p_target and d = p_target - p_prev,
 * each with its fluid mean removed; loss[b] = sum e^2 / sum d^2 (may be
 * NULL) and gq = gradient of the batch mean with respect to q (may be NULL).
 * work holds 5 * batch floats. */
int strm_nn_error_loss(const float *pprev, const float *q, const float *ptarget,
                       const uint8_t *flags, const float *smax, float dx2, float *work,
                       float *loss, float *gq, int batch, int nx, int ny, void *stream);
/* cudaMemsetAsync(p, 0, bytes) on stream. */
int strm_nn_zero(void *p, long long bytes, void *stream);
/* Adam on FP32 master weights (step counts from 1); writes a BF16 copy to
 * wbf when not NULL. */
int strm_nn_adam(float *w, const float *g, float *m, float *v, long long n, float lr, float b1,
                 float b2, float eps, int step, void *wbf, void *stream);

#ifdef __cplusplus
}
#endif
#endif
