/* trapbec_surrogate.h -- kernels of the learned warm start for imaginary time.
 *
 * None of these entry points has a counterpart in the reference: the
 * reference starts imaginary-time relaxation from its analytic initial
 * states only (initial.f90).  The surrogate is a 3D convolutional
 * encoder-decoder that predicts the ground-state amplitude from the trap
 * potential and the instance parameters; its prediction is only ever used as
 * the initial guess of trapbec_step_imag / trapbec_batch_solve_imag, and the
 * Thomas-Fermi guess remains both the fallback and the yardstick.
 *
 * Conventions: all pointers are device pointers; activations are BF16,
 * channels-last [batch][D][H][W][C] with C a multiple of 16; gradients of
 * activations are FP32 in the same layout; weights of a 3x3x3 convolution
 * are [27][Cout][Cin] (tap = (kd*3 + kh)*3 + kw, offsets -1..1), FP32 master
 * copies and BF16 working copies.  `stream` is a cudaStream_t (NULL = the
 * legacy default stream).  Calls are asynchronous on that stream and return
 * TBSG_OK or an error code; nothing allocates device memory.
 */
#ifndef TRAPBEC_SURROGATE_H
#define TRAPBEC_SURROGATE_H

#include <stddef.h>

#ifdef __cplusplus
extern "C" {
#endif

enum tbsg_status { TBSG_OK = 0, TBSG_ERR_ARG = 1, TBSG_ERR_SHAPE = 2, TBSG_ERR_CUDA = 3 };

/* 3x3x3 convolution, stride 1, zero padding, on the BF16 tensor cores with
 * FP32 accumulation.  (Cin, Cout) in {(16,16),(16,32),(32,16),(32,32),(32,64),
 * (64,32),(64,64),(64,128),(128,64),(128,128)}.
 *  y != NULL:  y = act(conv(x, w) + bias + skip) in BF16 (bias, skip optional;
 *              act = 1: leaky ReLU with `slope`, 0: none)
 *  yf != NULL: yf = conv(x, w) (yf_accumulate = 0) or yf += conv(x, w), FP32;
 *              with the flipped, transposed kernel this is the input gradient. */
int tbsg_conv3_fwd(const void* x, int cin, const void* w, const float* bias, const void* skip, void* y,
                   float* yf, int yf_accumulate, int cout, int batch, int D, int H, int W, int act, float slope,
                   void* stream);

/* Input gradient of a convolution fused with the leaky-ReLU derivative of
 * the activation below it: with g = conv(dz, wt) (dz [..][cout], wt the
 * flipped, transposed weights of tbsg_weight_prep, g [..][cin] in FP32
 * accumulation), writes dz_in = BF16(g * act'(y_in)) (act' = 1 where
 * y_in > 0, else slope; y_in the activation's BF16 output [..][cin]) and, if
 * dskip != NULL, dskip += g * act'(y_in) (FP32).  Equal, bit for bit, to
 * tbsg_conv3_fwd(dz, cout, wt, .., yf = g, cin, ..) followed by
 * tbsg_act_bwd(g, y_in, dz_in, dskip, ..), without the FP32 g in memory.
 * y_in, dz_in and dskip must be 16-byte aligned.                          */
int tbsg_conv3_dgrad_act(const void* dz, int cout, const void* wt, const void* y_in, void* dz_in, float* dskip,
                         int cin, int batch, int D, int H, int W, float slope, void* stream);

/* Kernel family of tbsg_conv3_fwd and tbsg_conv3_wgrad: 0 (default) =
 * tcgen05.mma with TMEM accumulators (forward: 16/32 -> 16/32 channels,
 * mma.sync for the others; weight gradients: every pair); 1 = mma.sync for
 * all.  tbsg_tc_status reports (and clears) whether a tcgen05 launch gave up
 * waiting for its copies or MMAs (bounded, 2 s).                          */
int tbsg_set_conv_path(int path);
int tbsg_tc_status(int* timed_out);

/* Weight and bias gradients of a 3x3x3 convolution:
 *  dw[tap][co][ci] = sum_{b,v} dz[b][v][co] x[b][v + tap][ci],  db[co] = sum dz[.][co]
 * (db optional).  Deterministic: per-chunk partials in `scratch` (at least
 * tbsg_conv3_wgrad_scratch_bytes bytes) reduced in a fixed order.  The
 * tensor-core kernel takes batches of up to 8 (one halo tensor map per
 * sample); larger batches run on the mma.sync kernel.                      */
size_t tbsg_conv3_wgrad_scratch_bytes(int cin, int cout, int batch, int D, int H, int W);
int tbsg_conv3_wgrad(const void* x, int cin, const void* dz, int cout, int batch, int D, int H, int W,
                     float* dw, float* db, void* scratch, size_t scratch_bytes, void* stream);

/* FP32 master weights [27][Cout][Cin] -> BF16 working copy w and the BF16
 * flipped, transposed copy wt[26 - tap][ci][co] used for input gradients.  */
int tbsg_weight_prep(const float* w32, void* w, void* wt, int cin, int cout, void* stream);

/* dz = dy * act'(y) in BF16 for the leaky ReLU (y is the activation's output);
 * if dskip != NULL also dskip += dz (gradient of a skip added before act). */
int tbsg_act_bwd(const float* dy, const void* y, void* dz, float* dskip, size_t n, float slope, void* stream);

/* 2x2x2 mean pooling (D, H, W of the fine grid, all even) and its gradient
 * (dx_fine += dy_coarse / 8); nearest-neighbour 2x upsampling (D, H, W of the
 * coarse grid) and its gradient (dx_coarse = sum of the 8 fine gradients). */
int tbsg_pool2_fwd(const void* x, void* y, int c, int batch, int D, int H, int W, void* stream);
int tbsg_pool2_bwd(const float* dy, float* dx, int c, int batch, int D, int H, int W, void* stream);
int tbsg_up2_fwd(const void* x, void* y, int c, int batch, int D, int H, int W, void* stream);
int tbsg_up2_bwd(const float* dy, float* dx, int c, int batch, int D, int H, int W, void* stream);

/* Output head (FP32): amp[v] = base[v] + bh + sum_c feat[v][c] wh[c].
 * tbsg_head_fwd writes amp.  tbsg_head_loss also takes the target amplitude
 * and returns, for loss = mean_v (amp - target)^2:
 *  dfeat = d loss / d feat (FP32, overwritten) and out[0] = loss,
 *  out[1..c] = d loss / d wh, out[c+1] = d loss / d bh, reduced in a fixed
 *  order through `partials` (at least tbsg_head_partials(nvox, c) floats). */
int tbsg_head_fwd(const void* feat, int c, const float* wh, const float* bh, const float* base, float* amp,
                  size_t nvox, void* stream);
size_t tbsg_head_partials(size_t nvox, int c);
int tbsg_head_loss(const void* feat, int c, const float* wh, const float* bh, const float* base,
                   const float* target, size_t nvox, float* dfeat, float* partials, float* out, void* stream);

/* The activation-gradient fusions of the backward pass (act' = 1 where y > 0,
 * else slope; y the leaky ReLU's BF16 output; results equal, bit for bit, to
 * the unfused kernel followed by tbsg_act_bwd, without the FP32 gradient in
 * memory; pointers 16-byte aligned, c a multiple of 8):
 *  tbsg_head_loss_act: tbsg_head_loss for 16 feature channels, writing
 *    dz = BF16(d loss / d feat * act'(feat)) instead of d loss / d feat;
 *  tbsg_pool2_bwd_act: dz = BF16((g + up(dy) / 8) * act'(y)) on the fine grid
 *    (D, H, W fine; g the fine gradient so far, dy the coarse one);
 *  tbsg_up2_bwd_act: dz = BF16(sum of the 8 fine gradients * act'(y)) on the
 *    coarse grid (D, H, W coarse).                                          */
int tbsg_head_loss_act(const void* feat, const float* wh, const float* bh, const float* base, const float* target,
                       size_t nvox, void* dz, float slope, float* partials, float* out, void* stream);
int tbsg_pool2_bwd_act(const float* dy, const float* g, const void* y, void* dz, int c, int batch, int D, int H, int W,
                       float slope, void* stream);
int tbsg_up2_bwd_act(const float* dy, const void* y, void* dz, int c, int batch, int D, int H, int W, float slope,
                     void* stream);

/* Adam with decoupled weight decay on FP32 parameters (step t >= 1); the
 * gradient is multiplied by grad_scale[0] (device scalar, e.g. a clipping
 * factor from tbsg_clip_scale; NULL = 1).                                  */
int tbsg_adam(float* p, const float* g, float* m, float* v, size_t n, float lr, float beta1, float beta2,
              float eps, float weight_decay, int t, const float* grad_scale, void* stream);

/* Global-norm clipping factor: out[0] = ||g||_2, out[1] = min(1, max_norm / ||g||_2),
 * reduced in a fixed order through `partials` (1024 floats).               */
int tbsg_clip_scale(const float* g, size_t n, float max_norm, float* partials, float* out, void* stream);

/* FP32 -> BF16 conversion (inputs of the first layer).                     */
int tbsg_f32_to_bf16(const float* x, void* y, size_t n, void* stream);

/* Input features of one instance on the device: x receives [nx][ny][nz][16]
 * BF16 channels (0: harmonic potential wx X^2 + wy Y^2 + wz Z^2 of the scaled
 * coordinates X = x/Lx ..., clipped at 2; 1: Thomas-Fermi amplitude
 * sqrt(max(0, 1 - potential)); 2-9: consts[0..7] (host memory); 10-15: 0),
 * base receives the FP32 amplitude [nx][ny][nz].  Equal to the host recipe
 * computed in FP64, rounded to FP32 and then to BF16.                      */
int tbsg_features(void* x, float* base, int nx, int ny, int nz, double lx, double ly, double lz, double wx, double wy,
                  double wz, const float* consts, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* TRAPBEC_SURROGATE_H */
