/* tracer_nn.h -- C ABI of the learned multigrid initial guess.
 *
 * No counterpart in the reference (tracer_code has no learned component).
 * The network predicts the change of the streamfunction between two
 * multigrid solves from three fields on the nx x nz grid nodes
 * (i = 0..nx-1, k = 0..nz-1, image row k, column i):
 *   channel 0: log10 of the level-1 viscosity, standardised per image;
 *   channel 1: the streamfunction RHS (compute_RHS), divided by its RMS;
 *   channel 2: the previous streamfunction, divided by its RMS s.
 * Its output o is (SF_new - SF_prev)/s on the interior nodes; the guess is
 * SF_prev + s*o.  Multigrid then iterates to the unchanged tolerance from
 * whichever of SF_prev and the guess has the smaller level-1 residual, so
 * the solution meets the same test with or without the network.
 *
 * Architecture: 4-level encoder-decoder, 32/64/128/128 channels, two 3x3
 * convolutions (bias, ReLU) per level and per decoder level, 2x2 average
 * pooling, nearest upsampling, skip connections by concatenation, 1x1
 * output head.  BF16 activations and weights, FP32 accumulation on the
 * tensor cores (tcgen05), FP32 master weights and Adam.
 *
 * Raw sample layout (device, FP32): raw[n][3][H][W] with H = nz, W = nx;
 * targets sf_new[n][H][W].  All pointers are device pointers unless named
 * *_host.  Calls are ordered on the network's stream (tcnn_set_stream). */
#ifndef TRACER_NN_H
#define TRACER_NN_H

#include <stdint.h>

#include "tracer_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct tc_net tc_net;

/* Network for batches of up to nb_max images of H x W (multiples of 16),
 * He-normal initial weights from `seed`. */
tc_status tcnn_create(int32_t nb_max, int32_t H, int32_t W, uint64_t seed, tc_net** out);
tc_status tcnn_destroy(tc_net* net);
tc_status tcnn_set_stream(tc_net* net, void* stream);
/* Timeout-path test (no counterpart in the reference).  With on != 0 every
 * 3x3 convolution of the network first waits, with a bounded poll, for a
 * device word that nothing sets, after allocating its tensor memory and
 * before issuing any copy; the poll runs out, the convolution reports
 * failure, frees its tensor memory and returns, and a solve that uses the
 * network returns TC_ERR_DEVICE_TIMEOUT.  on = 0 restores normal
 * convolutions. */
tc_status tcnn_debug_wait_test(tc_net* net, int32_t on);
int64_t tcnn_param_count(const tc_net* net);
/* Flat FP32 parameter / gradient vectors (layer by layer: W[cout][9][cin],
 * b[cout]; head w[32], b). */
tc_status tcnn_get_params(tc_net* net, float* params_host);
tc_status tcnn_set_params(tc_net* net, const float* params_host);
tc_status tcnn_get_grads(tc_net* net, float* grads_host);
/* Normalised output o[n][H][W] of nb images. */
tc_status tcnn_forward(tc_net* net, const float* raw, int32_t nb, float* out);
/* Forward, masked mean-squared error against the normalised target over the
 * interior nodes (i >= 1, k >= 1), backward; gradients stay in the network. */
tc_status tcnn_loss_backward(tc_net* net, const float* raw, const float* sf_new, int32_t nb, float* loss_host);
/* Adam step (bias-corrected) on the FP32 master weights with the stored
 * gradients, then the BF16 copies are refreshed. */
tc_status tcnn_adam(tc_net* net, float lr, float beta1, float beta2, float eps);

/* One 3x3 convolution (zero padding, stride 1) as the network computes it,
 * for tests: x[nb][H][W][cin] BF16 (cin a multiple of 16), w[cout][9][cin]
 * FP32 (rounded to BF16), b[cout] FP32, y[nb][H][W][cout] BF16 with
 * cout in {32, 64, 128, 256}; relu != 0 applies ReLU. */
tc_status tcnn_conv3x3(const uint16_t* x, int32_t nb, int32_t H, int32_t W, int32_t cin, const float* w,
                       const float* b, int32_t cout, int32_t relu, uint16_t* y);

/* Solver side.  tc_attach_net gives the handle a network of H = nz, W = nx
 * (batch 1) used when learned_guess = 1 in its parameters; the handle does
 * not own it.  tc_record_solves makes every later tc_multigrid call (also the
 * ones inside tc_energy_time/tc_step) append one training sample while fewer
 * than `capacity` are stored: raw[n][3][nz][nx] (channels as above, taken
 * when the solve starts) and sf_new[n][nz][nx] (the converged streamfunction).
 * tc_record_count returns how many are stored; tc_guess_stats how many
 * solves used the network's guess and how many were offered one (solves
 * skipped by the back-off of learned_guess = 1 are not offered one). */
tc_status tc_attach_net(tc_handle* h, tc_net* net);
tc_status tc_record_solves(tc_handle* h, float* raw, float* sf_new, int32_t capacity);
int32_t tc_record_count(const tc_handle* h);
tc_status tc_guess_stats(const tc_handle* h, int64_t* used, int64_t* offered);

#ifdef __cplusplus
}
#endif
#endif /* TRACER_NN_H */
