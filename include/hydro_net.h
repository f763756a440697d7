/*
 * hydro_net.h -- C-ABI of the learned pressure guess of the GB300 hot path:
 * a 3-level convolutional encoder-decoder (16 / 32 / 64 channels, 3x3x3
 * kernels, BF16 weights and activations, FP32 accumulation on the tensor
 * cores) that maps the right-hand side f and the density rho of the
 * pressure-correction system (fluid.hpp:972-1027) to an initial guess of
 * its solution p'.  Trained on the GPU by its own forward and backward
 * kernels on snapshots the solver itself produces.
 *
 * The reference has no counterpart: its pressure solve starts from zero
 * every time (GaussSeidel::Solve, linear.hpp:685-715, behind
 * LinearSolver::Solve, linear.hpp:302-310, called at fluid.hpp:1029-1031).
 * The network never replaces the solve: the guess is scaled by the
 * Galerkin factor alpha = <x, f> / <x, A x> (which never increases the
 * energy-norm error of the zero guess), dropped when alpha is not positive
 * and finite or when its residual is not below that of the zero guess, and
 * the solve then runs to the unchanged tolerance relative to ||f||.
 *
 * Grids: 3D, nx, ny, nz multiples of 4 (two 2:1 poolings).  Tensors are
 * BF16 channels-last [batch][z][y][x][channels], device memory.  Weights of
 * a layer: FP32 [cout][cin][3][3][3] (tap = kz*9 + ky*3 + kx reads the
 * input at offset (kx-1, ky-1, kz-1)), then FP32 bias [cout].
 *
 * Layers (cin -> cout, grid): e1a 2->16, e1b 16->16 (N); average pool;
 * e2a 16->32, e2b 32->32 (N/2); pool; e3a 32->64, e3b 64->64 (N/4);
 * nearest upsample; d2a 64->32 (+ e2b), d2b 32->32 (N/2); upsample;
 * d1a 32->16 (+ e1b), d1b 16->16 (N); out 16->1 (N).  ReLU after every
 * layer but the last.  Inputs: channel 0 (f - mean f) / rms, channel 1
 * rho * rho_scale; output: (p' - mean p') / rms (the guess is rescaled by
 * alpha).  Parameters are stored with the padded channel counts the
 * kernels use: e1a has 16 input channels (2..15 stay zero) and out 16
 * output channels (1..15 stay zero).
 */
#ifndef HYDRO_NET_H_
#define HYDRO_NET_H_

#include <stddef.h>

#include "hydro_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct hydro_net hydro_net;

/* A network for grids of nx * ny * nz cells and up to `batch` samples per
 * training step, weights drawn from `seed` (He-normal).  Allocates its
 * activations, gradients and Adam moments once. */
int hydro_net_create(int nx, int ny, int nz, int batch, unsigned long long seed,
                     hydro_net** out);
int hydro_net_destroy(hydro_net* net);
/* Number of FP32 parameters (weights and biases of all layers, in layer
 * order, each layer's weights then its bias). */
int hydro_net_num_params(hydro_net* net, size_t* n);
int hydro_net_get_params(hydro_net* net, float* host, size_t n);
int hydro_net_set_params(hydro_net* net, const float* host, size_t n);

/* One packed training sample: per cell f / rms(f), rho * rho_scale,
 * p' / rms(p') in BF16 (6 bytes a cell). */
size_t hydro_net_sample_bytes(hydro_net* net);
/* Packs a sample from the solver's FP64 fields (device pointers, cells in
 * raw order): the pressure-correction right-hand side, the density and the
 * converged correction.  dst: device, hydro_net_sample_bytes bytes. */
int hydro_net_pack_sample(hydro_net* net, const double* rhs, const double* rho,
                          const double* pcorr, double rho_scale, void* dst, void* stream);
/* One Adam step (lr; beta 0.9 / 0.999) on `count` packed samples (device
 * pointers, count <= batch) with the mean-squared error of the output
 * against p' / rms(p'); *loss (may be NULL) receives the loss before the
 * step. */
int hydro_net_train_step(hydro_net* net, const void* const* samples, int count, double lr,
                         double* loss, void* stream);
/* The loss and its gradient with respect to every parameter (host array
 * of hydro_net_num_params floats, the parameter layout) on `count` packed
 * samples, without an update. */
int hydro_net_gradient(hydro_net* net, const void* const* samples, int count, float* grad,
                       size_t n, double* loss, void* stream);
/* Loss of the current weights on `count` packed samples (no update). */
int hydro_net_eval_loss(hydro_net* net, const void* const* samples, int count, double* loss,
                        void* stream);
/* Forward pass on one sample given as FP64 fields: out (device, cells)
 * receives the network's output (the shape of p', unit RMS scale). */
int hydro_net_predict(hydro_net* net, const double* rhs, const double* rho, double rho_scale,
                      double* out, void* stream);
/* Device milliseconds of the last hydro_net_predict and the number of its
 * kernel launches (CUDA events on its stream). */
int hydro_net_last_predict(hydro_net* net, double* ms, int* launches);

/* Attach a network to a context: the pressure solves of the first
 * `iterations` SIMPLE iterations of every step start from the network's
 * guess (0 detaches).  The context uses the network's buffers during its
 * steps (the network belongs to one context at a time) and does not own
 * it.  Needs the refinement solvers (precision MIXED, or pressure_solver
 * MGCG), dim 3 and the network's grid; otherwise HYDRO_ERR_UNSUPPORTED.
 * rho_scale: the density scaling of the network's input (the one its
 * samples were packed with). */
int hydro_gpu_set_pressure_guess(hydro_ctx* ctx, hydro_net* net, int iterations,
                                 double rho_scale);
/* Counters since the last call: pressure solves that started from the
 * network's guess, solves whose guess was dropped (alpha not positive, or a
 * residual not below the zero guess's), and steps that skipped the guess.
 * Back-off: a dropped guess makes the next 1, 2, 4, 8 and then 16 steps run
 * without the network (no forward pass); a kept guess resets it. */
int hydro_gpu_get_guess_stats(hydro_ctx* ctx, long long* used, long long* dropped,
                              long long* skipped);

/* ---- single layers, for checks against a CPU convolution -------------
 * Device buffers; x, y, g*: BF16 [nb][nz][ny][nx][c] with c in {16,32,64};
 * w: FP32 [cout][cin][27]; bias may be NULL.  Any grid size >= 1. */
/* y = relu?(conv(x, w) + bias + addend); addend may be NULL. */
int hydro_conv3d_forward(int nx, int ny, int nz, int nb, int cin, int cout, const void* x,
                         const float* w, const float* bias, const void* addend, int relu,
                         void* y, void* stream);
/* gx = (conv^T(gy, w) + addend) * (mask > 0): the gradient with respect to
 * the layer's input; addend and mask may be NULL. */
int hydro_conv3d_backward_data(int nx, int ny, int nz, int nb, int cin, int cout,
                               const void* gy, const float* w, const void* addend,
                               const void* mask, void* gx, void* stream);
/* dw (FP32 [cout][cin][27]) = sum_p gy[p][co] x[p + off(tap)][ci] and, when
 * db is not NULL, db[co] = sum_p gy[p][co] (both overwritten). */
int hydro_conv3d_backward_weight(int nx, int ny, int nz, int nb, int cin, int cout,
                                 const void* x, const void* gy, float* dw, float* db,
                                 void* stream);

#ifdef __cplusplus
}
#endif

#endif /* HYDRO_NET_H_ */
