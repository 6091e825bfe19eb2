/*
 * rg300 learned Newton warm start -- C ABI.
 *
 * A small per-node network predicts U, V and S of the next time level from
 * the last two time levels on a one-ring mesh stencil, the bed elevation and
 * the inflow-discharge ratio: its outputs correct the linear extrapolation
 * 2 L1 - L2 of the last two levels (L1 where the node was dry at level 2).
 * The prediction is only a starting point for the Newton iteration of
 * rg_sim_step: the plain Newton /
 * BiCGStab iteration still judges convergence, and the step starts from the
 * previous time level whenever the predicted start has the larger residual.
 * No counterpart in the reference (EQS_UVS2D::Predict, EqsUVS2D.cpp:1101,
 * starts every step from the last time level).
 *
 * Network: 128 inputs (15 stencil nodes x 8 features + discharge ratios),
 * three hidden layers of 128 with GELU, 3 outputs; BF16 weights and
 * activations, FP32 accumulation; forward and the backward products of the
 * 128-wide layers on the tensor cores (mma.sync bf16, the upstream gradient
 * rounded to bf16), the 3-output layer's backward and Adam in FP32.  Trained on the GPU from time-level
 * triples a caller collects from the plain solver.
 *
 * All arrays are HOST memory; node arrays are indexed like the rg_sim node
 * arrays.  Every function returns an rg_status.
 */
#ifndef RG300_MLP_H
#define RG300_MLP_H

#include "rg300.h"

#ifdef __cplusplus
extern "C" {
#endif

typedef struct rg_mlp rg_mlp;

#define RG_MLP_IN 128
#define RG_MLP_HIDDEN 128
#define RG_MLP_OUT 3
#define RG_MLP_STENCIL 15
/* parameters, in this order: W1 (128x128, row = output), b1, W2, b2, W3, b3, W4 (3x128), b4 */
#define RG_MLP_NPARAM (3 * (128 * 128 + 128) + 3 * 128 + 3)

/* Create on CUDA device `device` (the current device when negative) with
 * weights drawn from a seeded uniform(-1/sqrt(fan_in), 1/sqrt(fan_in)). */
rg_status rg_mlp_create(int device, unsigned seed, rg_mlp** out);
rg_status rg_mlp_destroy(rg_mlp* mlp);
const char* rg_mlp_last_error(rg_mlp* mlp);

/* Mesh of the stencils: node coordinates and bed elevation, six-node region
 * triangles (corners, then mid-sides).  A node's stencil is the node and its
 * 14 nearest one-ring neighbours (nodes sharing a triangle), ordered by angle
 * from the +x axis. */
rg_status rg_mlp_set_mesh(rg_mlp* mlp, int np, const double* x, const double* y, const double* z,
                          int ne, const int* elem_nodes);

/* Scales: in_ref3 = inputs H [m], velocity [m/s], bed difference [m];
 * step_scale3 = one step's change of U, V, S (the dU, dV, dS inputs);
 * out_scale3 = the outputs' unit: the deviation of the next level's U, V, S
 * from the linear extrapolation.  A NULL array keeps its scales. */
rg_status rg_mlp_set_scales(rg_mlp* mlp, const float* in_ref3, const float* step_scale3, const float* out_scale3);
rg_status rg_mlp_get_params(rg_mlp* mlp, float* params);
rg_status rg_mlp_set_params(rg_mlp* mlp, const float* params);

/* Input features of the given nodes (bf16 values returned as float,
 * 128 per node) for a state pair: level 1 = the last time level, level 2 =
 * the one before; q_next / q_prev = Q(t+dt)/Q(t) and Q(t)/Q(t-dt). */
rg_status rg_mlp_features(rg_mlp* mlp, int n, const int* nodes, const double* U1, const double* V1,
                          const double* S1, const double* U2, const double* V2, const double* S2, double q_next,
                          double q_prev, float* X_out);

/* Append the wet nodes of one time-level triple (levels 2, 1 and the solved
 * level 0) to the training set: features from levels 1 and 2, target
 * (level 0 - extrapolation) / output scales.  wet2 / wet1 / wet0 flag the
 * nodes wet at each level (nonzero = wet); nodes wet at levels 1 and 0 are
 * added.  *added receives the number of samples appended. */
rg_status rg_mlp_add_samples(rg_mlp* mlp, const double* U2, const double* V2, const double* S2, const double* U1,
                             const double* V1, const double* S1, const double* U0, const double* V0,
                             const double* S0, const int* wet2, const int* wet1, const int* wet0, double q_next,
                             double q_prev, long long* added);
rg_status rg_mlp_clear_samples(rg_mlp* mlp);

/* Adam on the mean squared error over the training set: `epochs` passes in
 * mini-batches of `batch` samples (shuffled with `seed`); loss_out[e] (may be
 * NULL) receives each epoch's mean loss. */
rg_status rg_mlp_train(rg_mlp* mlp, int epochs, int batch, float lr, unsigned seed, double* loss_out);

/* Loss and gradient of one batch given directly (n rows of 128 inputs, which
 * are rounded to bf16; targets n x 3; mask n): the training kernels' result,
 * for checking them.  y_out (n x 3) and grad_out (RG_MLP_NPARAM) may be NULL. */
rg_status rg_mlp_loss_grad(rg_mlp* mlp, int n, const float* X, const float* T, const float* mask, double* loss,
                           float* y_out, float* grad_out);

/* Predicted next time level: for the nodes wet at level 1, U/V/S_out =
 * extrapolation (2 L1 - L2, or L1 where wet2 is zero) + outputs x output
 * scales; other nodes copy level 1. */
rg_status rg_mlp_predict(rg_mlp* mlp, const double* U2, const double* V2, const double* S2, const double* U1,
                         const double* V1, const double* S1, const int* wet2, const int* wet1, double q_next,
                         double q_prev, double* U_out, double* V_out, double* S_out);

#ifdef __cplusplus
}
#endif

#endif
