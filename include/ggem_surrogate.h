/*
 * ggem_surrogate.h -- the learned eigen-interval surrogate of the GGEM
 * Brownian step.
 *
 * Replaces the spectral-bound estimate BrownianSystem::compute_eigenvalue(s)
 * (brownian_system.C:527-657 with the SLEPc Krylov-Schur solver;
 * Copss::fixman_integrate widens it by eig_factor, copss.C:1598-1639) by a
 * small network that predicts [log lambda_min, log lambda_max] of the local
 * mobility from configuration features.  The FP64 Chebyshev error check
 * (ggem_brownian_displacement*) judges every prediction; the caller falls
 * back to ggem_lanczos_bounds when the check fails, as the reference
 * recomputes its eigenvalues when the Chebyshev series fails.
 *
 * Network: 35 features -> 3 hidden layers of 128 SiLU units -> 2 outputs,
 * BF16 weights with FP32 accumulation on the tensor cores (tcgen05),
 * trained on the GPU with Adam on FP32 master weights.
 *
 * Features (ggem_surrogate_features): [phi, log N, g(r) in 32 bins over
 * [2a, rc) from the FP32 pair list, chain fraction].
 */
#ifndef GGEM_SURROGATE_H
#define GGEM_SURROGATE_H

#include <stdint.h>

#include "ggem_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

#define GGEM_SUR_FEATURES 35
#define GGEM_SUR_OUTPUTS 2
#define GGEM_SUR_HIST_BINS 32
/* flat FP32 parameter vector: W1^T [128 x 48] (input columns >= 35 zero),
 * b1 [128], W2^T [128 x 128], b2, W3^T [128 x 128], b3, W4^T [128 x 128]
 * (rows >= 2 zero), b4 [128] (entries >= 2 zero) */
#define GGEM_SUR_PARAMS (128 * 48 + 128 + 3 * (128 * 128 + 128))
/* normalisation block: feature mean [35], feature 1/std [35], output mean [2],
 * output std [2] */
#define GGEM_SUR_NORM (2 * GGEM_SUR_FEATURES + 2 * GGEM_SUR_OUTPUTS)

typedef struct ggem_surrogate ggem_surrogate;

/* a network with seeded Glorot-uniform weights on the device; NULL when no
 * CUDA device is usable (ggem_last_error-free: see ggem_surrogate_status) */
ggem_surrogate *ggem_surrogate_create(int device, uint64_t seed);
void ggem_surrogate_destroy(ggem_surrogate *s);
/* status of the last call on s (GGEM_OK or a negative code) and its message */
const char *ggem_surrogate_last_error(const ggem_surrogate *s);

/* normalisation of inputs and outputs (GGEM_SUR_NORM floats) */
int ggem_surrogate_set_norm(ggem_surrogate *s, const float *norm);
int ggem_surrogate_get_norm(const ggem_surrogate *s, float *norm);
/* parameters (GGEM_SUR_PARAMS floats, FP32 master copy) */
int ggem_surrogate_set_params(ggem_surrogate *s, const float *params);
int ggem_surrogate_get_params(ggem_surrogate *s, float *params);

/* Adam training on host arrays X [n x 35] (raw features) and Y [n x 2]
 * (log lambda_min, log lambda_max), minibatches of `batch` rows (a multiple
 * of 128) in a seeded shuffle per epoch; loss[e] = mean squared error of the
 * standardised outputs over epoch e (may be NULL). */
int ggem_surrogate_train(ggem_surrogate *s, const float *X, const float *Y, int64_t n,
                         int epochs, int batch, float lr, uint64_t seed, float *loss);
/* predictions Y [n x 2] (log lambda) for raw features X [n x 35] */
int ggem_surrogate_predict(ggem_surrogate *s, const float *X, int64_t n, float *Y);
/* the same predictions through the layer-by-layer path of training (one
 * tensor-core product and one bias/activation kernel per layer; the default
 * ggem_surrogate_predict runs all layers in one kernel with the weights
 * resident in shared memory) */
int ggem_surrogate_predict_layers(ggem_surrogate *s, const float *X, int64_t n, float *Y);
/* measurement and test hooks: the mean time of the one-kernel forward pass
 * over n rows (CUDA events, reps launches); and the number of polls the
 * first mbarrier wait of every product makes before the kernel gives up and
 * reports GGEM_ERR_TIMEOUT (default 4194304; the wait that drains a product
 * before its TMEM is freed keeps the full budget) */
int ggem_surrogate_time_forward(ggem_surrogate *s, int64_t n, int reps, double *ms);
int ggem_surrogate_set_poll_budget(ggem_surrogate *s, uint32_t polls);
/* one forward + backward pass over X, Y (n <= 4096 rows) without an update:
 * the loss and the gradient with respect to every parameter (GGEM_SUR_PARAMS
 * floats, same layout as the parameters) */
int ggem_surrogate_gradient(ggem_surrogate *s, const float *X, const float *Y, int64_t n,
                            float *loss, float *grad);

/* configuration features of the context's current particles (FP32 pair
 * list required): phi = n (4/3) pi a^3 / V with a = br0, log n, the pair
 * distance histogram g(r) over [2 br0, rc) in 32 bins (ordered pairs per
 * bead divided by the ideal-gas count of the shell), chain fraction as
 * given */
int ggem_surrogate_features(ggem_ctx *ctx, double chain_fraction, float *features);
/* eigen interval of the context's mobility from the network: the predicted
 * log-bounds widened by margin_lo / margin_hi (in log units) */
int ggem_surrogate_interval(ggem_ctx *ctx, ggem_surrogate *s, double chain_fraction,
                            double margin_lo, double margin_hi, double *eig_min,
                            double *eig_max);

#ifdef __cplusplus
}
#endif
#endif
