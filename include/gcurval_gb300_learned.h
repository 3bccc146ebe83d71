/* gcurval_gb300 learned form: the MLP that predicts, per B-spline knot
 * interval, where the adaptive length walk should start (the depth of its
 * shallowest leaf and the share of leaves per quarter of the interval) and 8
 * local parameters at arc-length fractions (j + 1/2) / 8.  No reference
 * counterpart: the reference's walk always starts from 64 uniform pieces per
 * interval (gcurval/detail/cuda/kernel/generic.inl.cuh:10-48).
 *
 * Network: 16 features -> 128 -> 128 -> 128 (GELU, tanh form) -> 32 outputs
 * (13 depth logits, 4 quarter logits, 8 parameters, 7 unused).  Weights are
 * one packed FP32 array of gcv_mlp_param_count() values: W1[16][128], b1,
 * W2[128][128], b2, W3[128][128], b3, W4[128][32], b4 (row-major W[in][out]).
 *
 * Training runs on the GPU with the library's FP32 kernels; inference inside
 * createArclengthTable runs BF16 tensor-core (tcgen05) kernels with FP32
 * accumulation.  Every interval the network places is re-checked by the
 * Kronrod error estimate and refined further where it misses the tolerance.
 * All pointers named d_* are device memory.
 */
#ifndef GCURVAL_GB300_LEARNED_H
#define GCURVAL_GB300_LEARNED_H

#include "gcurval_gb300.h"

#ifdef __cplusplus
extern "C" {
#endif

int gcv_mlp_param_count(void);
const char* gcv_mlp_last_error(void);

/* ---- training data from a context -------------------------------------- */

/* The 16 features of every knot interval of the context's batch into
 * d_features (n_segments x 16 floats); non-B-spline intervals get zeros. */
gcv_status gcv_learned_features(gcv_ctx* ctx, float* d_features);

/* Labels from the context's current table, built by the plain method:
 * d_depth (n_segments ints, the shallowest leaf depth, capped at 12),
 * d_share (n_segments x 4 floats, leaves per quarter over all leaves),
 * d_tguess (n_segments x 8 floats, local parameters v in [-1, 1] at the
 * arc-length fractions (j + 1/2) / 8). */
gcv_status gcv_learned_labels(gcv_ctx* ctx, int* d_depth, float* d_share, float* d_tguess);

/* ---- training (FP32) ----------------------------------------------------- */

typedef struct gcv_mlp_trainer gcv_mlp_trainer;

/* He-initialised network and Adam state for batches of up to max_batch rows. */
gcv_status gcv_mlp_trainer_create(gcv_mlp_trainer** out, int max_batch, unsigned long long seed);
gcv_status gcv_mlp_trainer_destroy(gcv_mlp_trainer* tr);
gcv_status gcv_mlp_trainer_set_weights(gcv_mlp_trainer* tr, const float* host_weights);
gcv_status gcv_mlp_trainer_get_weights(gcv_mlp_trainer* tr, float* host_weights);
/* FP32 forward pass: d_out (n x 32). */
gcv_status gcv_mlp_trainer_forward(gcv_mlp_trainer* tr, const float* d_features, int n, float* d_out);
/* Gradients of the mean loss (cross-entropy of the depth class + cross-
 * entropy of the quarter shares + half the squared error of the 8
 * parameters) into host_grad (packed like the weights; may be NULL) and the
 * three mean loss parts into host_loss3 (may be NULL).  No update. */
gcv_status gcv_mlp_trainer_gradients(gcv_mlp_trainer* tr, const float* d_features, const int* d_depth,
                                     const float* d_share, const float* d_tguess, int n, float* host_grad,
                                     float* host_loss3);
/* One Adam step (beta 0.9 / 0.999) on one batch. */
gcv_status gcv_mlp_trainer_step(gcv_mlp_trainer* tr, const float* d_features, const int* d_depth,
                                const float* d_share, const float* d_tguess, int n, float lr, float* host_loss3);

/* ---- inference (BF16 tensor cores) -------------------------------------- */

/* Outputs of the tensor-core network for n feature rows: d_out (n x 32
 * floats).  The same kernel body that createArclengthTable runs, with the
 * features read from memory instead of computed in the kernel. */
gcv_status gcv_mlp_infer(const float* host_weights, const float* d_features, int n, float* d_out);

/* Installs a trained network in the context (host_weights packed as above;
 * NULL removes it).  With a network installed and options.learned set, the
 * length pass starts every B-spline interval at the predicted depths. */
gcv_status gcv_set_learned_model(gcv_ctx* ctx, const float* host_weights);

#ifdef __cplusplus
}
#endif

#endif
