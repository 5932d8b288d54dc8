/* fc3dgpu_mlp: learned warm start for the GPU NSGS solver.
 *
 * No counterpart in the reference: a per-contact multilayer perceptron
 * (17 -> 128 -> 128 -> 128 -> 3, ReLU) proposes each contact's reaction in its
 * local frame from
 *   features 0-8   the diagonal Delassus block W_ii (column-major),
 *   features 9-11  q_i,
 *   feature  12    mu_i,
 *   features 13-15 the previous-step reaction r_i (0 on a first step),
 *   feature  16    the normal gap (0 when the caller has none).
 * Inputs are standardised with the training set's mean and standard
 * deviation; targets likewise.  Weights are BF16 for the matrix products
 * (tensor cores, FP32 accumulation) with FP32 master copies for Adam.
 *
 * Parameter layout (FP32, fc3dgpu_mlp_nparams() values): for layer l = 0..3
 * the weights W_l as [K_l][N_l] row-major, then the biases [N_l], with
 * (K, N) = (32, 128), (128, 128), (128, 128), (128, 16): the 17 inputs are
 * zero-padded to 32 and the 3 outputs to 16 (padding weights are unused).
 * Statistics (40 floats): feature mean[17], feature std[17], target mean[3],
 * target std[3].
 */
#ifndef FC3DGPU_MLP_H
#define FC3DGPU_MLP_H

#include <stddef.h>

#include "fc3dgpu.h"

#ifdef __cplusplus
extern "C" {
#endif

#define FC3DGPU_MLP_FEATURES 17
#define FC3DGPU_MLP_OUTPUTS 3
#define FC3DGPU_MLP_STATS 40

typedef struct fc3dgpu_mlp fc3dgpu_mlp;

int fc3dgpu_mlp_nparams(void);
fc3dgpu_mlp *fc3dgpu_mlp_create(int device);
void fc3dgpu_mlp_destroy(fc3dgpu_mlp *m);
/* Load parameters and statistics (host arrays); resets Adam's moments. */
int fc3dgpu_mlp_set_params(fc3dgpu_mlp *m, const float *params, const float *stats);
int fc3dgpu_mlp_get_params(fc3dgpu_mlp *m, float *params, float *stats);
/* Training set: X[n][17] raw features, T[n][3] target reactions (host). */
int fc3dgpu_mlp_set_data(fc3dgpu_mlp *m, size_t n, const float *X, const float *T);
/* One training step on the samples idx[0..nbatch) of the training set:
 * forward, mean-squared-error gradient on standardised targets, backward;
 * with apply != 0 an Adam step (lr, decoupled weight decay wd on weights;
 * beta1 0.9, beta2 0.999, eps 1e-8).  grad_out (NULL or fc3dgpu_mlp_nparams()
 * floats) receives the gradient, *loss_out (NULL or 1 float) the loss before
 * the step. */
int fc3dgpu_mlp_train_step(fc3dgpu_mlp *m, int nbatch, const int *idx, float lr, float wd, float *grad_out,
                           float *loss_out, int apply);
/* As fc3dgpu_mlp_train_step on the samples idx[0..nbatch) given as a DEVICE
 * array, without host synchronisation (for loops of many steps); an index
 * outside the training set counts as an absent sample. */
int fc3dgpu_mlp_train_step_device(fc3dgpu_mlp *m, int nbatch, const int *idx_dev, float lr, float wd);
/* Proposals Y[n][3] for raw features X[n][17]: host arrays when on_device
 * is 0, else device arrays used on the model's stream. */
int fc3dgpu_mlp_infer(fc3dgpu_mlp *m, size_t n, const float *X, float *Y, int on_device);
/* Device arrays, on `stream` (cudaStream_t) instead of the model's stream. */
int fc3dgpu_mlp_infer_stream(fc3dgpu_mlp *m, size_t n, const float *X, float *Y, void *stream);

/* Matrix products on the Blackwell tensor cores (tcgen05.mma with TMEM
 * accumulators, 128 samples per block; tcgen05 != 0, the default) or on the
 * warp-level mma.sync path (64 samples per block), the checked reference.
 * Same network, same BF16 operands and FP32 accumulation; the two differ
 * in the order of the FP32 sums only.  Returns the previous setting. */
int fc3dgpu_mlp_set_tensor_path(fc3dgpu_mlp *m, int tcgen05);

/* What the network's three outputs mean: 0 (default) the reaction itself,
 * 1 the change from the previous-step reaction (features 13-15).  Returns the
 * previous setting; fc3dgpu_mlp_residual reads it. */
int fc3dgpu_mlp_set_residual(fc3dgpu_mlp *m, int residual);
int fc3dgpu_mlp_residual(const fc3dgpu_mlp *m);

/* Learned warm start of a device context.  The reaction currently in the
 * context (the previous step's, or what fc3dgpu_ctx_set_r gave) is the
 * fallback.  Features are formed on the device (gap: host array of nc
 * values in the caller's contact order, or NULL for 0) and the network
 * proposes a target (its output, or the fallback plus its output for a
 * residual network).  The candidates fallback + alpha (target - fallback),
 * alpha = 1, 1/2, 1/4, each projected on every friction cone, are evaluated
 * with fc3d_compute_error; the best replaces the reaction only when its error
 * is below the fallback's.  out3 (NULL or 3 doubles): error of the fallback,
 * error of the best candidate, 1 when it was taken.  The norm of q is the
 * context's. */
int fc3dgpu_ctx_warm_start(fc3dgpu_ctx *ctx, fc3dgpu_mlp *m, const double *gap, double *out3);
/* The 17 features of every contact, as the warm start forms them, in the
 * caller's contact order (X: host array of nc*17 floats). */
int fc3dgpu_ctx_features(fc3dgpu_ctx *ctx, const double *gap, float *X);

#ifdef __cplusplus
}
#endif
#endif
