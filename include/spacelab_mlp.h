/*
 * spacelab_mlp.h -- the collision-outcome surrogate's network
 * (libspacelab_gb300.so).  No counterpart in the reference.
 *
 * An MLP n_in -> hidden_layers x hidden (GELU) -> n_out with BF16 weights and
 * activations and FP32 accumulation on the tensor cores, FP32 biases and
 * FP32 master weights updated by Adam, trained and evaluated by the
 * library's own kernels.  Loss: mean squared error over the n_out outputs.
 * Parameter vector layout (sl_mlp_get_params): for each linear layer l,
 * W_l as [dout_l][din_l] row-major then b_l [dout_l], where din/dout are the
 * layer widths rounded up to multiples of 32 (padding entries are 0).
 * All arrays here are host arrays; x is [n][n_in], y is [n][n_out].
 */
#ifndef SPACELAB_MLP_H
#define SPACELAB_MLP_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct sl_mlp sl_mlp;

int sl_mlp_create(int n_in, int hidden, int hidden_layers, int n_out, int max_batch, uint64_t seed, sl_mlp** out);
int sl_mlp_destroy(sl_mlp* m);
int sl_mlp_num_params(const sl_mlp* m, int64_t* n);
int sl_mlp_get_params(sl_mlp* m, float* params);
int sl_mlp_set_params(sl_mlp* m, const float* params);
/* Loss and gradient (same layout as the parameters) of one batch of M rows
 * (M a multiple of 32, at most max_batch). */
int sl_mlp_gradients(sl_mlp* m, const float* x, const float* y, int M, float* grads, float* loss);
/* Adam training: `epochs` passes over n rows in shuffled batches of `batch`
 * (a multiple of 32); loss_per_epoch (may be NULL) gets each epoch's mean
 * batch loss. */
int sl_mlp_train(sl_mlp* m, const float* x, const float* y, int n, int epochs, int batch, float lr, uint64_t seed,
                 float* loss_per_epoch);
/* Outputs for n rows. */
int sl_mlp_predict(sl_mlp* m, const float* x, int n, float* y);

#ifdef __cplusplus
}
#endif
#endif /* SPACELAB_MLP_H */
