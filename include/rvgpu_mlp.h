/* Learned candidate filter of librvgpu: a small MLP over the per-candidate
 * feature vector, trained and run on the GPU with hand-written tcgen05
 * (BF16 operands, FP32 accumulation) kernels.
 *
 * No counterpart in the reference: RabbitVar filters candidates only with the
 * hard thresholds of Variant::isGoodVar (include/Variant.h:197-248); its
 * XGBoost scripts (XGBoost/train_xgb.py, XGBoost/call_xgboost.py) score the
 * emitted records offline.  This filter scores the same candidates the device
 * pipeline builds, with the hard filter kept as the fallback and as the yard
 * stick of its precision and recall.
 *
 * Network: 40 -> 128 -> 128 -> 128 -> 1, GELU (erf form) after each hidden
 * layer, logistic output, weighted binary cross-entropy, Adam.  Parameters
 * are FP32 in this order (RV_MLP_PARAMS floats): W1[128][64] (input columns
 * 40..63 are padding and stay 0), b1[128], W2[128][128], b2[128],
 * W3[128][128], b3[128], w4[128], b4[1]; W[out][in].
 *
 * Calls on one model are not thread-safe.  Every call returns rv_status
 * (0 = RV_OK) and never exits the process. */
#ifndef RVGPU_MLP_H
#define RVGPU_MLP_H
#include <stddef.h>
#include <stdint.h>

#include "rvgpu.h"

#ifdef __cplusplus
extern "C" {
#endif

#define RV_MLP_FEATURES 40
#define RV_MLP_PARAMS 41473

typedef struct rv_mlp rv_mlp;

/* `batch` rows per training step: a multiple of 512, at most 65536.
 * Weights get a He-normal initialisation from `seed`. */
rv_status rv_mlp_create(rv_mlp **out, int device, int batch, uint64_t seed);
void rv_mlp_destroy(rv_mlp *m);
const char *rv_mlp_last_error(const rv_mlp *m);

rv_status rv_mlp_set_params(rv_mlp *m, const float *params);
rv_status rv_mlp_get_params(rv_mlp *m, float *params);

/* Host features [n][40] and labels (0/1); `epochs` passes in a seeded
 * shuffled order; epoch_loss[epochs] receives the mean loss of each epoch. */
rv_status rv_mlp_train(rv_mlp *m, const float *features, const float *labels, int64_t n, int epochs, float lr,
                       float pos_weight, uint64_t seed, float *epoch_loss);

/* Mean device time of one training step in the last rv_mlp_train call (a
 * step is one captured CUDA graph: gather, forward, backward, Adam). */
rv_status rv_mlp_step_ms(const rv_mlp *m, double *ms);

/* One forward and backward pass over n <= batch rows without an update:
 * the FP32 gradients (RV_MLP_PARAMS floats) and the mean loss. */
rv_status rv_mlp_gradients(rv_mlp *m, const float *features, const float *labels, int64_t n, float pos_weight,
                           float *grad, float *loss);

/* Probabilities (logistic of the output) for n feature rows. */
rv_status rv_mlp_predict(rv_mlp *m, const float *features, int64_t n, float *scores);

#ifdef __cplusplus
}
#endif
#endif
