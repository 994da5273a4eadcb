/* cor_window.h -- C ABI of the learned rigidity window (libcortrace.so).
 *
 * No counterpart in the reference: a small MLP maps a site-direction and its
 * conditions (COR_MLP_IN features) to predicted log R_U and log R_L; the scan
 * then traces only a window around the prediction and falls back to the full
 * scan when a boundary lands on a window edge, so every reported cutoff is
 * still traced.
 *
 * Network: COR_MLP_IN -> COR_MLP_LAYERS x COR_MLP_HIDDEN (SiLU) -> COR_MLP_OUT.
 * Weights and activations are BF16 on the tensor cores (tcgen05.mma, FP32
 * accumulation in tensor memory); FP32 master weights, AdamW.
 *
 * Parameters travel as one FP32 array in this order: W1[256][19], b1[256],
 * W2[256][256], b2[256], W3[256][256], b3[256], W4[256][256], b4[256],
 * W5[2][256], b5[2]  (W[out][in], y = W x + b).
 */
#ifndef COR_WINDOW_H
#define COR_WINDOW_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define COR_MLP_IN 19
#define COR_MLP_HIDDEN 256
#define COR_MLP_LAYERS 4
#define COR_MLP_OUT 2
#define COR_MLP_PARAMS (256 * 19 + 256 + 3 * (256 * 256 + 256) + 2 * 256 + 2)

typedef struct cor_mlp cor_mlp;

/* A network on `device` for batches of at most max_batch samples.  Every
 * buffer it needs is allocated here; the calls below allocate nothing. */
int cor_mlp_create(int device, int32_t max_batch, cor_mlp **out);
int cor_mlp_destroy(cor_mlp *m);
const char *cor_mlp_error(const cor_mlp *m);

/* Host FP32 parameters in, out (COR_MLP_PARAMS floats).  Setting them
 * resets the AdamW moments and step count. */
int cor_mlp_set_params(cor_mlp *m, const float *params);
int cor_mlp_get_params(cor_mlp *m, float *params);

/* Inference: x_dev n x COR_MLP_IN FP32 (normalised features), y_dev n x
 * COR_MLP_OUT FP32, both device memory; queued on `stream` (cudaStream_t). */
int cor_mlp_forward(cor_mlp *m, const float *x_dev, int32_t n, float *y_dev, void *stream);

/* One training step on a batch: forward, mean squared error against t_dev
 * (n x COR_MLP_OUT), backward, AdamW (lr, betas 0.9/0.999, eps 1e-8, decoupled
 * weight decay on the weight matrices).  loss_dev (device, 1 float) gets the
 * batch loss before the update; grads_dev (device, COR_MLP_PARAMS floats, may
 * be NULL) gets the gradient in the parameter layout. */
int cor_mlp_train_step(cor_mlp *m, const float *x_dev, const float *t_dev, int32_t n, float lr,
                       float weight_decay, float *loss_dev, float *grads_dev, void *stream);

/* The gradient alone (no update), for checking against a CPU restatement. */
int cor_mlp_gradient(cor_mlp *m, const float *x_dev, const float *t_dev, int32_t n, float *loss_dev,
                     float *grads_dev, void *stream);

#ifdef __cplusplus
}
#endif

#endif
