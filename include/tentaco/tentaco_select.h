/*
 * tentaco_select.h -- the learned variant selector of libtentaco_gb300.
 *
 * No counterpart in the reference, which chooses kernel variants with an
 * offline codegen sweep (generated_kernels/codegen.py:44-247, *_tune.sh) read
 * by a person.  Here a small network scores every variant of the MTTKRP walk
 * table from 12 tensor features (tt_csf_features in tentaco_gen.h); plans
 * created with TT_SELECT_MODEL run the variant it ranks first (the next one if
 * a staged variant does not fit the tensor's largest fiber window); for a tensor
 * outside the feature range the network was trained on, or when asked
 * (tt_plan_options::model_topk), they time its best-ranked few and keep the
 * fastest.  The
 * exhaustive sweep (TT_SELECT_SWEEP) stays the fallback and produces the
 * timings the network is trained on.  Selection never changes numerics beyond
 * the summation order of the chosen variant.
 *
 * Network: 12 -> 64 -> 64 -> 64 -> nout, ReLU on the hidden layers, FP32.
 * Parameters are one flat array, layer by layer: W (K x N row-major) then b (N).
 * Training kernels (forward, masked-MSE gradient, Adam) take DEVICE pointers
 * and run on the given stream; they are deterministic.
 */
#ifndef TENTACO_TENTACO_SELECT_H
#define TENTACO_TENTACO_SELECT_H
#include <stdint.h>
#include "tentaco.h"

#ifdef __cplusplus
extern "C" {
#endif

#define TT_MLP_IN 12
#define TT_MLP_HIDDEN 64

int64_t tt_mlp_num_params(int32_t nout);
/* FP32 scratch entries tt_mlp_forward / tt_mlp_grad need for a batch. */
int64_t tt_mlp_scratch_floats(int32_t batch, int32_t nout);

/* out (batch x nout) = network(X) for X (batch x 12, already normalised). */
tt_status tt_mlp_forward(const float* params, int32_t nout, const float* X, int32_t batch,
                         float* scratch, float* out, void* stream);

/*
 * Loss and gradient of the masked mean squared error
 *   loss = sum M (out - T)^2 / sum M
 * over batch x nout targets T and 0/1 mask M.  grads (tt_mlp_num_params
 * entries) and *loss (one float) are overwritten.
 */
tt_status tt_mlp_grad(const float* params, int32_t nout, const float* X, int32_t batch,
                      const float* T, const float* M, float* scratch, float* grads, float* loss,
                      void* stream);

/* One Adam step (bias-corrected, step >= 1) with decoupled weight decay. */
tt_status tt_mlp_adam(float* params, const float* grads, float* m, float* v, int64_t n, float lr,
                      float beta1, float beta2, float eps, float weight_decay, int32_t step,
                      void* stream);

/*
 * Selector model file ("TTSEL001"): header {magic[8], int32 version, n_in,
 * hidden, nout, n_models}, (version 3) int32 tensor order, then per model
 * {int32 storage class (0: FP32 storage, 1: 16-bit storage), float mean[12],
 * float std[12], (versions 2 and 3) float lo[12], float hi[12] (the training
 * tensors' feature range), float params[tt_mlp_num_params(nout)]}.
 * Little-endian.  Versions 1 and 2 hold three-mode models; a version 3 file
 * names its order (3 or 4) and replaces that order's models.
 *
 * path NULL: selector_model.bin in the directory of this library.  Each order's
 * default file (selector_model.bin, selector_model_o4.bin) is loaded on first use
 * by TT_SELECT_MODEL.  Returns TT_ERR_INVALID_ARGUMENT for a missing or malformed
 * file; the previously loaded models, if any, are kept.
 */
tt_status tt_selector_load(const char* path);
/* Number of three-mode models loaded (0: TT_SELECT_MODEL falls back to the heuristic). */
int32_t tt_selector_models(void);
/* Number of models loaded for tensors of this order (3 or 4; 0 otherwise). */
int32_t tt_selector_models_for_order(int32_t order);

/*
 * Run the network (on the current device) for tensor B at the given rank and
 * storage precision: scores[v] for v < n (n <= tt_num_variants()), lower
 * meaning predicted faster; variants not valid for the shape get +inf.
 * TT_ERR_UNSUPPORTED when no model covers the shape (orders 3 and 4).
 */
tt_status tt_selector_scores(const taco_tensor_t* B, int32_t rank, tt_precision prec, float* scores,
                             int32_t n);

/* How a plan's variant was chosen: 0 heuristic or fixed, 1 network, 2 sweep,
 * 3 fastest of the network's timed top-k candidates (tt_plan_options::model_topk). */
int32_t tt_plan_selected_by(const tt_plan* plan);

#ifdef __cplusplus
}
#endif
#endif
