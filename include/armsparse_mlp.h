/*
 * armsparse_mlp.h -- the small dense-network kernels the learned kernel selector is trained
 * with (no counterpart in the reference, whose only kernel choice is a static switch on the
 * dense width, gcn/pytorch-custom/spmm_kernel.cu:437-457). FP32, deterministic (one thread
 * per output element, fixed reduction order), asynchronous on `stream`.
 *
 * Shapes: X [B x I] row-major, W [O x I] (one row per output unit), bias [O], Y [B x O].
 */
#ifndef ARMSPARSE_MLP_H
#define ARMSPARSE_MLP_H

#include "armsparse_gpu.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Y = X W^T + bias (bias may be NULL); relu != 0 applies max(0, .). */
as_status as_mlp_linear_fwd(as_ctx *ctx, int B, int I, int O, const float *X, const float *W,
                            const float *bias, float *Y, int relu, void *stream);
/* dW = dY^T X, dbias = column sums of dY (may be NULL), dX = dY W (may be NULL); when relu_in is
 * given (the layer input, itself a ReLU output), dX is zeroed where relu_in <= 0. */
as_status as_mlp_linear_bwd(as_ctx *ctx, int B, int I, int O, const float *dY, const float *X,
                            const float *W, const float *relu_in, float *dX, float *dW,
                            float *dbias, void *stream);
/* Soft-target cross entropy over V classes per row: loss[r] = -sum_v T log softmax(Z)[v] (loss
 * may be NULL), dZ = (softmax(Z) - T) * scale (dZ may be NULL). */
as_status as_mlp_softmax_xent(as_ctx *ctx, int B, int V, const float *Z, const float *T,
                              float *loss, float *dZ, float scale, void *stream);
/* Adam with bias correction and decoupled-style L2 term: g' = g + weight_decay * p. */
as_status as_mlp_adam(as_ctx *ctx, long n, float *param, const float *grad, float *m, float *v,
                      float lr, float beta1, float beta2, float eps, float weight_decay, int step,
                      void *stream);

#ifdef __cplusplus
}
#endif

#endif /* ARMSPARSE_MLP_H */
