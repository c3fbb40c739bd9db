// Small dense-network kernels for the learned kernel selector (sm_103a, FP32).
//
// The selector is a multilayer perceptron over a few dozen matrix features; its training
// batches have a few hundred rows and its layers a few dozen units, so every kernel maps one
// thread to one output element and loops over the reduction in a fixed order: results are
// deterministic run to run (no atomics). Shapes: X [B x I], W [O x I] (row-major, one row per
// output unit), bias [O], Y [B x O].
#include "armsparse_mlp.h"
#include "common.cuh"
#include "internal.h"

namespace as {
namespace {

constexpr int kThreads = 256;

// Y = X W^T + b, optionally ReLU
__global__ void __launch_bounds__(kThreads)
linear_fwd(int Bn, int I, int O, const float *__restrict__ X, const float *__restrict__ W,
           const float *__restrict__ b, float *__restrict__ Y, int relu) {
    const long idx = static_cast<long>(blockIdx.x) * kThreads + threadIdx.x;
    if (idx >= static_cast<long>(Bn) * O) return;
    const int r = static_cast<int>(idx / O), o = static_cast<int>(idx % O);
    float s = b ? b[o] : 0.0f;
    for (int i = 0; i < I; ++i) s = fmaf(X[static_cast<long>(r) * I + i], W[static_cast<long>(o) * I + i], s);
    Y[idx] = relu && s < 0.0f ? 0.0f : s;
}

// dX = dY W (optionally masked by the ReLU of the layer input's producer: dX *= (A > 0))
__global__ void __launch_bounds__(kThreads)
linear_bwd_x(int Bn, int I, int O, const float *__restrict__ dY, const float *__restrict__ W,
             const float *__restrict__ relu_out, float *__restrict__ dX) {
    const long idx = static_cast<long>(blockIdx.x) * kThreads + threadIdx.x;
    if (idx >= static_cast<long>(Bn) * I) return;
    const int r = static_cast<int>(idx / I), i = static_cast<int>(idx % I);
    float s = 0.0f;
    for (int o = 0; o < O; ++o) s = fmaf(dY[static_cast<long>(r) * O + o], W[static_cast<long>(o) * I + i], s);
    if (relu_out && relu_out[idx] <= 0.0f) s = 0.0f;
    dX[idx] = s;
}

// dW = dY^T X, db = column sums of dY
__global__ void __launch_bounds__(kThreads)
linear_bwd_w(int Bn, int I, int O, const float *__restrict__ dY, const float *__restrict__ X,
             float *__restrict__ dW, float *__restrict__ db) {
    const long idx = static_cast<long>(blockIdx.x) * kThreads + threadIdx.x;
    const long nw = static_cast<long>(O) * I;
    if (idx < nw) {
        const int o = static_cast<int>(idx / I), i = static_cast<int>(idx % I);
        float s = 0.0f;
        for (int r = 0; r < Bn; ++r) s = fmaf(dY[static_cast<long>(r) * O + o], X[static_cast<long>(r) * I + i], s);
        dW[idx] = s;
    } else if (idx < nw + O && db) {
        const int o = static_cast<int>(idx - nw);
        float s = 0.0f;
        for (int r = 0; r < Bn; ++r) s += dY[static_cast<long>(r) * O + o];
        db[o] = s;
    }
}

// Soft-target cross entropy over V classes, one warp per row: loss[r] = -sum_v t log softmax(z),
// dZ = (softmax(z) - t) * scale.
__global__ void __launch_bounds__(kThreads)
softmax_xent(int Bn, int V, const float *__restrict__ Z, const float *__restrict__ T,
             float *__restrict__ loss, float *__restrict__ dZ, float scale) {
    const long w = (static_cast<long>(blockIdx.x) * kThreads + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= Bn) return;
    const float *z = Z + w * V;
    const float *t = T + w * V;
    float m = -INFINITY;
    for (int v = lane; v < V; v += 32) m = fmaxf(m, z[v]);
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    float se = 0.0f;
    for (int v = lane; v < V; v += 32) se += expf(z[v] - m);
    for (int o = 16; o > 0; o >>= 1) se += __shfl_xor_sync(0xffffffffu, se, o);
    const float lse = m + logf(se);
    float l = 0.0f;
    for (int v = lane; v < V; v += 32) {
        const float p = expf(z[v] - lse);
        l -= t[v] * (z[v] - lse);
        if (dZ) dZ[w * V + v] = (p - t[v]) * scale;
    }
    for (int o = 16; o > 0; o >>= 1) l += __shfl_xor_sync(0xffffffffu, l, o);
    if (lane == 0 && loss) loss[w] = l;
}

// Adam (bias-corrected), in place.
__global__ void __launch_bounds__(kThreads)
adam(long n, float *__restrict__ p, const float *__restrict__ g, float *__restrict__ m,
     float *__restrict__ v, float lr, float b1, float b2, float eps, float wd, int step) {
    const long i = static_cast<long>(blockIdx.x) * kThreads + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i] + wd * p[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float mh = mi / (1.0f - powf(b1, static_cast<float>(step)));
    const float vh = vi / (1.0f - powf(b2, static_cast<float>(step)));
    p[i] -= lr * mh / (sqrtf(vh) + eps);
}

unsigned blocks(long n) { return static_cast<unsigned>(ceil_div(n, kThreads)); }

}  // namespace
}  // namespace as

using namespace as;

extern "C" {

as_status as_mlp_linear_fwd(as_ctx *ctx, int B, int I, int O, const float *X, const float *W,
                            const float *bias, float *Y, int relu, void *stream) {
    if (!ctx || B < 0 || I < 0 || O < 0 || (B * O > 0 && (!X || !W || !Y)))
        return fail(AS_ERR_INVALID_VALUE, "as_mlp_linear_fwd: bad arguments");
    if (static_cast<long>(B) * O == 0) return AS_OK;
    linear_fwd<<<blocks(static_cast<long>(B) * O), kThreads, 0, static_cast<cudaStream_t>(stream)>>>(
        B, I, O, X, W, bias, Y, relu);
    ctx->launches++;
    return check_cuda(cudaGetLastError(), "as_mlp_linear_fwd");
}

as_status as_mlp_linear_bwd(as_ctx *ctx, int B, int I, int O, const float *dY, const float *X,
                            const float *W, const float *relu_in, float *dX, float *dW,
                            float *dbias, void *stream) {
    if (!ctx || B < 0 || I < 0 || O < 0 || !dY || !X || !W || !dW)
        return fail(AS_ERR_INVALID_VALUE, "as_mlp_linear_bwd: bad arguments");
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (dX && static_cast<long>(B) * I > 0) {
        linear_bwd_x<<<blocks(static_cast<long>(B) * I), kThreads, 0, s>>>(B, I, O, dY, W, relu_in, dX);
        ctx->launches++;
    }
    linear_bwd_w<<<blocks(static_cast<long>(O) * I + O), kThreads, 0, s>>>(B, I, O, dY, X, dW, dbias);
    ctx->launches++;
    return check_cuda(cudaGetLastError(), "as_mlp_linear_bwd");
}

as_status as_mlp_softmax_xent(as_ctx *ctx, int B, int V, const float *Z, const float *T,
                              float *loss, float *dZ, float scale, void *stream) {
    if (!ctx || B < 0 || V <= 0 || !Z || !T) return fail(AS_ERR_INVALID_VALUE, "as_mlp_softmax_xent: bad arguments");
    if (B == 0) return AS_OK;
    softmax_xent<<<blocks(static_cast<long>(B) * 32), kThreads, 0, static_cast<cudaStream_t>(stream)>>>(
        B, V, Z, T, loss, dZ, scale);
    ctx->launches++;
    return check_cuda(cudaGetLastError(), "as_mlp_softmax_xent");
}

as_status as_mlp_adam(as_ctx *ctx, long n, float *param, const float *grad, float *m, float *v,
                      float lr, float beta1, float beta2, float eps, float weight_decay, int step,
                      void *stream) {
    if (!ctx || n < 0 || (n > 0 && (!param || !grad || !m || !v)) || step < 1)
        return fail(AS_ERR_INVALID_VALUE, "as_mlp_adam: bad arguments");
    if (n == 0) return AS_OK;
    adam<<<blocks(n), kThreads, 0, static_cast<cudaStream_t>(stream)>>>(n, param, grad, m, v, lr, beta1,
                                                                       beta2, eps, weight_decay, step);
    ctx->launches++;
    return check_cuda(cudaGetLastError(), "as_mlp_adam");
}

}  // extern "C"
