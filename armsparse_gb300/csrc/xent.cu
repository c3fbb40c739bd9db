// Softmax cross-entropy over rows of class scores in bf16 storage (sm_103a): the GCN's loss,
// log_softmax followed by the mean negative log-likelihood (gcn/pytorch-custom/gcn_custom.py,
// model output :90, loss :122-126), as two passes over the scores instead of torch's chain of
// slice, widen, log_softmax, gather, mean and their backward kernels.
//
// Forward: one thread per row holds the row's C scores (widened to fp32); m = max, lse = m +
// log(sum exp(x - m)), loss_i = lse - x[label]. Rows are summed per CTA by a fixed tree, the
// CTA sums by one more fixed tree, then divided by n: deterministic.
// Backward: the same per-row lse, recomputed, and G[i, j] = (exp(x_j - lse) - [j == label]) *
// gscale / n in bf16 (round to nearest even), zero in the padding columns C .. width-1; gscale
// is read from device memory (the upstream gradient), so nothing synchronises.
#include "common.cuh"
#include "internal.h"

namespace as {
namespace {

constexpr int kThreads = 256;
constexpr int kMaxC = 64;  // classes held in registers per row

// The row's scores: 16-byte loads of 8 bf16 when VEC (row stride and base 16-byte aligned,
// room for whole vectors up to the next multiple of 8), else element loads.
template <bool VEC>
__device__ __forceinline__ void load_row(const uint16_t *row, int C, float (&x)[kMaxC]) {
    if (VEC) {
#pragma unroll
        for (int v = 0; v < kMaxC / 8; ++v) {
            if (8 * v < C) {
                const uint4 w = __ldcs(reinterpret_cast<const uint4 *>(row) + v);
                const unsigned u[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    x[8 * v + 2 * q] = __uint_as_float(u[q] << 16);
                    x[8 * v + 2 * q + 1] = __uint_as_float(u[q] & 0xffff0000u);
                }
            }
        }
    } else {
#pragma unroll
        for (int j = 0; j < kMaxC; ++j)
            if (j < C) x[j] = bf16_to_f32(row[j]);
    }
}

// log(sum_j exp(x_j)) over the first C entries, shifted by the maximum.
__device__ __forceinline__ float row_lse(const float (&x)[kMaxC], int C) {
    float m = x[0];
#pragma unroll
    for (int j = 1; j < kMaxC; ++j)
        if (j < C) m = fmaxf(m, x[j]);
    float s = 0.0f;
#pragma unroll
    for (int j = 0; j < kMaxC; ++j)
        if (j < C) s += expf(x[j] - m);
    return m + logf(s);
}

// Fixed-order sum over the CTA: butterfly within warps, then warp totals in warp order.
__device__ __forceinline__ float block_sum(float v, float *sm) {
#pragma unroll
    for (int off = 16; off >= 1; off >>= 1) v += __shfl_xor_sync(0xffffffffu, v, off);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    if (lane == 0) sm[warp] = v;
    __syncthreads();
    float t = 0.0f;
    if (threadIdx.x == 0)
        for (int w = 0; w < kThreads / 32; ++w) t += sm[w];
    return t;  // meaningful in thread 0
}

template <bool VEC>
__global__ void __launch_bounds__(kThreads)
xent_fwd(int n, int C, const uint16_t *__restrict__ S, long lds,
         const int64_t *__restrict__ labels, float *__restrict__ partial, unsigned *status) {
    __shared__ float sm[kThreads / 32];
    const long i = static_cast<long>(blockIdx.x) * kThreads + threadIdx.x;
    float li = 0.0f;
    if (i < n) {
        float x[kMaxC];
        load_row<VEC>(S + i * lds, C, x);
        const int64_t t = labels[i];
        if (t < 0 || t >= C) {
            flag(status, kFlagBadLabel);
        } else {
            float xt = x[0];
#pragma unroll
            for (int j = 1; j < kMaxC; ++j)
                if (j == t) xt = x[j];
            li = row_lse(x, C) - xt;
        }
    }
    const float t = block_sum(li, sm);
    if (threadIdx.x == 0) partial[blockIdx.x] = t;
}

// One CTA: the partials in a fixed order (each thread a strided run, then block_sum), / n.
__global__ void __launch_bounds__(kThreads)
xent_finish(int nparts, const float *__restrict__ partial, float inv_n, float *__restrict__ loss) {
    __shared__ float sm[kThreads / 32];
    float v = 0.0f;
    for (int p = threadIdx.x; p < nparts; p += kThreads) v += partial[p];
    const float t = block_sum(v, sm);
    if (threadIdx.x == 0) *loss = t * inv_n;
}

template <bool VEC>
__global__ void __launch_bounds__(kThreads)
xent_bwd(int n, int C, const uint16_t *__restrict__ S, long lds,
         const int64_t *__restrict__ labels, const float *__restrict__ gscale, float inv_n,
         uint16_t *__restrict__ G, long ldg, int width) {
    const long i = static_cast<long>(blockIdx.x) * kThreads + threadIdx.x;
    if (i >= n) return;
    float x[kMaxC];
    load_row<VEC>(S + i * lds, C, x);
    const int64_t t = labels[i];
    const float scale = __ldg(gscale) * inv_n;
    const float lse = row_lse(x, C);
    uint16_t *grow = G + i * ldg;
    const bool ok = t >= 0 && t < C;  // a bad label was flagged by the forward: zero gradient
#pragma unroll
    for (int j = 0; j < kMaxC; j += 2) {  // compile-time j: x[] stays in registers
        if (j >= width) break;
        float g[2];
#pragma unroll
        for (int q = 0; q < 2; ++q)
            g[q] = (ok && j + q < C) ? (expf(x[j + q] - lse) - (j + q == t ? 1.0f : 0.0f)) * scale
                                     : 0.0f;
        if (VEC) {  // width is even and the row 4-byte aligned
            *reinterpret_cast<unsigned *>(grow + j) =
                static_cast<unsigned>(f32_to_bf16(g[0])) |
                (static_cast<unsigned>(f32_to_bf16(g[1])) << 16);
        } else {
            grow[j] = f32_to_bf16(g[0]);
            if (j + 1 < width) grow[j + 1] = f32_to_bf16(g[1]);
        }
    }
}

bool vec_rows(int C, long ld, int width, const void *p, const void *q) {
    const int Cv = (C + 7) / 8 * 8;  // whole 8-element vectors of the scores
    return ld % 8 == 0 && ld >= Cv && width % 2 == 0 &&
           reinterpret_cast<uintptr_t>(p) % 16 == 0 && (q == nullptr || reinterpret_cast<uintptr_t>(q) % 4 == 0);
}

}  // namespace

as_status xent_fwd_launch(as_ctx *ctx, int n, int C, const uint16_t *S, long lds,
                          const int64_t *labels, float *loss, cudaStream_t s) {
    if (C < 1 || C > kMaxC) return fail(AS_ERR_UNSUPPORTED, "softmax xent: 1 <= C <= 64 classes");
    const int blocks = static_cast<int>(ceil_div(n, kThreads));
    void *w = nullptr;
    as_status st = scratch(ctx, sizeof(float) * static_cast<size_t>(blocks > 0 ? blocks : 1), &w);
    if (st != AS_OK) return st;
    float *partial = static_cast<float *>(w);
    if (blocks > 0) {
        if (vec_rows(C, lds, 2, S, nullptr))
            xent_fwd<true><<<blocks, kThreads, 0, s>>>(n, C, S, lds, labels, partial, ctx->d_status);
        else
            xent_fwd<false><<<blocks, kThreads, 0, s>>>(n, C, S, lds, labels, partial, ctx->d_status);
        ctx->launches++;
    }
    xent_finish<<<1, kThreads, 0, s>>>(blocks, partial, n > 0 ? 1.0f / static_cast<float>(n) : 0.0f,
                                       loss);
    ctx->launches++;
    return check_cuda(cudaGetLastError(), "softmax xent launch");
}

as_status xent_bwd_launch(as_ctx *ctx, int n, int C, const uint16_t *S, long lds,
                          const int64_t *labels, const float *gscale, uint16_t *G, long ldg,
                          int width, cudaStream_t s) {
    if (C < 1 || C > kMaxC || width < C || width > kMaxC)
        return fail(AS_ERR_UNSUPPORTED, "softmax xent: 1 <= C <= width <= 64 classes");
    if (n == 0) return AS_OK;
    const unsigned blocks = static_cast<unsigned>(ceil_div(n, kThreads));
    const float inv_n = 1.0f / static_cast<float>(n);
    if (vec_rows(C, lds, width, S, G) && ldg % 2 == 0)
        xent_bwd<true><<<blocks, kThreads, 0, s>>>(n, C, S, lds, labels, gscale, inv_n, G, ldg, width);
    else
        xent_bwd<false><<<blocks, kThreads, 0, s>>>(n, C, S, lds, labels, gscale, inv_n, G, ldg, width);
    ctx->launches++;
    return check_cuda(cudaGetLastError(), "softmax xent backward launch");
}

}  // namespace as
