// Softmax cross-entropy over rows of class scores in bf16 storage (sm_103a): the GCN's loss,
// log_softmax followed by the mean negative log-likelihood (gcn/pytorch-custom/gcn_custom.py,
// model output :90, loss :122-126), as one pass over the scores each way instead of torch's
// chain of slice, widen, log_softmax, gather, mean and their backward kernels.
//
// Forward: one thread per row streams the row in 8-score vectors with the running maximum and
// rescaled sum of the online softmax, so nothing is held per class: lse = m + log(s),
// loss_i = lse - x[label], and lse is kept for the backward. Rows are summed per CTA by a fixed
// tree, the CTA sums by one more fixed tree, then divided by n: deterministic.
// Backward: G[i, j] = (exp(x_j - lse_i) - [j == label]) * gscale / n in bf16 (round to nearest
// even), zero in the padding columns C .. width-1; gscale is read from device memory (the
// upstream gradient), so nothing synchronises.
#include "common.cuh"
#include "internal.h"

namespace as {
namespace {

constexpr int kThreads = 256;
constexpr int kMaxC = 64;  // classes per row (bounds the unrolled vector loops)

// Scores [8v, 8v + 8) of a row as fp32: one 16-byte load when VEC, else element loads (with
// elements at or past `lim` left at -inf).
template <bool VEC>
__device__ __forceinline__ void load8(const uint16_t *row, int v, int lim, float (&x)[8]) {
    if (VEC) {
        const uint4 w = __ldcs(reinterpret_cast<const uint4 *>(row) + v);
        const unsigned u[4] = {w.x, w.y, w.z, w.w};
#pragma unroll
        for (int q = 0; q < 4; ++q) {
            x[2 * q] = __uint_as_float(u[q] << 16);
            x[2 * q + 1] = __uint_as_float(u[q] & 0xffff0000u);
        }
    } else {
#pragma unroll
        for (int q = 0; q < 8; ++q) x[q] = 8 * v + q < lim ? bf16_to_f32(row[8 * v + q]) : -INFINITY;
    }
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
         const int64_t *__restrict__ labels, float *__restrict__ lse_out,
         float *__restrict__ partial, unsigned *status) {
    __shared__ float sm[kThreads / 32];
    const long i = static_cast<long>(blockIdx.x) * kThreads + threadIdx.x;
    float li = 0.0f;
    if (i < n) {
        const uint16_t *row = S + i * lds;
        const int64_t t = labels[i];
        float m = -INFINITY, sum = 0.0f, xt = 0.0f;
#pragma unroll
        for (int v = 0; v < kMaxC / 8; ++v) {
            if (8 * v >= C) break;
            float x[8];
            load8<VEC>(row, v, C, x);
            float mv = m;
#pragma unroll
            for (int q = 0; q < 8; ++q)
                if (8 * v + q < C) mv = fmaxf(mv, x[q]);
            float sv = 0.0f;
#pragma unroll
            for (int q = 0; q < 8; ++q) {
                if (8 * v + q < C) sv += expf(x[q] - mv);
                if (8 * v + q == t) xt = x[q];
            }
            sum = sum * expf(m - mv) + sv;  // exp(-inf) = 0 on the first vector
            m = mv;
        }
        const float lse = m + logf(sum);
        lse_out[i] = lse;
        if (t < 0 || t >= C)
            flag(status, kFlagBadLabel);
        else
            li = lse - xt;
    }
    const float tot = block_sum(li, sm);
    if (threadIdx.x == 0) partial[blockIdx.x] = tot;
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

// VEC: 16-byte score loads and 16-byte gradient stores (width a multiple of 8, rows aligned).
template <bool VEC>
__global__ void __launch_bounds__(kThreads)
xent_bwd(int n, int C, const uint16_t *__restrict__ S, long lds,
         const int64_t *__restrict__ labels, const float *__restrict__ lse_in,
         const float *__restrict__ gscale, float inv_n, uint16_t *__restrict__ G, long ldg,
         int width) {
    const long i = static_cast<long>(blockIdx.x) * kThreads + threadIdx.x;
    if (i >= n) return;
    const uint16_t *row = S + i * lds;
    const int64_t t = labels[i];
    const float lse = lse_in[i];
    const float scale = __ldg(gscale) * inv_n;
    const bool ok = t >= 0 && t < C;  // a bad label was flagged by the forward: zero gradient
    uint16_t *grow = G + i * ldg;
#pragma unroll
    for (int v = 0; v < kMaxC / 8; ++v) {
        if (8 * v >= width) break;
        float x[8], g[8];
        if (8 * v < C) {
            load8<VEC>(row, v, C, x);
        } else {
#pragma unroll
            for (int q = 0; q < 8; ++q) x[q] = -INFINITY;
        }
#pragma unroll
        for (int q = 0; q < 8; ++q) {
            const int j = 8 * v + q;
            g[q] = (ok && j < C) ? (expf(x[q] - lse) - (j == t ? 1.0f : 0.0f)) * scale : 0.0f;
        }
        if (VEC) {
            auto pk = [](float lo, float hi) {
                return static_cast<unsigned>(f32_to_bf16(lo)) |
                       (static_cast<unsigned>(f32_to_bf16(hi)) << 16);
            };
            *reinterpret_cast<uint4 *>(grow + 8 * v) =
                make_uint4(pk(g[0], g[1]), pk(g[2], g[3]), pk(g[4], g[5]), pk(g[6], g[7]));
        } else {
#pragma unroll
            for (int q = 0; q < 8; ++q)
                if (8 * v + q < width) grow[8 * v + q] = f32_to_bf16(g[q]);
        }
    }
}

// Whole 8-score vectors can be loaded (and, with G, stored) for every row.
bool vec_rows(int C, long lds, const void *S, int width, long ldg, const void *G) {
    const int Cv = (C + 7) / 8 * 8;
    const bool s_ok = lds % 8 == 0 && lds >= Cv && reinterpret_cast<uintptr_t>(S) % 16 == 0;
    if (!G) return s_ok;
    return s_ok && width % 8 == 0 && ldg % 8 == 0 && reinterpret_cast<uintptr_t>(G) % 16 == 0;
}

}  // namespace

as_status xent_fwd_launch(as_ctx *ctx, int n, int C, const uint16_t *S, long lds,
                          const int64_t *labels, float *lse, float *loss, cudaStream_t s) {
    if (C < 1 || C > kMaxC) return fail(AS_ERR_UNSUPPORTED, "softmax xent: 1 <= C <= 64 classes");
    const int blocks = static_cast<int>(ceil_div(n, kThreads));
    void *w = nullptr;
    as_status st = scratch(ctx, sizeof(float) * static_cast<size_t>(blocks > 0 ? blocks : 1), &w);
    if (st != AS_OK) return st;
    float *partial = static_cast<float *>(w);
    if (blocks > 0) {
        if (vec_rows(C, lds, S, 0, 0, nullptr))
            xent_fwd<true><<<blocks, kThreads, 0, s>>>(n, C, S, lds, labels, lse, partial,
                                                       ctx->d_status);
        else
            xent_fwd<false><<<blocks, kThreads, 0, s>>>(n, C, S, lds, labels, lse, partial,
                                                        ctx->d_status);
        ctx->launches++;
    }
    xent_finish<<<1, kThreads, 0, s>>>(blocks, partial, n > 0 ? 1.0f / static_cast<float>(n) : 0.0f,
                                       loss);
    ctx->launches++;
    return check_cuda(cudaGetLastError(), "softmax xent launch");
}

as_status xent_bwd_launch(as_ctx *ctx, int n, int C, const uint16_t *S, long lds,
                          const int64_t *labels, const float *lse, const float *gscale,
                          uint16_t *G, long ldg, int width, cudaStream_t s) {
    if (C < 1 || C > kMaxC || width < C || width > kMaxC)
        return fail(AS_ERR_UNSUPPORTED, "softmax xent: 1 <= C <= width <= 64 classes");
    if (n == 0) return AS_OK;
    const unsigned blocks = static_cast<unsigned>(ceil_div(n, kThreads));
    const float inv_n = 1.0f / static_cast<float>(n);
    if (vec_rows(C, lds, S, width, ldg, G))
        xent_bwd<true><<<blocks, kThreads, 0, s>>>(n, C, S, lds, labels, lse, gscale, inv_n, G,
                                                   ldg, width);
    else
        xent_bwd<false><<<blocks, kThreads, 0, s>>>(n, C, S, lds, labels, lse, gscale, inv_n, G,
                                                    ldg, width);
    ctx->launches++;
    return check_cuda(cudaGetLastError(), "softmax xent backward launch");
}

}  // namespace as
