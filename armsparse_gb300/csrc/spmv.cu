// CSR SpMV, y = A*x + beta*y (sm_103a).
//
// Plain CSR: a group of GROUP lanes per row (GROUP picked from the mean row length so that
// short rows do not idle a whole warp); lane g sums entries g, g+GROUP, ... with fmaf, then
// the group reduces with xor shuffles (fixed tree, deterministic).
//
// 1x4-blocked layout of the reference (SpMV.cpp:15-38, consumed at SpMV.cpp:155-179): four
// lanes per row keep the reference's four lane sums s_l += val[idx+l] * x[k+l] over the row's
// blocks in order (fused steps, as GCC emits vmlaq_f32 under -ffp-contract=fast) and combine
// them as (s2 + s0) + (s3 + s1) before adding to y.
#include "common.cuh"
#include "internal.h"

namespace as {
namespace {

constexpr int kThreads = 256;

template <int GROUP>
__global__ void __launch_bounds__(kThreads)
spmv_csr(int M, int K, int nnz, const int *__restrict__ rowptr, const int *__restrict__ colind,
         const float *__restrict__ val, const float *__restrict__ x, float *__restrict__ y,
         float beta, unsigned *status) {
    const int lane = threadIdx.x & 31;
    const int g = threadIdx.x % GROUP;
    const unsigned gmask =
        GROUP == 32 ? 0xffffffffu : (((1u << GROUP) - 1u) << (lane & ~(GROUP - 1)));
    const long row = static_cast<long>(blockIdx.x) * (kThreads / GROUP) + threadIdx.x / GROUP;
    if (row >= M) return;
    int lo, hi;
    row_range(rowptr, static_cast<int>(row), nnz, status, lo, hi);
    float s = 0.0f;
    for (int e = lo + g; e < hi; e += GROUP) {
        const int k = ld_stream(colind + e);
        if (static_cast<unsigned>(k) >= static_cast<unsigned>(K)) {
            flag(status, kFlagBadColind);
            continue;
        }
        s = fmaf(ld_stream(val + e), __ldg(x + k), s);
    }
#pragma unroll
    for (int off = GROUP / 2; off > 0; off >>= 1) s += __shfl_xor_sync(gmask, s, off, GROUP);
    if (g == 0) y[row] = beta == 0.0f ? s : fmaf(beta, y[row], s);
}

// Four lanes per row: lane l keeps the chain s_l (so each chain stays in block order) and
// issues U blocks' loads before their FMAs; the lanes combine with two xor shuffles, lane 0
// ending with (s2 + s0) + (s3 + s1).
template <int U>
__global__ void __launch_bounds__(kThreads)
spmv_vcsr4(int M, int K, int nslots, const int *__restrict__ rowptr,
           const int *__restrict__ colind, const float *__restrict__ val,
           const float *__restrict__ x, float *__restrict__ y, float beta, unsigned *status) {
    const long row = (static_cast<long>(blockIdx.x) * kThreads + threadIdx.x) >> 2;
    const int l = threadIdx.x & 3;
    const unsigned gmask = 0xfu << (threadIdx.x & 28);
    if (row >= M) return;  // the four lanes of a row leave together
    int lo, hi;
    row_range(rowptr, static_cast<int>(row), nslots, status, lo, hi);
    if ((lo & 3) || (hi & 3)) {
        flag(status, kFlagBadRowptr);
        lo = hi = 0;
    }
    float s = 0.f;
    int idx = lo;
    for (; idx + 4 * U <= hi; idx += 4 * U) {
        int k[U];
        float v[U], xv[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            k[u] = ld_stream(colind + idx + 4 * u);
            v[u] = ld_stream(val + idx + 4 * u + l);
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const bool ok = k[u] >= 0 && k[u] <= K - 4;
            if (!ok) {
                flag(status, kFlagBadColind);
                k[u] = -1;
            }
            xv[u] = ok ? __ldg(x + k[u] + l) : 0.f;
        }
#pragma unroll
        for (int u = 0; u < U; ++u)
            if (k[u] >= 0) s = fmaf(v[u], xv[u], s);
    }
    for (; idx < hi; idx += 4) {
        const int k = ld_stream(colind + idx);
        if (k < 0 || k > K - 4) {
            flag(status, kFlagBadColind);
            continue;
        }
        s = fmaf(ld_stream(val + idx + l), __ldg(x + k + l), s);
    }
    const float p = __fadd_rn(__shfl_xor_sync(gmask, s, 2), s);  // lane 0: s2+s0, lane 1: s3+s1
    const float r = __fadd_rn(p, __shfl_xor_sync(gmask, p, 1));
    if (l == 0) y[row] = beta == 0.0f ? r : __fadd_rn(beta * y[row], r);
}

}  // namespace

as_status spmv_csr_launch(as_ctx *ctx, int M, int K, int nnz, const int *rowptr,
                          const int *colind, const float *val, const float *x, float *y,
                          float beta, cudaStream_t s) {
    const double mean = M > 0 ? static_cast<double>(nnz) / M : 0.0;
    int group = 2;
    while (group < 32 && group < mean) group <<= 1;
    const unsigned grid = static_cast<unsigned>(ceil_div(M, kThreads / group));
    switch (group) {
        case 2: spmv_csr<2><<<grid, kThreads, 0, s>>>(M, K, nnz, rowptr, colind, val, x, y, beta, ctx->d_status); break;
        case 4: spmv_csr<4><<<grid, kThreads, 0, s>>>(M, K, nnz, rowptr, colind, val, x, y, beta, ctx->d_status); break;
        case 8: spmv_csr<8><<<grid, kThreads, 0, s>>>(M, K, nnz, rowptr, colind, val, x, y, beta, ctx->d_status); break;
        case 16: spmv_csr<16><<<grid, kThreads, 0, s>>>(M, K, nnz, rowptr, colind, val, x, y, beta, ctx->d_status); break;
        default: spmv_csr<32><<<grid, kThreads, 0, s>>>(M, K, nnz, rowptr, colind, val, x, y, beta, ctx->d_status); break;
    }
    ctx->launches++;
    return check_cuda(cudaGetLastError(), "spmv_csr launch");
}

as_status spmv_vcsr4_launch(as_ctx *ctx, int M, int K, int nslots, const int *rowptr,
                            const int *colind, const float *val, const float *x, float *y,
                            float beta, cudaStream_t s) {
    if (reinterpret_cast<uintptr_t>(val) % 16)
        return fail(AS_ERR_INVALID_VALUE, "as_spmv_vcsr4_f32: val must be 16-byte aligned");
    const unsigned grid = static_cast<unsigned>(ceil_div(static_cast<long>(M) * 4, kThreads));
    spmv_vcsr4<8><<<grid, kThreads, 0, s>>>(M, K, nslots, rowptr, colind, val, x, y, beta,
                                         ctx->d_status);
    ctx->launches++;
    return check_cuda(cudaGetLastError(), "spmv_vcsr4 launch");
}

}  // namespace as
