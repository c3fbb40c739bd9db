// CSR SpMV, y = A*x + beta*y (sm_103a).
//
// Plain CSR: a group of GROUP lanes per row (GROUP picked from the mean row length so that
// short rows do not idle a whole warp); lane g sums entries g, g+GROUP, ... with fmaf, then
// the group reduces with xor shuffles (fixed tree, deterministic).
//
// 1x4-blocked layout of the reference (SpMV.cpp:15-38, consumed at SpMV.cpp:155-179): one
// thread per row keeps the reference's four lane sums s_l += val[idx+l] * x[k+l] over the
// row's blocks in order (fused steps, as GCC emits vmlaq_f32 under -ffp-contract=fast) and
// combines them as (s2 + s0) + (s3 + s1) before adding to y.
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

__global__ void __launch_bounds__(kThreads)
spmv_vcsr4(int M, int K, int nslots, const int *__restrict__ rowptr,
           const int *__restrict__ colind, const float *__restrict__ val,
           const float *__restrict__ x, float *__restrict__ y, float beta, unsigned *status) {
    const long row = static_cast<long>(blockIdx.x) * kThreads + threadIdx.x;
    if (row >= M) return;
    int lo, hi;
    row_range(rowptr, static_cast<int>(row), nslots, status, lo, hi);
    if ((lo & 3) || (hi & 3)) {
        flag(status, kFlagBadRowptr);
        lo = hi = 0;
    }
    float s0 = 0.f, s1 = 0.f, s2 = 0.f, s3 = 0.f;
    for (int idx = lo; idx < hi; idx += 4) {
        const int k = ld_stream(colind + idx);
        if (k < 0 || k > K - 4) {
            flag(status, kFlagBadColind);
            continue;
        }
        const float4 v = __ldcs(reinterpret_cast<const float4 *>(val + idx));
        s0 = fmaf(v.x, __ldg(x + k + 0), s0);
        s1 = fmaf(v.y, __ldg(x + k + 1), s1);
        s2 = fmaf(v.z, __ldg(x + k + 2), s2);
        s3 = fmaf(v.w, __ldg(x + k + 3), s3);
    }
    const float r = __fadd_rn(__fadd_rn(s2, s0), __fadd_rn(s3, s1));
    y[row] = beta == 0.0f ? r : __fadd_rn(beta * y[row], r);
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
    const unsigned grid = static_cast<unsigned>(ceil_div(M, kThreads));
    spmv_vcsr4<<<grid, kThreads, 0, s>>>(M, K, nslots, rowptr, colind, val, x, y, beta,
                                         ctx->d_status);
    ctx->launches++;
    return check_cuda(cudaGetLastError(), "spmv_vcsr4 launch");
}

}  // namespace as
