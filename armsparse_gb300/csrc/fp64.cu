// FP64 SpMM and SDDMM, used only to check the autograd op's gradients against finite
// differences (float64 is required for a meaningful finite-difference check). Simple
// mappings: one thread per output element (SpMM) or per pattern entry (SDDMM).
#include "common.cuh"
#include "internal.h"

namespace as {
namespace {

constexpr int kThreads = 256;

__global__ void __launch_bounds__(kThreads)
spmm_f64_kernel(int M, int K, int N, int nnz, const int *__restrict__ rowptr,
                const int *__restrict__ colind, const double *__restrict__ val,
                const double *__restrict__ B, long ldb, double *__restrict__ C, long ldc,
                double beta, unsigned *status) {
    const long idx = static_cast<long>(blockIdx.x) * kThreads + threadIdx.x;
    if (idx >= static_cast<long>(M) * N) return;
    const int r = static_cast<int>(idx / N), j = static_cast<int>(idx % N);
    int lo, hi;
    row_range(rowptr, r, nnz, status, lo, hi);
    double acc = beta == 0.0 ? 0.0 : beta * C[r * ldc + j];
    for (int e = lo; e < hi; ++e) {
        const int k = __ldg(colind + e);
        if (static_cast<unsigned>(k) >= static_cast<unsigned>(K)) {
            flag(status, kFlagBadColind);
            continue;
        }
        acc = fma(__ldg(B + k * ldb + j), __ldg(val + e), acc);
    }
    C[r * ldc + j] = acc;
}

__global__ void __launch_bounds__(kThreads)
sddmm_f64_kernel(int M, int N, int K, int nnz, const int *__restrict__ rowptr,
                 const int *__restrict__ colind, const double *__restrict__ aval,
                 const double *__restrict__ X, long ldx, const double *__restrict__ Y, long ldy,
                 double *__restrict__ out, unsigned *status) {
    const long e = static_cast<long>(blockIdx.x) * kThreads + threadIdx.x;
    if (e >= nnz) return;
    int lo = 0, hi = M;
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(rowptr + mid) <= e) lo = mid; else hi = mid;
    }
    const int r = lo, c = __ldg(colind + e);
    if (__ldg(rowptr + r) > e || __ldg(rowptr + r + 1) <= e ||
        static_cast<unsigned>(c) >= static_cast<unsigned>(N)) {
        flag(status, kFlagBadColind);
        out[e] = 0.0;
        return;
    }
    double s = 0.0;
    for (int k = 0; k < K; ++k) s = fma(__ldg(X + r * ldx + k), __ldg(Y + c * ldy + k), s);
    out[e] = aval ? __ldg(aval + e) * s : s;
}

}  // namespace

as_status spmm_f64_launch(as_ctx *ctx, int M, int K, int N, int nnz, const int *rowptr,
                          const int *colind, const double *val, const double *B, long ldb,
                          double *C, long ldc, double beta, cudaStream_t s) {
    const long total = static_cast<long>(M) * N;
    spmm_f64_kernel<<<static_cast<unsigned>(ceil_div(total, kThreads)), kThreads, 0, s>>>(
        M, K, N, nnz, rowptr, colind, val, B, ldb, C, ldc, beta, ctx->d_status);
    ctx->launches++;
    return check_cuda(cudaGetLastError(), "spmm_f64 launch");
}

as_status sddmm_f64_launch(as_ctx *ctx, int M, int N, int K, int nnz, const int *rowptr,
                           const int *colind, const double *aval, const double *X, long ldx,
                           const double *Y, long ldy, double *out, cudaStream_t s) {
    if (M == 0) return fail(AS_ERR_INVALID_CSR, "sddmm_f64: nnz > 0 with zero rows");
    sddmm_f64_kernel<<<static_cast<unsigned>(ceil_div(nnz, kThreads)), kThreads, 0, s>>>(
        M, N, K, nnz, rowptr, colind, aval, X, ldx, Y, ldy, out, ctx->d_status);
    ctx->launches++;
    return check_cuda(cudaGetLastError(), "sddmm_f64 launch");
}

}  // namespace as
