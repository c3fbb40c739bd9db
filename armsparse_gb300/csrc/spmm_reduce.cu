// SpMM over other reductions (sm_103a): C[i, :] = reduce_{e in row i} w_e * B[col(e), :] with
// reduce = sum or max, w_e = val[e] or 1 (val == NULL). The unweighted sum is the copy-sum
// aggregation of the reference's topo*SPMMKernel family (gcn/pytorch-custom/spmm_kernel.cu:
// 31-207; each output is acc += B[...] in CSR order, reproduced here add for add); the
// weighted sum is the FMA chain of the SpMM; max is the copy-max aggregation of the DGL
// kernels (binary_reduce_max.cu:26-168). OP 0 = sum, 1 = max from -inf (fmaxf), both giving 0
// for rows without entries; OP 2 = the DGL kernels' own max: the accumulator starts at -10000
// (max_init, binary_reduce_max.cu:22-24) and takes acc = acc > x ? acc : x (max_reduce, :18-20)
// in CSR order, so an empty row stays at -10000.
//
// One warp per row; lane l owns columns l, l+32, ... of a 32*CPL-column tile (scalar loads,
// any N); 4 entries per step.
#include "common.cuh"
#include "internal.h"

namespace as {
namespace {

constexpr int kThreads = 256;

template <int OP, bool WEIGHTED, int CPL>
__global__ void __launch_bounds__(kThreads)
spmm_reduce(int M, int K, int N, int nnz, const int *__restrict__ rowptr,
            const int *__restrict__ colind, const float *__restrict__ val,
            const float *__restrict__ B, long ldb, float *__restrict__ C, long ldc,
            unsigned *status) {
    const int lane = threadIdx.x & 31;
    const long row = static_cast<long>(blockIdx.x) * (kThreads / 32) + (threadIdx.x >> 5);
    if (row >= M) return;
    int lo, hi;
    row_range(rowptr, static_cast<int>(row), nnz, status, lo, hi);
    const int tile0 = blockIdx.y * 32 * CPL;
    float acc[CPL];
#pragma unroll
    for (int j = 0; j < CPL; ++j) acc[j] = OP == 0 ? 0.0f : OP == 1 ? -INFINITY : -10000.0f;
    for (int base = lo; base < hi; base += 32) {
        const int e = base + lane;
        int k = -1;
        float w = 1.0f;
        if (e < hi) {
            k = ld_stream(colind + e);
            if (WEIGHTED) w = ld_stream(val + e);
            if (static_cast<unsigned>(k) >= static_cast<unsigned>(K)) {
                flag(status, kFlagBadColind);
                k = -1;
            }
        }
        const int cnt = min(32, hi - base);
        for (int t = 0; t < cnt; ++t) {
            const int kk = __shfl_sync(0xffffffffu, k, t);
            const float ww = __shfl_sync(0xffffffffu, w, t);
            if (kk < 0) continue;
            const float *brow = B + static_cast<long>(kk) * ldb;
#pragma unroll
            for (int j = 0; j < CPL; ++j) {
                const int c = tile0 + j * 32 + lane;
                if (c < N) {
                    const float b = __ldg(brow + c);
                    if (OP == 0)  // weighted: the FMA chain of the SpMM; unweighted: plain adds
                        acc[j] = WEIGHTED ? fmaf(b, ww, acc[j]) : __fadd_rn(acc[j], b);
                    else if (OP == 1)
                        acc[j] = fmaxf(acc[j], WEIGHTED ? __fmul_rn(ww, b) : b);
                    else {
                        const float x = WEIGHTED ? __fmul_rn(ww, b) : b;
                        acc[j] = acc[j] > x ? acc[j] : x;
                    }
                }
            }
        }
    }
#pragma unroll
    for (int j = 0; j < CPL; ++j) {
        const int c = tile0 + j * 32 + lane;
        if (c < N) C[row * ldc + c] = (hi == lo && OP != 2) ? 0.0f : acc[j];
    }
}

template <int OP, bool W>
void launch(const SpmmArgs &a, cudaStream_t s) {
    constexpr int CPL = 4;
    dim3 grid(static_cast<unsigned>(ceil_div(a.M, kThreads / 32)),
              static_cast<unsigned>(ceil_div(a.N, 32 * CPL)));
    spmm_reduce<OP, W, CPL><<<grid, kThreads, 0, s>>>(a.M, a.K, a.N, a.nnz, a.rowptr, a.colind,
                                                      static_cast<const float *>(a.val),
                                                      static_cast<const float *>(a.B), a.ldb,
                                                      a.C, a.ldc, a.status);
}

}  // namespace

as_status spmm_reduce_launch(as_ctx *ctx, int op, const SpmmArgs &a, cudaStream_t s) {
    if (ceil_div(a.N, 128) > 65535) return fail(AS_ERR_UNSUPPORTED, "spmm reduce: N too large");
    const bool w = a.val != nullptr;
    if (op == 0) w ? launch<0, true>(a, s) : launch<0, false>(a, s);
    else if (op == 1) w ? launch<1, true>(a, s) : launch<1, false>(a, s);
    else w ? launch<2, true>(a, s) : launch<2, false>(a, s);
    ctx->launches++;
    return check_cuda(cudaGetLastError(), "spmm reduce launch");
}

}  // namespace as
