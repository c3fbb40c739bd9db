// SpMM over other reductions (sm_103a): C[i, :] = reduce_{e in row i} w_e * B[col(e), :] with
// reduce = sum or max, w_e = val[e] or 1 (val == NULL). The weighted sum runs as the SpMM
// (spmm.cu: the same fused multiply-add chain from zero). The unweighted sum is the copy-sum
// aggregation of the reference's topo*SPMMKernel family (gcn/pytorch-custom/spmm_kernel.cu:
// 31-207; each output is acc += B[...] in CSR order, reproduced here add for add); the
// weighted sum is the FMA chain of the SpMM; max is the copy-max aggregation of the DGL
// kernels (binary_reduce_max.cu:26-168). OP 0 = sum, 1 = max from -inf (fmaxf), both giving 0
// for rows without entries; OP 2 = the DGL kernels' own max: the accumulator starts at -10000
// (max_init, binary_reduce_max.cu:22-24) and takes acc = acc > x ? acc : x (max_reduce, :18-20)
// in CSR order, so an empty row stays at -10000.
//
// One warp per row; each lane owns CPL vectors of E columns of the row's column tile (16-byte
// loads where the layout allows, scalar otherwise). Rows with more than kLongRow entries are left to the long-row kernel (spmm_long.cu,
// launched next with the same reduction as its chain step), as in the row-split SpMM: a hub
// row would otherwise keep one warp busy for the whole call.
#include <limits.h>

#include "common.cuh"
#include "internal.h"

namespace as {
namespace {

constexpr int kThreads = 256;

// E columns per lane (4: 16-byte loads and stores, when N, ldb, ldc and the pointers allow
// them; 1: scalar), CPL vectors per lane: a 32 * E * CPL-column tile.
template <int OP, bool WEIGHTED, int CPL, int E>
__global__ void __launch_bounds__(kThreads)
spmm_reduce(int M, int K, int N, int nnz, const int *__restrict__ rowptr,
            const int *__restrict__ colind, const float *__restrict__ val,
            const float *__restrict__ B, long ldb, float *__restrict__ C, long ldc,
            unsigned *status, int long_thresh, int *long_list, unsigned *long_count) {
    // let the long-row kernel (a programmatic dependent) be scheduled early; it waits for this
    // grid to complete before it reads the list
    asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory");
    const int lane = threadIdx.x & 31;
    const long row = static_cast<long>(blockIdx.x) * (kThreads / 32) + (threadIdx.x >> 5);
    if (row >= M) return;
    int lo, hi;
    row_range(rowptr, static_cast<int>(row), nnz, status, lo, hi);
    if (hi - lo > long_thresh) {  // left to the long-row kernel
        if (blockIdx.y == 0 && lane == 0) list_long_row(row, hi - lo, M, long_list, long_count, status);
        return;
    }
    const int tile0 = blockIdx.y * 32 * E * CPL;
    float acc[CPL][E];
#pragma unroll
    for (int j = 0; j < CPL; ++j)
#pragma unroll
        for (int i = 0; i < E; ++i) acc[j][i] = OP == 0 ? 0.0f : OP == 1 ? -INFINITY : -10000.0f;
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
                const int c = tile0 + (j * 32 + lane) * E;
                if (c < N) {
                    float b[E];
                    if constexpr (E == 4) {
                        const float4 q = __ldg(reinterpret_cast<const float4 *>(brow + c));
                        b[0] = q.x; b[1] = q.y; b[2] = q.z; b[3] = q.w;
                    } else {
                        b[0] = __ldg(brow + c);
                    }
#pragma unroll
                    for (int i = 0; i < E; ++i) {
                        if (OP == 0)  // weighted: the FMA chain of the SpMM; unweighted: plain adds
                            acc[j][i] = WEIGHTED ? fmaf(b[i], ww, acc[j][i]) : __fadd_rn(acc[j][i], b[i]);
                        else if (OP == 1)
                            acc[j][i] = fmaxf(acc[j][i], WEIGHTED ? __fmul_rn(ww, b[i]) : b[i]);
                        else {
                            const float x = WEIGHTED ? __fmul_rn(ww, b[i]) : b[i];
                            acc[j][i] = acc[j][i] > x ? acc[j][i] : x;
                        }
                    }
                }
            }
        }
    }
    const bool empty = hi == lo && OP != 2;
#pragma unroll
    for (int j = 0; j < CPL; ++j) {
        const int c = tile0 + (j * 32 + lane) * E;
        if (c < N) {
            if constexpr (E == 4) {
                *reinterpret_cast<float4 *>(C + row * ldc + c) =
                    empty ? make_float4(0.0f, 0.0f, 0.0f, 0.0f)
                          : make_float4(acc[j][0], acc[j][1], acc[j][2], acc[j][3]);
            } else {
                C[row * ldc + c] = empty ? 0.0f : acc[j][0];
            }
        }
    }
}

template <int OP, bool W>
void launch(const SpmmArgs &a, bool vec, int thresh, int *list, unsigned *counters,
            cudaStream_t s) {
    auto go = [&](auto kernel, int tile) {
        dim3 grid(static_cast<unsigned>(ceil_div(a.M, kThreads / 32)),
                  static_cast<unsigned>(ceil_div(a.N, tile)));
        kernel<<<grid, kThreads, 0, s>>>(a.M, a.K, a.N, a.nnz, a.rowptr, a.colind,
                                         static_cast<const float *>(a.val),
                                         static_cast<const float *>(a.B), a.ldb, a.C, a.ldc,
                                         a.status, thresh, list, counters);
    };
    if (vec && a.N <= 128)
        go(spmm_reduce<OP, W, 1, 4>, 128);
    else if (vec)
        go(spmm_reduce<OP, W, 2, 4>, 256);
    else
        go(spmm_reduce<OP, W, 4, 1>, 128);
}

}  // namespace

as_status spmm_reduce_launch(as_ctx *ctx, int op, const SpmmArgs &a, cudaStream_t s) {
    const bool w = a.val != nullptr;
    // the weighted sum is the SpMM's chain from zero (C = A * B): its library default runs the
    // width-matched row-split kernels and the long-row kernel
    if (op == 0 && w && a.beta == 0.0f && !a.C16 && a.K > 0)
        return spmm_launch(ctx, 0,
                           spmm_default_variant(0, a.M, a.K, a.N, a.nnz, a.ldb, a.ldc, a.B, a.C),
                           a, s);
    if (ceil_div(a.N, 128) > 65535) return fail(AS_ERR_UNSUPPORTED, "spmm reduce: N too large");
    // rows longer than kLongRow entries go to the long-row kernel when its copies can serve
    // the layout
    int thresh = INT_MAX;
    int *list = nullptr;
    const int granule = a.nnz > kLongRow && a.M > 0 ? spmm_long_granule(0, a.N, a.ldb, a.B) : 0;
    if (granule) {
        void *p = nullptr;
        as_status st = scratch(ctx, static_cast<size_t>(a.M) * sizeof(int), &p);
        if (st != AS_OK) return st;
        thresh = kLongRow;
        list = static_cast<int *>(p);
    }
    const bool vec = a.N % 4 == 0 && a.ldb % 4 == 0 && a.ldc % 4 == 0 &&
                     reinterpret_cast<uintptr_t>(a.B) % 16 == 0 &&
                     reinterpret_cast<uintptr_t>(a.C) % 16 == 0;
    unsigned *cnt = ctx->d_long;
    if (op == 0) w ? launch<0, true>(a, vec, thresh, list, cnt, s) : launch<0, false>(a, vec, thresh, list, cnt, s);
    else if (op == 1) w ? launch<1, true>(a, vec, thresh, list, cnt, s) : launch<1, false>(a, vec, thresh, list, cnt, s);
    else w ? launch<2, true>(a, vec, thresh, list, cnt, s) : launch<2, false>(a, vec, thresh, list, cnt, s);
    ctx->launches++;
    as_status st = check_cuda(cudaGetLastError(), "spmm reduce launch");
    if (st != AS_OK || !granule) return st;
    // the long rows' chain step: the weighted sum is the SpMM's fused multiply-add
    const int step = op == 0 ? (w ? 0 : 1) : op == 1 ? 2 : 3;
    st = spmm_long_launch(ctx, 0, granule, a, list, s, step);
    if (st != AS_OK) cudaMemsetAsync(ctx->d_long, 0, 3 * sizeof(unsigned), s);
    return st;
}

}  // namespace as
