// SpMM over the row-pair reuse layout (sm_103a), bit-identical to the reference's
// DataReuseSpmm (suitesparse_sdmm.cpp:25-44) with its saxpy fused per element.
//
// Layout (toDataReuseFormat, suitesparse_sdmm.cpp:150-179; as_csr_to_rowpair_* build it):
// rows are paired (2p, 2p+1); row 2p's segment holds its entries in column order, each
// followed by row 2p+1's entry in the same column when there is one (flag 1); row 2p+1's
// segment holds its other entries. The reference computes C[m + flag] += val * B[col] per
// entry, a pair's two rows in order on one thread, so:
//   - row 2p: one fused chain over its own entries (its CSR order);
//   - row 2p+1: one fused chain over the entries flagged in row 2p's segment, then over its
//     own segment.
// One warp per pair keeps both chains in registers (acc0, acc1). A flagged entry has the same
// column as the entry before it, so it reuses the B segment already in registers instead of
// gathering it again: the data reuse the layout exists for. Lane g holds CPL vectors of E
// consecutive columns of a 32*E*CPL-column tile (grid.y over tiles); (colind, val, flag) come
// in coalesced batches of 32 and are broadcast by shuffles.
//
// A flag is honoured only in the segment of an even row that has a partner; anywhere else it
// is ignored (the entry counts for its own row), and a flagged first entry of a segment reuses
// a zero segment. A column index out of range is flagged and its entry skipped.
//
// Pairs with more than kLongRow entries are left to the long-row kernel (spmm_long.cu, its
// row-pair step): a unit per row of the pair runs the same chain over the entries it includes,
// each with its own column's B segment (identical to the reused one in a well-formed layout).
#include <limits.h>

#include "common.cuh"
#include "internal.h"
#include "spmm_vec.cuh"

namespace as {
namespace {

constexpr int kThreads = 256;

template <int VB, int CPL>
__global__ void __launch_bounds__(kThreads)
spmm_rowpair(int M, int K, int N, int nnz, const int *__restrict__ rowptr2,
             const int *__restrict__ colind2, const float *__restrict__ val2,
             const uint8_t *__restrict__ flag2, const float *__restrict__ B, long ldb,
             float *__restrict__ C, long ldc, float beta, unsigned *status, int long_thresh,
             int *long_list, unsigned *long_count) {
    // let the long-row kernel (a programmatic dependent) be scheduled early; it waits for this
    // grid to complete before it reads the list
    asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory");
    using V = Vec<float, VB>;
    constexpr int E = V::E;
    constexpr int TILE = 32 * E * CPL;
    const int lane = threadIdx.x & 31;
    const long pair = static_cast<long>(blockIdx.x) * (kThreads / 32) + (threadIdx.x >> 5);
    const long ra = 2 * pair;
    if (ra >= M) return;
    const bool paired = ra + 1 < M;
    {   // a long pair is left to the long-row kernel
        int plo, phi, qlo, qhi;
        row_range(rowptr2, static_cast<int>(ra), nnz, status, plo, phi);
        qlo = qhi = 0;
        if (paired) row_range(rowptr2, static_cast<int>(ra + 1), nnz, status, qlo, qhi);
        const int len = (phi - plo) + (qhi - qlo);
        if (len > long_thresh) {
            if (blockIdx.y == 0 && lane == 0) list_long_row(ra, len, M, long_list, long_count, status);
            return;
        }
    }
    const int tile0 = blockIdx.y * TILE;

    float acc0[CPL][E], acc1[CPL][E], b[CPL][E];
#pragma unroll
    for (int j = 0; j < CPL; ++j) {
        const int c = tile0 + (j * 32 + lane) * E;
#pragma unroll
        for (int i = 0; i < E; ++i) {
            acc0[j][i] = 0.0f;
            acc1[j][i] = 0.0f;
            b[j][i] = 0.0f;
        }
        if (beta != 0.0f && c < N) {
#pragma unroll
            for (int i = 0; i < E; ++i) {
                acc0[j][i] = C[ra * ldc + c + i] * beta;
                if (paired) acc1[j][i] = C[(ra + 1) * ldc + c + i] * beta;
            }
        }
    }

    // walk the segments of row a (flags honoured) and then row b (flags ignored)
    for (int seg = 0; seg < (paired ? 2 : 1); ++seg) {
        int lo, hi;
        row_range(rowptr2, static_cast<int>(ra + seg), nnz, status, lo, hi);
        const bool honour = seg == 0 && paired;
#pragma unroll
        for (int j = 0; j < CPL; ++j)
#pragma unroll
            for (int i = 0; i < E; ++i) b[j][i] = 0.0f;  // what a flagged first entry reuses
        for (int base = lo; base < hi; base += 32) {
            const int e = base + lane;
            int k = -1, f = 0;
            float v = 0.0f;
            if (e < hi) {
                k = ld_stream(colind2 + e);
                v = ld_stream(val2 + e);
                f = honour && __ldg(flag2 + e) != 0;
                if (static_cast<unsigned>(k) >= static_cast<unsigned>(K)) {
                    flag(status, kFlagBadColind);
                    k = -1;
                }
            }
            const int cnt = min(32, hi - base);
            for (int t = 0; t < cnt; ++t) {
                const int kk = __shfl_sync(0xffffffffu, k, t);
                const float vv = __shfl_sync(0xffffffffu, v, t);
                const int ff = __shfl_sync(0xffffffffu, f, t);
                if (kk < 0) continue;
                if (!ff) {  // a new column: gather its B segment
                    const float *brow = B + static_cast<long>(kk) * ldb;
#pragma unroll
                    for (int j = 0; j < CPL; ++j) {
                        const int c = tile0 + (j * 32 + lane) * E;
                        if (c < N) V::load(brow + c, b[j]);
                    }
                }
                if (ff || seg == 1) {
#pragma unroll
                    for (int j = 0; j < CPL; ++j) fma_vec_f32<E>(b[j], vv, acc1[j]);
                } else {
#pragma unroll
                    for (int j = 0; j < CPL; ++j) fma_vec_f32<E>(b[j], vv, acc0[j]);
                }
            }
        }
    }

#pragma unroll
    for (int j = 0; j < CPL; ++j) {
        const int c = tile0 + (j * 32 + lane) * E;
        if (c < N) {
#pragma unroll
            for (int i = 0; i < E; ++i) {
                C[ra * ldc + c + i] = acc0[j][i];
                if (paired) C[(ra + 1) * ldc + c + i] = acc1[j][i];
            }
        }
    }
}

template <int VB, int CPL>
void launch(const SpmmArgs &a, const uint8_t *flag2, int thresh, int *list, unsigned *counters,
            cudaStream_t s) {
    constexpr int TILE = 32 * Vec<float, VB>::E * CPL;
    const long pairs = (static_cast<long>(a.M) + 1) / 2;
    dim3 grid(static_cast<unsigned>(ceil_div(pairs, kThreads / 32)),
              static_cast<unsigned>(ceil_div(a.N, TILE)));
    spmm_rowpair<VB, CPL><<<grid, kThreads, 0, s>>>(
        a.M, a.K, a.N, a.nnz, a.rowptr, a.colind, static_cast<const float *>(a.val), flag2,
        static_cast<const float *>(a.B), a.ldb, a.C, a.ldc, a.beta, a.status, thresh, list,
        counters);
}

}  // namespace

as_status spmm_rowpair_launch(as_ctx *ctx, const SpmmArgs &a, const uint8_t *flag2,
                              cudaStream_t s) {
    const uintptr_t pb = reinterpret_cast<uintptr_t>(a.B), pc = reinterpret_cast<uintptr_t>(a.C);
    const bool wide = a.N >= 256 && a.N % 4 == 0 && a.ldb % 4 == 0 && a.ldc % 4 == 0 &&
                      pb % 16 == 0 && pc % 16 == 0;
    const bool pairs = a.N % 2 == 0 && a.ldb % 2 == 0 && a.ldc % 2 == 0 && pb % 8 == 0 && pc % 8 == 0;
    if (ceil_div(a.N, wide ? 256 : pairs ? 64 : 32) > 65535)
        return fail(AS_ERR_UNSUPPORTED, "spmm rowpair: N too large");
    // pairs longer than kLongRow entries go to the long-row kernel when its copies can serve
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
    // widest vectors the layout allows: float4 x 2 for wide B, float2, then scalars
    if (wide)
        launch<16, 2>(a, flag2, thresh, list, ctx->d_long, s);
    else if (pairs)
        launch<8, 1>(a, flag2, thresh, list, ctx->d_long, s);
    else
        launch<4, 1>(a, flag2, thresh, list, ctx->d_long, s);
    ctx->launches++;
    as_status st = check_cuda(cudaGetLastError(), "spmm rowpair launch");
    if (st != AS_OK || !granule) return st;
    st = spmm_long_launch(ctx, 0, granule, a, list, s, 5, flag2);
    if (st != AS_OK) cudaMemsetAsync(ctx->d_long, 0, 3 * sizeof(unsigned), s);
    return st;
}

}  // namespace as
