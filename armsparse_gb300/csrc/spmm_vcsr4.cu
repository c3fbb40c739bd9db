// SpMM over the reference's 1x4-blocked "vector-aware" CSR (sm_103a): C = A*B + beta*C with A
// in the layout toVectorAwareCSR writes (SpMV.cpp:15-38; as_csr_to_vcsr4_* build it): per row,
// blocks of four slots for the aligned 4-column groups that hold an entry, slot l of a block
// having column 4g + l and the entry's value, or 0 where the group has no entry in that column.
// It is the SpMM counterpart of sparse_dense_vector (SpMV.cpp:155-179).
//
// One warp per row and column tile; lane g holds CPL vectors of E columns. Slot values of 0 are
// skipped (the layout cannot tell a stored zero from an empty slot), so every output is one
// fused chain over the row's nonzero entries in column order: bit for bit the CSR SpMM of the
// same matrix without stored zeros. The four rows of a block are adjacent in B, which the
// gathers see as one run of 4 * ldb elements. Rows with more than kLongRow slots are left to
// the long-row kernel (spmm_long.cu, its zero-skipping step), as in the row-split SpMM.
#include <limits.h>

#include "common.cuh"
#include "internal.h"
#include "spmm_vec.cuh"

namespace as {
namespace {

constexpr int kThreads = 256;

template <int VB, int CPL>
__global__ void __launch_bounds__(kThreads)
spmm_vcsr4(int M, int K, int N, int nslots, const int *__restrict__ vrowptr,
           const int *__restrict__ vcolind, const float *__restrict__ vval,
           const float *__restrict__ B, long ldb, float *__restrict__ C, long ldc, float beta,
           unsigned *status, int long_thresh, int *long_list, unsigned *long_count) {
    // let the long-row kernel (a programmatic dependent) be scheduled early; it waits for this
    // grid to complete before it reads the list
    asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory");
    using V = Vec<float, VB>;
    constexpr int E = V::E;
    constexpr int TILE = 32 * E * CPL;
    const int lane = threadIdx.x & 31;
    const long row = static_cast<long>(blockIdx.x) * (kThreads / 32) + (threadIdx.x >> 5);
    if (row >= M) return;
    int lo, hi;
    row_range(vrowptr, static_cast<int>(row), nslots, status, lo, hi);
    if (hi - lo > long_thresh) {  // left to the long-row kernel
        if (blockIdx.y == 0 && lane == 0) list_long_row(row, hi - lo, M, long_list, long_count, status);
        return;
    }
    const int tile0 = blockIdx.y * TILE;
    float acc[CPL][E];
#pragma unroll
    for (int j = 0; j < CPL; ++j) {
        const int c = tile0 + (j * 32 + lane) * E;
#pragma unroll
        for (int i = 0; i < E; ++i)
            acc[j][i] = (beta != 0.0f && c < N) ? C[row * ldc + c + i] * beta : 0.0f;
    }
    for (int base = lo; base < hi; base += 32) {
        const int e = base + lane;
        int k = -1;
        float v = 0.0f;
        if (e < hi) {
            k = ld_stream(vcolind + e);
            v = ld_stream(vval + e);
            if (static_cast<unsigned>(k) >= static_cast<unsigned>(K)) {
                if (v != 0.0f) flag(status, kFlagBadColind);  // an empty slot may point past K
                k = -1;
            }
        }
        const int cnt = min(32, hi - base);
        for (int t = 0; t < cnt; ++t) {
            const int kk = __shfl_sync(0xffffffffu, k, t);
            const float vv = __shfl_sync(0xffffffffu, v, t);
            if (kk < 0 || vv == 0.0f) continue;  // an empty slot (or a malformed one)
            const float *brow = B + static_cast<long>(kk) * ldb;
#pragma unroll
            for (int j = 0; j < CPL; ++j) {
                const int c = tile0 + (j * 32 + lane) * E;
                if (c < N) {
                    float b[E];
                    V::load(brow + c, b);
                    fma_vec_f32<E>(b, vv, acc[j]);
                }
            }
        }
    }
#pragma unroll
    for (int j = 0; j < CPL; ++j) {
        const int c = tile0 + (j * 32 + lane) * E;
        if (c < N) {
#pragma unroll
            for (int i = 0; i < E; ++i) C[row * ldc + c + i] = acc[j][i];
        }
    }
}

struct LongList {
    int thresh;
    int *list;
    unsigned *counters;
};

template <int VB, int CPL>
void launch(int M, int K, int N, int nslots, const int *vrowptr, const int *vcolind,
            const float *vval, const float *B, long ldb, float *C, long ldc, float beta,
            unsigned *status, const LongList &lr, cudaStream_t s) {
    constexpr int TILE = 32 * Vec<float, VB>::E * CPL;
    dim3 grid(static_cast<unsigned>(ceil_div(M, kThreads / 32)),
              static_cast<unsigned>(ceil_div(N, TILE)));
    spmm_vcsr4<VB, CPL><<<grid, kThreads, 0, s>>>(M, K, N, nslots, vrowptr, vcolind, vval, B, ldb,
                                                   C, ldc, beta, status, lr.thresh, lr.list,
                                                   lr.counters);
}

}  // namespace

as_status spmm_vcsr4_launch(as_ctx *ctx, int M, int K, int N, int nslots, const int *vrowptr,
                            const int *vcolind, const float *vval, const float *B, long ldb,
                            float *C, long ldc, float beta, cudaStream_t s) {
    const uintptr_t pb = reinterpret_cast<uintptr_t>(B), pc = reinterpret_cast<uintptr_t>(C);
    const bool wide = N >= 256 && N % 4 == 0 && ldb % 4 == 0 && ldc % 4 == 0 && pb % 16 == 0 && pc % 16 == 0;
    const bool pairs = N % 2 == 0 && ldb % 2 == 0 && ldc % 2 == 0 && pb % 8 == 0 && pc % 8 == 0;
    if (ceil_div(N, wide ? 256 : pairs ? 64 : 32) > 65535)
        return fail(AS_ERR_UNSUPPORTED, "spmm vcsr4: N too large");
    // rows longer than kLongRow slots go to the long-row kernel when its copies can serve the
    // layout
    LongList lr{INT_MAX, nullptr, ctx->d_long};
    const int granule = nslots > kLongRow && M > 0 ? spmm_long_granule(0, N, ldb, B) : 0;
    if (granule) {
        void *p = nullptr;
        as_status st = scratch(ctx, static_cast<size_t>(M) * sizeof(int), &p);
        if (st != AS_OK) return st;
        lr.thresh = kLongRow;
        lr.list = static_cast<int *>(p);
    }
    if (wide)
        launch<16, 2>(M, K, N, nslots, vrowptr, vcolind, vval, B, ldb, C, ldc, beta, ctx->d_status, lr, s);
    else if (pairs)
        launch<8, 1>(M, K, N, nslots, vrowptr, vcolind, vval, B, ldb, C, ldc, beta, ctx->d_status, lr, s);
    else
        launch<4, 1>(M, K, N, nslots, vrowptr, vcolind, vval, B, ldb, C, ldc, beta, ctx->d_status, lr, s);
    ctx->launches++;
    as_status st = check_cuda(cudaGetLastError(), "spmm vcsr4 launch");
    if (st != AS_OK || !granule) return st;
    SpmmArgs a{M, K, N, nslots, vrowptr, vcolind, vval, B, ldb, C, ldc, beta, ctx->d_status};
    st = spmm_long_launch(ctx, 0, granule, a, lr.list, s, 4);
    if (st != AS_OK) cudaMemsetAsync(ctx->d_long, 0, 3 * sizeof(unsigned), s);
    return st;
}

}  // namespace as
