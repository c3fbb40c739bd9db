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
// gathers see as one run of 4 * ldb elements.
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
           unsigned *status) {
    using V = Vec<float, VB>;
    constexpr int E = V::E;
    constexpr int TILE = 32 * E * CPL;
    const int lane = threadIdx.x & 31;
    const long row = static_cast<long>(blockIdx.x) * (kThreads / 32) + (threadIdx.x >> 5);
    if (row >= M) return;
    int lo, hi;
    row_range(vrowptr, static_cast<int>(row), nslots, status, lo, hi);
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

template <int VB, int CPL>
void launch(int M, int K, int N, int nslots, const int *vrowptr, const int *vcolind,
            const float *vval, const float *B, long ldb, float *C, long ldc, float beta,
            unsigned *status, cudaStream_t s) {
    constexpr int TILE = 32 * Vec<float, VB>::E * CPL;
    dim3 grid(static_cast<unsigned>(ceil_div(M, kThreads / 32)),
              static_cast<unsigned>(ceil_div(N, TILE)));
    spmm_vcsr4<VB, CPL><<<grid, kThreads, 0, s>>>(M, K, N, nslots, vrowptr, vcolind, vval, B, ldb,
                                                   C, ldc, beta, status);
}

}  // namespace

as_status spmm_vcsr4_launch(as_ctx *ctx, int M, int K, int N, int nslots, const int *vrowptr,
                            const int *vcolind, const float *vval, const float *B, long ldb,
                            float *C, long ldc, float beta, cudaStream_t s) {
    const uintptr_t pb = reinterpret_cast<uintptr_t>(B), pc = reinterpret_cast<uintptr_t>(C);
    if (N >= 256 && N % 4 == 0 && ldb % 4 == 0 && ldc % 4 == 0 && pb % 16 == 0 && pc % 16 == 0) {
        if (ceil_div(N, 256) > 65535) return fail(AS_ERR_UNSUPPORTED, "spmm vcsr4: N too large");
        launch<16, 2>(M, K, N, nslots, vrowptr, vcolind, vval, B, ldb, C, ldc, beta, ctx->d_status, s);
    } else if (N % 2 == 0 && ldb % 2 == 0 && ldc % 2 == 0 && pb % 8 == 0 && pc % 8 == 0) {
        if (ceil_div(N, 64) > 65535) return fail(AS_ERR_UNSUPPORTED, "spmm vcsr4: N too large");
        launch<8, 1>(M, K, N, nslots, vrowptr, vcolind, vval, B, ldb, C, ldc, beta, ctx->d_status, s);
    } else {
        if (ceil_div(N, 32) > 65535) return fail(AS_ERR_UNSUPPORTED, "spmm vcsr4: N too large");
        launch<4, 1>(M, K, N, nslots, vrowptr, vcolind, vval, B, ldb, C, ldc, beta, ctx->d_status, s);
    }
    ctx->launches++;
    return check_cuda(cudaGetLastError(), "spmm vcsr4 launch");
}

}  // namespace as
