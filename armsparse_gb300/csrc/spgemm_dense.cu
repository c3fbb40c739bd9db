// Sparse x sparse -> dense (sm_103a): C = beta*C + A*B with A (M x K) and B (K x N) in CSR and
// C dense row-major, bit-identical to the reference's sparse_matrix_mul3 (SpMM.cpp:309-327,
// built with FMA contraction): every output element is one fused-FMA chain over the entries
// of A's row in CSR order, each entry k contributing B[k, j] when B's row k holds column j.
//
// One warp per (row of A, tile of kTile output columns). The tile's accumulators live in
// shared memory, start as beta*C, and take A's entries in order: for each, the lanes walk B's
// row k (one B entry per lane) and update acc[j] = fmaf(a, b, acc[j]) for the j in the tile.
// The columns of one B row are distinct, so no two lanes touch one accumulator in a step, and
// __syncwarp orders the steps. The (row start, row end) of B for 32 entries of A come with one
// load per lane, and the first 32 entries of four consecutive B rows are loaded before any of
// them is applied.
#include "common.cuh"
#include "internal.h"

namespace as {
namespace {

constexpr int kThreads = 256;
constexpr int kWarps = kThreads / 32;
constexpr int kTile = 1024;  // output columns per warp (4 KB of accumulators)
constexpr int kBatch = 4;    // A entries whose B rows are loaded together

__global__ void __launch_bounds__(kThreads)
spgemm_dense(int M, int K, int N, int nnz_a, int nnz_b, const int *__restrict__ rp1,
             const int *__restrict__ ci1, const float *__restrict__ v1,
             const int *__restrict__ rp2, const int *__restrict__ ci2,
             const float *__restrict__ v2, float *__restrict__ C, long ldc, float beta,
             unsigned *status) {
    __shared__ float acc_s[kWarps][kTile];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long row = static_cast<long>(blockIdx.x) * kWarps + warp;
    if (row >= M) return;  // warps are independent: no CTA-wide barrier below
    const int tile0 = blockIdx.y * kTile;
    const int tw = min(kTile, N - tile0);
    float *acc = acc_s[warp];
    float *crow = C + row * ldc + tile0;
    for (int j = lane; j < tw; j += 32) acc[j] = beta != 0.0f ? crow[j] * beta : 0.0f;
    __syncwarp();

    int lo, hi;
    row_range(rp1, static_cast<int>(row), nnz_a, status, lo, hi);
    for (int base = lo; base < hi; base += 32) {
        // this lane's A entry: its value and the extent of B's row
        const int e = base + lane;
        float a = 0.0f;
        int bs = 0, be = 0;
        if (e < hi) {
            const int k = ld_stream(ci1 + e);
            a = ld_stream(v1 + e);
            if (static_cast<unsigned>(k) >= static_cast<unsigned>(K)) {
                flag(status, kFlagBadColind);
            } else {
                bs = __ldg(rp2 + k);
                be = __ldg(rp2 + k + 1);
                if (bs < 0 || be < bs || be > nnz_b) {
                    flag(status, kFlagBadRowptr);
                    bs = be = 0;
                }
            }
        }
        const int cnt = min(32, hi - base);
        for (int u0 = 0; u0 < cnt; u0 += kBatch) {
            float au[kBatch], bv[kBatch];
            int su[kBatch], eu[kBatch], jv[kBatch];
#pragma unroll
            for (int q = 0; q < kBatch; ++q) {  // first 32 B entries of each row, loads first
                const int u = u0 + q < cnt ? u0 + q : cnt - 1;
                au[q] = __shfl_sync(0xffffffffu, a, u);
                su[q] = __shfl_sync(0xffffffffu, bs, u);
                eu[q] = __shfl_sync(0xffffffffu, be, u);
                if (u0 + q >= cnt) eu[q] = su[q];  // past the batch: nothing to apply
                const int t = su[q] + lane;
                jv[q] = -1;
                bv[q] = 0.0f;
                if (t < eu[q]) {
                    jv[q] = __ldg(ci2 + t);
                    bv[q] = __ldg(v2 + t);
                }
            }
#pragma unroll
            for (int q = 0; q < kBatch; ++q) {
                int j = jv[q];
                float b = bv[q];
                for (int t0 = su[q];; t0 += 32) {
                    if (t0 + lane < eu[q]) {
                        if (static_cast<unsigned>(j) >= static_cast<unsigned>(N))
                            flag(status, kFlagBadColind);
                        else if (j >= tile0 && j < tile0 + tw)
                            acc[j - tile0] = fmaf(au[q], b, acc[j - tile0]);
                    }
                    __syncwarp();
                    if (t0 + 32 >= eu[q]) break;
                    const int t = t0 + 32 + lane;  // B rows longer than 32: the next 32
                    j = -1;
                    b = 0.0f;
                    if (t < eu[q]) {
                        j = __ldg(ci2 + t);
                        b = __ldg(v2 + t);
                    }
                }
            }
        }
    }
    __syncwarp();
    for (int j = lane; j < tw; j += 32) crow[j] = acc[j];
}

}  // namespace

as_status spgemm_dense_launch(as_ctx *ctx, int M, int K, int N, int nnz_a, const int *rp1,
                              const int *ci1, const float *v1, int nnz_b, const int *rp2,
                              const int *ci2, const float *v2, float *C, long ldc, float beta,
                              cudaStream_t s) {
    const long tiles = ceil_div(N, kTile);
    if (tiles > 65535) return fail(AS_ERR_UNSUPPORTED, "spgemm_dense: N too large");
    dim3 grid(static_cast<unsigned>(ceil_div(M, kWarps)), static_cast<unsigned>(tiles));
    spgemm_dense<<<grid, kThreads, 0, s>>>(M, K, N, nnz_a, nnz_b, rp1, ci1, v1, rp2, ci2, v2, C,
                                           ldc, beta, ctx->d_status);
    ctx->launches++;
    return check_cuda(cudaGetLastError(), "spgemm_dense launch");
}

}  // namespace as
