// Format builders on the GPU (sm_103a): dense -> CSR (the reference's toCSR, SDMM.cpp:355-370)
// and CSR -> the 1x4-blocked "vector-aware" CSR (toVectorAwareCSR, SpMV.cpp:15-38). Both are
// two passes -- count per row, then fill -- with one warp per row, so the caller can size the
// outputs from row_ptr[M] between the passes. Output order is the reference's: row-major scan,
// ascending columns; a value is stored when value != 0 (so -0.0 is dropped and NaN kept, as
// in C). Deterministic: positions come from per-row prefix counts (ballot + popc), no atomics.
#include "common.cuh"
#include "internal.h"

namespace as {
namespace {

constexpr int kThreads = 256;

// counts[r] = nonzeros of dense row r
__global__ void __launch_bounds__(kThreads)
dense_count(int M, int K, const float *__restrict__ D, long ld, int *__restrict__ counts) {
    const long w = (static_cast<long>(blockIdx.x) * kThreads + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= M) return;
    const float *row = D + w * ld;
    int c = 0;
    for (int k = lane; k < K; k += 32) c += __ldg(row + k) != 0.0f;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if (lane == 0) counts[w] = c;
}

__global__ void __launch_bounds__(kThreads)
dense_fill(int M, int K, const float *__restrict__ D, long ld, const int *__restrict__ rowptr,
           int *__restrict__ colind, float *__restrict__ val) {
    const long w = (static_cast<long>(blockIdx.x) * kThreads + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= M) return;
    const float *row = D + w * ld;
    int pos = rowptr[w];
    for (int k0 = 0; k0 < K; k0 += 32) {
        const int k = k0 + lane;
        const float x = k < K ? __ldg(row + k) : 0.0f;
        const bool nz = x != 0.0f;
        const unsigned m = __ballot_sync(0xffffffffu, nz);
        if (nz) {
            const int p = pos + __popc(m & ((1u << lane) - 1u));
            colind[p] = k;
            val[p] = x;
        }
        pos += __popc(m);
    }
}

// counts[r] = 4 * (number of distinct aligned 4-column groups in row r)
__global__ void __launch_bounds__(kThreads)
vcsr4_count(int M, int nnz, const int *__restrict__ rowptr, const int *__restrict__ colind,
            int *__restrict__ counts, unsigned *status) {
    const long w = (static_cast<long>(blockIdx.x) * kThreads + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= M) return;
    int lo, hi;
    row_range(rowptr, static_cast<int>(w), nnz, status, lo, hi);
    int c = 0;
    for (int e = lo + lane; e < hi; e += 32) {
        const int g = __ldg(colind + e) >> 2;
        c += (e == lo) || (__ldg(colind + e - 1) >> 2) != g;  // a new group starts here
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
    if (lane == 0) counts[w] = 4 * c;
}

__global__ void __launch_bounds__(kThreads)
vcsr4_fill(int M, int nnz, const int *__restrict__ rowptr, const int *__restrict__ colind,
           const float *__restrict__ val, const int *__restrict__ vrowptr,
           int *__restrict__ vcolind, float *__restrict__ vval, unsigned *status) {
    const long w = (static_cast<long>(blockIdx.x) * kThreads + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= M) return;
    int lo, hi;
    row_range(rowptr, static_cast<int>(w), nnz, status, lo, hi);
    const int base = vrowptr[w];
    int started = 0;  // groups started in earlier batches of this row
    for (int e0 = lo; e0 < hi; e0 += 32) {
        const int e = e0 + lane;
        const bool valid = e < hi;
        const int col = valid ? __ldg(colind + e) : 0;
        const int g = col >> 2;
        const bool start = valid && ((e == lo) || (__ldg(colind + e - 1) >> 2) != g);
        const unsigned m = __ballot_sync(0xffffffffu, start);
        const int bidx = started + __popc(m & ((2u << lane) - 1u)) - 1;  // this entry's block
        if (start) {
#pragma unroll
            for (int l = 0; l < 4; ++l) {
                vcolind[base + 4 * bidx + l] = 4 * g + l;
                vval[base + 4 * bidx + l] = 0.0f;
            }
        }
        __syncwarp();
        if (valid) vval[base + 4 * bidx + (col & 3)] = __ldg(val + e);
        __syncwarp();
        started += __popc(m);
    }
}

// ---- CSR -> row-pair reuse layout (suitesparse_sdmm.cpp toDataReuseFormat, :150-179) ------
// Rows are paired (2p, 2p+1). Entry i of row a = 2p and entry f of row b = 2p+1 are matched when
// they hold the same column c, f is the first entry of row b with column c, and each is what a
// binary search for c finds in the other row. The predicate is evaluated the same way from both
// sides, so the two passes agree on every count even for rows that are not sorted (then the
// layout is memory-safe but not the reference's; sorted rows give exactly its layout): row a's
// segment lists its entries in order, each matched one followed by its partner from row b
// (flag 1); row b's segment keeps its unmatched entries in order. An unpaired last row is
// copied. Total entries are unchanged.
__device__ __forceinline__ int bsearch_col(const int *__restrict__ colind, int lo, int hi, int c) {
    // an index in [lo, hi) holding c, or -1
    while (lo < hi) {
        const int mid = (lo + hi) >> 1;
        const int v = __ldg(colind + mid);
        if (v == c) return mid;
        if (v < c)
            lo = mid + 1;
        else
            hi = mid;
    }
    return -1;
}

// partner in row b of entry i of row a (-1 if none)
__device__ __forceinline__ int pair_of_a(const int *__restrict__ colind, int a0, int a1, int b0,
                                         int b1, int i) {
    const int c = __ldg(colind + i);
    const int f = bsearch_col(colind, b0, b1, c);
    if (f < 0) return -1;
    if (f > b0 && __ldg(colind + f - 1) == c) return -1;  // f is not the first of its column
    return bsearch_col(colind, a0, a1, c) == i ? f : -1;
}

// whether entry f of row b moves into row a's segment
__device__ __forceinline__ bool moved_b(const int *__restrict__ colind, int a0, int a1, int b0,
                                        int b1, int f) {
    const int c = __ldg(colind + f);
    if (f > b0 && __ldg(colind + f - 1) == c) return false;
    const int i = bsearch_col(colind, a0, a1, c);
    return i >= 0 && bsearch_col(colind, b0, b1, c) == f;
}

// counts[2p] = len(a) + matched, counts[2p+1] = len(b) - matched; one warp per pair
__global__ void __launch_bounds__(kThreads)
rowpair_count(int M, int nnz, const int *__restrict__ rowptr, const int *__restrict__ colind,
              int *__restrict__ counts, unsigned *status) {
    const long w = (static_cast<long>(blockIdx.x) * kThreads + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const long ra = 2 * w;
    if (ra >= M) return;
    int a0, a1;
    row_range(rowptr, static_cast<int>(ra), nnz, status, a0, a1);
    if (ra + 1 >= M) {
        if (lane == 0) counts[ra] = a1 - a0;
        return;
    }
    int b0, b1;
    row_range(rowptr, static_cast<int>(ra + 1), nnz, status, b0, b1);
    int m = 0;
    for (int f = b0 + lane; f < b1; f += 32) m += moved_b(colind, a0, a1, b0, b1, f);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m += __shfl_xor_sync(0xffffffffu, m, o);
    if (lane == 0) {
        counts[ra] = (a1 - a0) + m;
        counts[ra + 1] = (b1 - b0) - m;
    }
}

__global__ void __launch_bounds__(kThreads)
rowpair_fill(int M, int nnz, const int *__restrict__ rowptr, const int *__restrict__ colind,
             const float *__restrict__ val, const int *__restrict__ rowptr2,
             int *__restrict__ colind2, float *__restrict__ val2, uint8_t *__restrict__ flag2,
             unsigned *status) {
    const long w = (static_cast<long>(blockIdx.x) * kThreads + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const long ra = 2 * w;
    if (ra >= M) return;
    int a0, a1, b0 = 0, b1 = 0;
    row_range(rowptr, static_cast<int>(ra), nnz, status, a0, a1);
    const bool paired = ra + 1 < M;
    if (paired) row_range(rowptr, static_cast<int>(ra + 1), nnz, status, b0, b1);
    // row a's segment: each entry, then its partner
    int pos = __ldg(rowptr2 + ra);
    const int end_a = __ldg(rowptr2 + ra + 1);
    for (int i0 = a0; i0 < a1; i0 += 32) {
        const int i = i0 + lane;
        const bool valid = i < a1;
        const int f = valid && paired ? pair_of_a(colind, a0, a1, b0, b1, i) : -1;
        const unsigned mv = __ballot_sync(0xffffffffu, valid);
        const unsigned mp = __ballot_sync(0xffffffffu, f >= 0);
        const unsigned below = (1u << lane) - 1u;
        if (valid) {
            const int p = pos + __popc(mv & below) + __popc(mp & below);
            if (p < end_a) {
                colind2[p] = __ldg(colind + i);
                val2[p] = __ldg(val + i);
                flag2[p] = 0;
            }
            if (f >= 0 && p + 1 < end_a) {
                colind2[p + 1] = __ldg(colind + f);
                val2[p + 1] = __ldg(val + f);
                flag2[p + 1] = 1;
            }
        }
        pos += __popc(mv) + __popc(mp);
    }
    if (!paired) return;
    // row b's segment: its unmatched entries
    pos = __ldg(rowptr2 + ra + 1);
    const int end_b = __ldg(rowptr2 + ra + 2);
    for (int f0 = b0; f0 < b1; f0 += 32) {
        const int f = f0 + lane;
        const bool keep = f < b1 && !moved_b(colind, a0, a1, b0, b1, f);
        const unsigned mk = __ballot_sync(0xffffffffu, keep);
        if (keep) {
            const int p = pos + __popc(mk & ((1u << lane) - 1u));
            if (p < end_b) {
                colind2[p] = __ldg(colind + f);
                val2[p] = __ldg(val + f);
                flag2[p] = 0;
            }
        }
        pos += __popc(mk);
    }
}

}  // namespace

// counts in arr[0..M-1] -> row pointer arr[0..M] (exclusive scan, arr[M] = total)
static as_status formats_scan(as_ctx *ctx, int M, int *arr, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(arr + M, 0, sizeof(int), s);
    if (e != cudaSuccess) return check_cuda(e, "format scan");
    return exclusive_scan_i32(ctx, arr, arr, static_cast<long>(M) + 1, s);
}



as_status dense_to_csr_count_launch(as_ctx *ctx, int M, int K, const float *D, long ld,
                                    int *rowptr, cudaStream_t s) {
    dense_count<<<static_cast<unsigned>(ceil_div(static_cast<long>(M) * 32, kThreads)), kThreads, 0, s>>>(
        M, K, D, ld, rowptr);
    ctx->launches++;
    as_status st = check_cuda(cudaGetLastError(), "dense_to_csr count");
    if (st != AS_OK) return st;
    return formats_scan(ctx, M, rowptr, s);
}

as_status dense_to_csr_fill_launch(as_ctx *ctx, int M, int K, const float *D, long ld,
                                   const int *rowptr, int *colind, float *val, cudaStream_t s) {
    dense_fill<<<static_cast<unsigned>(ceil_div(static_cast<long>(M) * 32, kThreads)), kThreads, 0, s>>>(
        M, K, D, ld, rowptr, colind, val);
    ctx->launches++;
    return check_cuda(cudaGetLastError(), "dense_to_csr fill");
}

as_status csr_to_vcsr4_count_launch(as_ctx *ctx, int M, int nnz, const int *rowptr,
                                    const int *colind, int *vrowptr, cudaStream_t s) {
    vcsr4_count<<<static_cast<unsigned>(ceil_div(static_cast<long>(M) * 32, kThreads)), kThreads, 0, s>>>(
        M, nnz, rowptr, colind, vrowptr, ctx->d_status);
    ctx->launches++;
    as_status st = check_cuda(cudaGetLastError(), "csr_to_vcsr4 count");
    if (st != AS_OK) return st;
    return formats_scan(ctx, M, vrowptr, s);
}

as_status csr_to_vcsr4_fill_launch(as_ctx *ctx, int M, int nnz, const int *rowptr,
                                   const int *colind, const float *val, const int *vrowptr,
                                   int *vcolind, float *vval, cudaStream_t s) {
    vcsr4_fill<<<static_cast<unsigned>(ceil_div(static_cast<long>(M) * 32, kThreads)), kThreads, 0, s>>>(
        M, nnz, rowptr, colind, val, vrowptr, vcolind, vval, ctx->d_status);
    ctx->launches++;
    return check_cuda(cudaGetLastError(), "csr_to_vcsr4 fill");
}

}  // namespace as

namespace as {

as_status csr_to_rowpair_count_launch(as_ctx *ctx, int M, int nnz, const int *rowptr,
                                      const int *colind, int *rowptr2, cudaStream_t s) {
    const long pairs = (static_cast<long>(M) + 1) / 2;
    rowpair_count<<<static_cast<unsigned>(ceil_div(pairs * 32, kThreads)), kThreads, 0, s>>>(
        M, nnz, rowptr, colind, rowptr2, ctx->d_status);
    ctx->launches++;
    as_status st = check_cuda(cudaGetLastError(), "csr_to_rowpair count");
    if (st != AS_OK) return st;
    return formats_scan(ctx, M, rowptr2, s);
}

as_status csr_to_rowpair_fill_launch(as_ctx *ctx, int M, int nnz, const int *rowptr,
                                     const int *colind, const float *val, const int *rowptr2,
                                     int *colind2, float *val2, uint8_t *flag2, cudaStream_t s) {
    const long pairs = (static_cast<long>(M) + 1) / 2;
    rowpair_fill<<<static_cast<unsigned>(ceil_div(pairs * 32, kThreads)), kThreads, 0, s>>>(
        M, nnz, rowptr, colind, val, rowptr2, colind2, val2, flag2, ctx->d_status);
    ctx->launches++;
    return check_cuda(cudaGetLastError(), "csr_to_rowpair fill");
}

}  // namespace as
