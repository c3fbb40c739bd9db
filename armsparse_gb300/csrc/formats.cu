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
