// Shared device helpers for the sm_103a sparse kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "armsparse_gpu.h"

namespace as {

// Bits of the device status word (the context's error flag). Kernels OR them in and keep
// going on a memory-safe path; the host maps them to as_status.
enum : unsigned {
    kFlagBadRowptr = 1u,
    kFlagBadColind = 2u,
    kFlagTimeout = 4u,
    kFlagLongList = 8u,  // the long-row list was not empty at the start of a call (internal)
    kFlagBadPerm = 16u,  // a permutation entry out of [0, nnz) (the write was skipped)
    kFlagBadLabel = 32u,  // a class label out of [0, C) (that row counts 0 in the loss)
};

__device__ __forceinline__ void flag(unsigned *status, unsigned bit) {
    if (status) atomicOr(status, bit);
}

// Read-only, no-allocate-in-L1 loads for streamed index/value arrays.
__device__ __forceinline__ int ld_stream(const int *p) { return __ldcs(p); }
__device__ __forceinline__ float ld_stream(const float *p) { return __ldcs(p); }
__device__ __forceinline__ uint16_t ld_stream(const uint16_t *p) {
    return __ldcs(reinterpret_cast<const unsigned short *>(p));
}

__device__ __forceinline__ float bf16_to_f32(uint16_t h) {
    return __uint_as_float(static_cast<unsigned>(h) << 16);
}

// Round to nearest even; NaN stays a quiet NaN.
__device__ __forceinline__ uint16_t f32_to_bf16(float f) {
    unsigned u = __float_as_uint(f);
    if ((u & 0x7fffffffu) > 0x7f800000u) return static_cast<uint16_t>((u >> 16) | 0x40u);
    u += 0x7fffu + ((u >> 16) & 1u);
    return static_cast<uint16_t>(u >> 16);
}

// A ReLU applied at an output store when `relu` is set (negative -> 0; -0 and NaN pass).
__device__ __forceinline__ float relu_if(float v, bool relu) { return relu && v < 0.0f ? 0.0f : v; }

// Rows with more than kLongRow entries are left by the row kernels to the long-row kernel
// (spmm_long.cu); rows with more than kHugeRow are listed from the end of its list, which it
// takes first.
constexpr int kLongRow = 256;
constexpr int kHugeRow = 16384;

// Lists row `row` (of `len` entries) for the long-row kernel: counters [0] rows listed from the
// front, [2] huge rows listed from the end of the M-entry list.
__device__ __forceinline__ void list_long_row(long row, int len, int M, int *long_list,
                                              unsigned *long_count, unsigned *status) {
    const bool huge = len > kHugeRow;
    const unsigned idx = atomicAdd(long_count + (huge ? 2 : 0), 1u);
    if (idx < static_cast<unsigned>(M))
        long_list[huge ? M - 1 - static_cast<int>(idx) : static_cast<int>(idx)] =
            static_cast<int>(row);
    else
        flag(status, kFlagLongList);
}

// Valid row range [lo, hi) of row r; rows with malformed pointers become empty and flag.
__device__ __forceinline__ void row_range(const int *rowptr, int r, int nnz, unsigned *status,
                                          int &lo, int &hi) {
    lo = __ldg(rowptr + r);
    hi = __ldg(rowptr + r + 1);
    if (lo < 0 || hi < lo || hi > nnz) {
        flag(status, kFlagBadRowptr);
        lo = hi = 0;
    }
}

__host__ __device__ __forceinline__ long long ceil_div(long long a, long long b) {
    return (a + b - 1) / b;
}

}  // namespace as
