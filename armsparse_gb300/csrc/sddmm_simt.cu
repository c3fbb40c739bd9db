// FP32 SDDMM on CUDA cores: out[e] = s_e * <X[row(e), :], Y[col(e), :]> (sm_103a).
//
// One lane per edge, edges in CSR order across the grid. A lane finds its row with one
// binary search over rowptr (the reference searches per edge as well, findRow in
// gcn/pytorch-custom/computeUtil.h:11-28), or reads it from the COO row array (the
// reference's sddmm_cuda_coo, sddmm.cu:427-457), and then streams both operand rows with 32-byte
// steps (two float4 loads per row per step when K and the leading dimensions are multiples
// of 8 floats, else scalar). Lanes of a warp mostly share the row, so the X loads
// broadcast; each lane's Y reads are full 32-byte sectors. Eight interleaved partial sums
// (k mod 8) are combined as ((p0+p4)+(p1+p5)) + ((p2+p6)+(p3+p7)), the same order the
// CPU baseline uses.
#include "common.cuh"
#include "internal.h"

namespace as {
namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ int find_row(const int *__restrict__ rowptr, int M, int e) {
    // largest r in [0, M) with rowptr[r] <= e
    int lo = 0, hi = M;  // invariant: rowptr[lo] <= e < rowptr[hi] for valid CSR
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(rowptr + mid) <= e)
            lo = mid;
        else
            hi = mid;
    }
    return lo;
}

// COO: rows come per entry from `rows` (any order); CSR: `rows` is the row pointer.
template <bool VEC, bool COO>
__global__ void __launch_bounds__(kThreads)
sddmm_f32_lane(int M, int N, int K, int nnz, const int *__restrict__ rows,
               const int *__restrict__ colind, const float *__restrict__ aval,
               const float *__restrict__ X, long ldx, const float *__restrict__ Y, long ldy,
               float *__restrict__ out, unsigned *status) {
    const long e = static_cast<long>(blockIdx.x) * kThreads + threadIdx.x;
    if (e >= nnz) return;
    const int c = ld_stream(colind + e);
    int r;
    if (COO) {
        r = ld_stream(rows + e);
        if (static_cast<unsigned>(r) >= static_cast<unsigned>(M)) {
            flag(status, kFlagBadRowptr);
            out[e] = 0.0f;
            return;
        }
    } else {
        r = find_row(rows, M, static_cast<int>(e));
        if (__ldg(rows + r) > e || __ldg(rows + r + 1) <= e) {
            flag(status, kFlagBadRowptr);
            out[e] = 0.0f;
            return;
        }
    }
    if (static_cast<unsigned>(c) >= static_cast<unsigned>(N)) {
        flag(status, kFlagBadColind);
        out[e] = 0.0f;
        return;
    }
    const float *xr = X + static_cast<long>(r) * ldx;
    const float *yr = Y + static_cast<long>(c) * ldy;
    float p[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    int k = 0;
    if (VEC) {
        for (; k + 8 <= K; k += 8) {
            const float4 x0 = __ldg(reinterpret_cast<const float4 *>(xr + k));
            const float4 x1 = __ldg(reinterpret_cast<const float4 *>(xr + k + 4));
            const float4 y0 = __ldg(reinterpret_cast<const float4 *>(yr + k));
            const float4 y1 = __ldg(reinterpret_cast<const float4 *>(yr + k + 4));
            p[0] = fmaf(x0.x, y0.x, p[0]); p[1] = fmaf(x0.y, y0.y, p[1]);
            p[2] = fmaf(x0.z, y0.z, p[2]); p[3] = fmaf(x0.w, y0.w, p[3]);
            p[4] = fmaf(x1.x, y1.x, p[4]); p[5] = fmaf(x1.y, y1.y, p[5]);
            p[6] = fmaf(x1.z, y1.z, p[6]); p[7] = fmaf(x1.w, y1.w, p[7]);
        }
    }
    for (; k < K; ++k) p[k & 7] = fmaf(__ldg(xr + k), __ldg(yr + k), p[k & 7]);
    const float t = ((p[0] + p[4]) + (p[1] + p[5])) + ((p[2] + p[6]) + (p[3] + p[7]));
    out[e] = aval ? __ldg(aval + e) * t : t;
}

// bf16 X and Y (fp32 products and partial sums, fp32 out): the same eight interleaved
// partials as sddmm_f32_lane, each step the mixed-precision FMA of sm_100+ on two bf16
// operands (their product is exact in fp32, so the bits equal the fp32 kernel run on the
// bf16 values widened to fp32). Half the gathered bytes of the fp32 kernel.
__device__ __forceinline__ void fma_bf16_pair(unsigned x, unsigned y, float &p0, float &p1) {
    asm("{\n .reg .b16 xl, xh, yl, yh;\n mov.b32 {xl, xh}, %2;\n mov.b32 {yl, yh}, %3;\n"
        " fma.rn.f32.bf16 %0, xl, yl, %0;\n fma.rn.f32.bf16 %1, xh, yh, %1;\n}\n"
        : "+f"(p0), "+f"(p1) : "r"(x), "r"(y));
}

template <bool VEC>
__global__ void __launch_bounds__(kThreads)
sddmm_bf16_lane(int M, int N, int K, int nnz, const int *__restrict__ rowptr,
                const int *__restrict__ colind, const float *__restrict__ aval,
                const uint16_t *__restrict__ X, long ldx, const uint16_t *__restrict__ Y,
                long ldy, float *__restrict__ out, unsigned *status) {
    const long e = static_cast<long>(blockIdx.x) * kThreads + threadIdx.x;
    if (e >= nnz) return;
    const int c = ld_stream(colind + e);
    const int r = find_row(rowptr, M, static_cast<int>(e));
    if (__ldg(rowptr + r) > e || __ldg(rowptr + r + 1) <= e) {
        flag(status, kFlagBadRowptr);
        out[e] = 0.0f;
        return;
    }
    if (static_cast<unsigned>(c) >= static_cast<unsigned>(N)) {
        flag(status, kFlagBadColind);
        out[e] = 0.0f;
        return;
    }
    const uint16_t *xr = X + static_cast<long>(r) * ldx;
    const uint16_t *yr = Y + static_cast<long>(c) * ldy;
    float p[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    int k = 0;
    if (VEC) {
        for (; k + 8 <= K; k += 8) {
            const uint4 x = __ldg(reinterpret_cast<const uint4 *>(xr + k));
            const uint4 y = __ldg(reinterpret_cast<const uint4 *>(yr + k));
            fma_bf16_pair(x.x, y.x, p[0], p[1]);
            fma_bf16_pair(x.y, y.y, p[2], p[3]);
            fma_bf16_pair(x.z, y.z, p[4], p[5]);
            fma_bf16_pair(x.w, y.w, p[6], p[7]);
        }
    }
    for (; k < K; ++k)
        p[k & 7] = fmaf(bf16_to_f32(xr[k]), bf16_to_f32(yr[k]), p[k & 7]);
    const float t = ((p[0] + p[4]) + (p[1] + p[5])) + ((p[2] + p[6]) + (p[3] + p[7]));
    out[e] = aval ? __ldg(aval + e) * t : t;
}

}  // namespace

static as_status sddmm_lane_launch(as_ctx *ctx, bool coo, int M, int N, int K, int nnz,
                                   const int *rows, const int *colind, const float *aval,
                                   const float *X, long ldx, const float *Y, long ldy,
                                   float *out, cudaStream_t s) {
    if (M == 0) {
        // a pattern with entries but no rows is malformed
        return fail(AS_ERR_INVALID_CSR, "sddmm: nnz > 0 with zero rows");
    }
    const bool vec = (K % 8 == 0) && (ldx % 4 == 0) && (ldy % 4 == 0) &&
                     reinterpret_cast<uintptr_t>(X) % 16 == 0 &&
                     reinterpret_cast<uintptr_t>(Y) % 16 == 0;
    const unsigned grid = static_cast<unsigned>(ceil_div(nnz, kThreads));
    auto k = vec ? (coo ? sddmm_f32_lane<true, true> : sddmm_f32_lane<true, false>)
                 : (coo ? sddmm_f32_lane<false, true> : sddmm_f32_lane<false, false>);
    k<<<grid, kThreads, 0, s>>>(M, N, K, nnz, rows, colind, aval, X, ldx, Y, ldy, out,
                                ctx->d_status);
    ctx->launches++;
    return check_cuda(cudaGetLastError(), "sddmm_f32 launch");
}

as_status sddmm_f32_launch(as_ctx *ctx, int M, int N, int K, int nnz, const int *rowptr,
                           const int *colind, const float *aval, const float *X, long ldx,
                           const float *Y, long ldy, float *out, cudaStream_t s) {
    return sddmm_lane_launch(ctx, false, M, N, K, nnz, rowptr, colind, aval, X, ldx, Y, ldy, out, s);
}

as_status sddmm_bf16_launch(as_ctx *ctx, int M, int N, int K, int nnz, const int *rowptr,
                            const int *colind, const float *aval, const uint16_t *X, long ldx,
                            const uint16_t *Y, long ldy, float *out, cudaStream_t s) {
    if (M == 0) return fail(AS_ERR_INVALID_CSR, "sddmm: nnz > 0 with zero rows");
    const bool vec = (K % 8 == 0) && (ldx % 8 == 0) && (ldy % 8 == 0) &&
                     reinterpret_cast<uintptr_t>(X) % 16 == 0 &&
                     reinterpret_cast<uintptr_t>(Y) % 16 == 0;
    const unsigned grid = static_cast<unsigned>(ceil_div(nnz, kThreads));
    auto k = vec ? sddmm_bf16_lane<true> : sddmm_bf16_lane<false>;
    k<<<grid, kThreads, 0, s>>>(M, N, K, nnz, rowptr, colind, aval, X, ldx, Y, ldy, out,
                                ctx->d_status);
    ctx->launches++;
    return check_cuda(cudaGetLastError(), "sddmm_bf16 launch");
}

as_status sddmm_coo_f32_launch(as_ctx *ctx, int M, int N, int K, int nnz, const int *rowind,
                               const int *colind, const float *aval, const float *X, long ldx,
                               const float *Y, long ldy, float *out, cudaStream_t s) {
    return sddmm_lane_launch(ctx, true, M, N, K, nnz, rowind, colind, aval, X, ldx, Y, ldy, out, s);
}

}  // namespace as
