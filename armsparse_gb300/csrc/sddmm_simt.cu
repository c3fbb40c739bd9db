// SDDMM on CUDA cores: out[e] = s_e * <X[row(e), :], Y[col(e), :]> (sm_103a), fp32 or bf16
// operands, fp32 products and sums.
//
// A group of G lanes takes one edge at a time (G = about one lane per four 4-element blocks of
// K, a power of two up to a warp), so each Y row is read by neighbouring lanes in 16-byte (fp32) or
// 8-byte (bf16) pieces -- coalesced -- and the X row, shared by the consecutive edges of one
// row, comes from L1. A group walks a chunk of consecutive edges in CSR order: one binary
// search over rowptr for its first edge (the reference searches per edge, findRow in
// gcn/pytorch-custom/computeUtil.h:11-28), then the row pointer steps forward; the COO form
// reads each edge's row from the row array (the reference's sddmm_cuda_coo, sddmm.cu:427-457).
//
// Summation order (the oracle's or_sddmm_csr_f32_group): lane l runs one fused-FMA chain over
// the blocks l, l + G, l + 2G, ... of K in order; the lanes are summed by a butterfly
// (acc += shfl_xor(acc, off), off = G/2 .. 1); lane 0 writes s_e * sum. bf16 operands use the
// mixed-precision FMA of sm_100+ (a bf16 x bf16 product is exact in fp32), so the bf16 kernel
// gives bit for bit the fp32 kernel's result on the widened values.
#include "common.cuh"
#include "internal.h"

namespace as {
namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ int find_row(const int *__restrict__ rowptr, int M, long e) {
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

// acc = fma(x0, y0, acc); acc = fma(x1, y1, acc) for the bf16 halves of x and y, in order.
__device__ __forceinline__ void fma_bf16_seq2(unsigned x, unsigned y, float &acc) {
    asm("{\n .reg .b16 xl, xh, yl, yh;\n mov.b32 {xl, xh}, %1;\n mov.b32 {yl, yh}, %2;\n"
        " fma.rn.f32.bf16 %0, xl, yl, %0;\n fma.rn.f32.bf16 %0, xh, yh, %0;\n}\n"
        : "+f"(acc) : "r"(x), "r"(y));
}

__device__ __forceinline__ float to_f32(float v) { return v; }
__device__ __forceinline__ float to_f32(uint16_t v) { return bf16_to_f32(v); }

// One 4-element block of the dot product, elements in order.
template <typename T>
struct Block;
template <>
struct Block<float> {
    using Raw = float4;
    __device__ static Raw load(const float *p) { return __ldg(reinterpret_cast<const float4 *>(p)); }
    __device__ static void chain(const Raw &x, const Raw &y, float &acc) {
        acc = fmaf(x.x, y.x, acc);
        acc = fmaf(x.y, y.y, acc);
        acc = fmaf(x.z, y.z, acc);
        acc = fmaf(x.w, y.w, acc);
    }
};
template <>
struct Block<uint16_t> {
    using Raw = uint2;
    __device__ static Raw load(const uint16_t *p) { return __ldg(reinterpret_cast<const uint2 *>(p)); }
    __device__ static void chain(const Raw &x, const Raw &y, float &acc) {
        fma_bf16_seq2(x.x, y.x, acc);
        fma_bf16_seq2(x.y, y.y, acc);
    }
};

// Lane's chain over the blocks g, g + G, ... of one edge, four blocks at a time with all
// their loads issued before the FMAs. VEC: K % 4 == 0 and 4-element aligned rows, one vector
// load per block; else element loads (elements past K contribute nothing).
template <typename T, bool VEC, int G>
__device__ __forceinline__ float lane_chain(const T *xr, const T *yr, int K, int g) {
    using B = Block<T>;
    const int nq = (K + 3) >> 2;
    float acc = 0.0f;
    for (int q = g; q < nq; q += 4 * G) {
        if (VEC) {
            typename B::Raw x[4], y[4];
#pragma unroll
            for (int u = 0; u < 4; ++u) {
                const int qq = q + u * G;
                if (qq < nq) {
                    x[u] = B::load(xr + 4 * qq);
                    y[u] = B::load(yr + 4 * qq);
                }
            }
#pragma unroll
            for (int u = 0; u < 4; ++u)
                if (q + u * G < nq) B::chain(x[u], y[u], acc);
        } else {
            float x[4][4], y[4][4];
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    const int k = 4 * (q + u * G) + i;
                    x[u][i] = k < K ? to_f32(xr[k]) : 0.0f;
                    y[u][i] = k < K ? to_f32(yr[k]) : 0.0f;
                }
#pragma unroll
            for (int u = 0; u < 4; ++u)
#pragma unroll
                for (int i = 0; i < 4; ++i)
                    if (4 * (q + u * G) + i < K) acc = fmaf(x[u][i], y[u][i], acc);
        }
    }
    return acc;
}

// COO: rows come per edge from `rows` (any order); CSR: `rows` is the row pointer.
template <typename T, bool VEC, int G, bool COO>
__global__ void __launch_bounds__(kThreads)
sddmm_group(int M, int N, int K, int nnz, int CH, const int *__restrict__ rows,
            const int *__restrict__ colind, const float *__restrict__ aval,
            const T *__restrict__ X, long ldx, const T *__restrict__ Y, long ldy,
            float *__restrict__ out, unsigned *status) {
    const long grp = (static_cast<long>(blockIdx.x) * kThreads + threadIdx.x) / G;
    const int g = threadIdx.x % G;
    const unsigned gmask =
        G == 32 ? 0xffffffffu : (((1u << G) - 1u) << ((threadIdx.x & 31) & ~(G - 1)));
    const long e0 = grp * CH;
    if (e0 >= nnz) return;  // the whole group leaves together
    const long e1 = e0 + CH < nnz ? e0 + CH : nnz;
    int r = 0, rs = 0, re = 0;
    if (!COO) {
        r = find_row(rows, M, e0);
        rs = __ldg(rows + r);
        re = __ldg(rows + r + 1);
    }
    for (long e = e0; e < e1; ++e) {  // every branch below is the same for the whole group
        int row;
        if (COO) {
            row = ld_stream(rows + e);
            if (static_cast<unsigned>(row) >= static_cast<unsigned>(M)) {
                if (g == 0) {
                    flag(status, kFlagBadRowptr);
                    out[e] = 0.0f;
                }
                continue;
            }
        } else {
            while (e >= re && r + 1 < M) {
                ++r;
                rs = re;
                re = __ldg(rows + r + 1);
            }
            if (rs > e || re <= e) {
                if (g == 0) {
                    flag(status, kFlagBadRowptr);
                    out[e] = 0.0f;
                }
                continue;
            }
            row = r;
        }
        const int c = ld_stream(colind + e);
        if (static_cast<unsigned>(c) >= static_cast<unsigned>(N)) {
            if (g == 0) {
                flag(status, kFlagBadColind);
                out[e] = 0.0f;
            }
            continue;
        }
        float acc = lane_chain<T, VEC, G>(X + static_cast<long>(row) * ldx,
                                          Y + static_cast<long>(c) * ldy, K, g);
#pragma unroll
        for (int off = G / 2; off > 0; off >>= 1) acc += __shfl_xor_sync(gmask, acc, off, G);
        if (g == 0) out[e] = aval ? __ldg(aval + e) * acc : acc;
    }
}

int group_size(int K) {  // the oracle's or_sddmm_group_size: about four blocks per lane
    const int q = (K + 15) / 16;
    int g = 1;
    while (g < q && g < 32) g <<= 1;
    return g;
}

template <typename T, bool COO>
as_status launch_group(as_ctx *ctx, int M, int N, int K, int nnz, const int *rows,
                       const int *colind, const float *aval, const T *X, long ldx, const T *Y,
                       long ldy, float *out, cudaStream_t s, const char *what) {
    if (M == 0) return fail(AS_ERR_INVALID_CSR, "sddmm: nnz > 0 with zero rows");
    const int esz = static_cast<int>(sizeof(T));
    const bool vec = K % 4 == 0 && ldx % 4 == 0 && ldy % 4 == 0 &&
                     reinterpret_cast<uintptr_t>(X) % (4 * esz) == 0 &&
                     reinterpret_cast<uintptr_t>(Y) % (4 * esz) == 0;
    const int G = group_size(K);
    const int CH = G >= 32 ? 4 : 128 / G;  // edges per group: more for short dot products
    const long groups = ceil_div(nnz, CH);
    const unsigned grid = static_cast<unsigned>(ceil_div(groups * G, kThreads));
#define AS_SDDMM_G(GV)                                                                      \
    case GV:                                                                                \
        if (vec)                                                                            \
            sddmm_group<T, true, GV, COO><<<grid, kThreads, 0, s>>>(                        \
                M, N, K, nnz, CH, rows, colind, aval, X, ldx, Y, ldy, out, ctx->d_status);  \
        else                                                                                \
            sddmm_group<T, false, GV, COO><<<grid, kThreads, 0, s>>>(                       \
                M, N, K, nnz, CH, rows, colind, aval, X, ldx, Y, ldy, out, ctx->d_status);  \
        break;
    switch (G) {
        AS_SDDMM_G(1) AS_SDDMM_G(2) AS_SDDMM_G(4) AS_SDDMM_G(8) AS_SDDMM_G(16) AS_SDDMM_G(32)
        default: return fail(AS_ERR_UNSUPPORTED, "sddmm: group size");
    }
#undef AS_SDDMM_G
    ctx->launches++;
    return check_cuda(cudaGetLastError(), what);
}

}  // namespace

as_status sddmm_f32_launch(as_ctx *ctx, int M, int N, int K, int nnz, const int *rowptr,
                           const int *colind, const float *aval, const float *X, long ldx,
                           const float *Y, long ldy, float *out, cudaStream_t s) {
    return launch_group<float, false>(ctx, M, N, K, nnz, rowptr, colind, aval, X, ldx, Y, ldy,
                                      out, s, "sddmm_f32 launch");
}

as_status sddmm_bf16_launch(as_ctx *ctx, int M, int N, int K, int nnz, const int *rowptr,
                            const int *colind, const float *aval, const uint16_t *X, long ldx,
                            const uint16_t *Y, long ldy, float *out, cudaStream_t s) {
    return launch_group<uint16_t, false>(ctx, M, N, K, nnz, rowptr, colind, aval, X, ldx, Y,
                                         ldy, out, s, "sddmm_bf16 launch");
}

as_status sddmm_coo_f32_launch(as_ctx *ctx, int M, int N, int K, int nnz, const int *rowind,
                               const int *colind, const float *aval, const float *X, long ldx,
                               const float *Y, long ldy, float *out, cudaStream_t s) {
    return launch_group<float, true>(ctx, M, N, K, nnz, rowind, colind, aval, X, ldx, Y, ldy,
                                     out, s, "sddmm_coo_f32 launch");
}

}  // namespace as
