// CSR SpMV, y = A*x + beta*y (sm_103a).
//
// Plain CSR: a group of GROUP lanes per row (GROUP picked from the mean row length so that
// short rows do not idle a whole warp); lane g sums entries g, g+GROUP, ... with fmaf, then
// the group reduces with xor shuffles (fixed tree, deterministic).
//
// 1x4-blocked layout of the reference (SpMV.cpp:15-38, consumed at SpMV.cpp:155-179): four
// lanes per row keep the reference's four lane sums s_l += val[idx+l] * x[k+l] over the row's
// blocks in order (fused steps, as GCC emits vmlaq_f32 under -ffp-contract=fast) and combine
// them as (s2 + s0) + (s3 + s1) before adding to y.
//
// Rows longer than kLongSpmv entries (slots) would keep one group walking dependent gathers
// long after the rest of the grid finished; both kernels list them (the long-row list of the
// context) and a second kernel gives each listed row a CTA: for plain CSR, 256 partial sums
// and a fixed reduction tree (deterministic); for the 1x4 layout, batches of 256 blocks staged
// in shared memory by all threads while four threads run the four chains over them in order
// (bit for bit the short-row kernel's result).
#include <limits.h>

#include <algorithm>

#include "common.cuh"
#include "internal.h"

namespace as {
namespace {

constexpr int kThreads = 256;
constexpr int kLongSpmv = 4096;  // entries (slots) of a row past which it gets a CTA

template <int GROUP>
__global__ void __launch_bounds__(kThreads)
spmv_csr(int M, int K, int nnz, const int *__restrict__ rowptr, const int *__restrict__ colind,
         const float *__restrict__ val, const float *__restrict__ x, float *__restrict__ y,
         float beta, unsigned *status, int long_thresh, int *long_list, unsigned *long_count) {
    asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory");
    const int lane = threadIdx.x & 31;
    const int g = threadIdx.x % GROUP;
    const unsigned gmask =
        GROUP == 32 ? 0xffffffffu : (((1u << GROUP) - 1u) << (lane & ~(GROUP - 1)));
    const long row = static_cast<long>(blockIdx.x) * (kThreads / GROUP) + threadIdx.x / GROUP;
    if (row >= M) return;
    int lo, hi;
    row_range(rowptr, static_cast<int>(row), nnz, status, lo, hi);
    if (hi - lo > long_thresh) {  // a CTA of the long-row kernel takes it
        if (g == 0) list_long_row(row, hi - lo, M, long_list, long_count, status);
        return;
    }
    // lane g sums its entries g, g + GROUP, ... in order, four gathers in flight
    float s = 0.0f;
    int e = lo + g;
    for (; e + 3 * GROUP < hi; e += 4 * GROUP) {
        int k[4];
        float v[4], xv[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            k[u] = ld_stream(colind + e + u * GROUP);
            v[u] = ld_stream(val + e + u * GROUP);
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const bool ok = static_cast<unsigned>(k[u]) < static_cast<unsigned>(K);
            if (!ok) flag(status, kFlagBadColind);
            xv[u] = ok ? __ldg(x + k[u]) : 0.0f;
            k[u] = ok ? k[u] : -1;
        }
#pragma unroll
        for (int u = 0; u < 4; ++u)
            if (k[u] >= 0) s = fmaf(v[u], xv[u], s);
    }
    for (; e < hi; e += GROUP) {
        const int k = ld_stream(colind + e);
        if (static_cast<unsigned>(k) >= static_cast<unsigned>(K)) {
            flag(status, kFlagBadColind);
            continue;
        }
        s = fmaf(ld_stream(val + e), __ldg(x + k), s);
    }
#pragma unroll
    for (int off = GROUP / 2; off > 0; off >>= 1) s += __shfl_xor_sync(gmask, s, off, GROUP);
    if (g == 0) y[row] = beta == 0.0f ? s : fmaf(beta, y[row], s);
}

// Four lanes per row: lane l keeps the chain s_l (so each chain stays in block order) and
// issues U blocks' loads before their FMAs; the lanes combine with two xor shuffles, lane 0
// ending with (s2 + s0) + (s3 + s1).
template <int U>
__global__ void __launch_bounds__(kThreads)
spmv_vcsr4(int M, int K, int nslots, const int *__restrict__ rowptr,
           const int *__restrict__ colind, const float *__restrict__ val,
           const float *__restrict__ x, float *__restrict__ y, float beta, unsigned *status,
           int long_thresh, int *long_list, unsigned *long_count) {
    asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory");
    const long row = (static_cast<long>(blockIdx.x) * kThreads + threadIdx.x) >> 2;
    const int l = threadIdx.x & 3;
    const unsigned gmask = 0xfu << (threadIdx.x & 28);
    if (row >= M) return;  // the four lanes of a row leave together
    int lo, hi;
    row_range(rowptr, static_cast<int>(row), nslots, status, lo, hi);
    if ((lo & 3) || (hi & 3)) {
        flag(status, kFlagBadRowptr);
        lo = hi = 0;
    }
    if (hi - lo > long_thresh) {  // a CTA of the long-row kernel takes it
        if (l == 0) list_long_row(row, hi - lo, M, long_list, long_count, status);
        return;
    }
    float s = 0.f;
    int idx = lo;
    for (; idx + 4 * U <= hi; idx += 4 * U) {
        int k[U];
        float v[U], xv[U];
#pragma unroll
        for (int u = 0; u < U; ++u) {
            k[u] = ld_stream(colind + idx + 4 * u);
            v[u] = ld_stream(val + idx + 4 * u + l);
        }
#pragma unroll
        for (int u = 0; u < U; ++u) {
            const bool ok = k[u] >= 0 && k[u] <= K - 4;
            if (!ok) {
                flag(status, kFlagBadColind);
                k[u] = -1;
            }
            xv[u] = ok ? __ldg(x + k[u] + l) : 0.f;
        }
#pragma unroll
        for (int u = 0; u < U; ++u)
            if (k[u] >= 0) s = fmaf(v[u], xv[u], s);
    }
    for (; idx < hi; idx += 4) {
        const int k = ld_stream(colind + idx);
        if (k < 0 || k > K - 4) {
            flag(status, kFlagBadColind);
            continue;
        }
        s = fmaf(ld_stream(val + idx + l), __ldg(x + k + l), s);
    }
    const float p = __fadd_rn(__shfl_xor_sync(gmask, s, 2), s);  // lane 0: s2+s0, lane 1: s3+s1
    const float r = __fadd_rn(p, __shfl_xor_sync(gmask, p, 1));
    if (l == 0) y[row] = beta == 0.0f ? r : __fadd_rn(beta * y[row], r);
}

// One CTA per listed long row (grid-stride over the list: the huge rows, listed from the end,
// first). MODE 0: plain CSR; MODE 1: the 1x4 layout.
template <int MODE>
__global__ void __launch_bounds__(kThreads)
spmv_long(int M, int K, int nnz, const int *__restrict__ rowptr, const int *__restrict__ colind,
          const float *__restrict__ val, const float *__restrict__ x, float *__restrict__ y,
          float beta, unsigned *status, const int *__restrict__ list, unsigned *counters) {
    __shared__ float red[kThreads / 32];
    // MODE 1: two buffers of a batch of kThreads blocks: values, their x entries, and whether
    // the block counts (a batch is staged by warps 1-7 while threads 0-3 run the other)
    __shared__ float sv[2][MODE == 1 ? 4 * kThreads : 1];
    __shared__ float sx[2][MODE == 1 ? 4 * kThreads : 1];
    __shared__ int sk[2][MODE == 1 ? kThreads : 1];
    // launched as a programmatic dependent of the row kernel: its list is complete after this
    asm volatile("griddepcontrol.wait;\n" ::: "memory");
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const unsigned cap = static_cast<unsigned>(M);
    const int n_long = static_cast<int>(min(*reinterpret_cast<volatile unsigned *>(counters), cap));
    const int n_huge =
        static_cast<int>(min(*reinterpret_cast<volatile unsigned *>(counters + 2), cap));
    for (int it = blockIdx.x; it < n_huge + n_long; it += gridDim.x) {
        const int r = it < n_huge ? list[M - 1 - it] : list[it - n_huge];
        if (r < 0 || r >= M) continue;
        int lo, hi;
        row_range(rowptr, r, nnz, status, lo, hi);
        if (MODE == 0) {
            // thread t sums entries lo + t, lo + t + 256, ... in order, four gathers in flight
            float s = 0.0f;
            int e = lo + tid;
            for (; e + 3 * kThreads < hi; e += 4 * kThreads) {
                int k[4];
                float v[4], xv[4];
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    k[u] = ld_stream(colind + e + u * kThreads);
                    v[u] = ld_stream(val + e + u * kThreads);
                }
#pragma unroll
                for (int u = 0; u < 4; ++u) {
                    const bool ok = static_cast<unsigned>(k[u]) < static_cast<unsigned>(K);
                    if (!ok) flag(status, kFlagBadColind);
                    xv[u] = ok ? __ldg(x + k[u]) : 0.0f;
                    k[u] = ok ? k[u] : -1;
                }
#pragma unroll
                for (int u = 0; u < 4; ++u)
                    if (k[u] >= 0) s = fmaf(v[u], xv[u], s);
            }
            for (; e < hi; e += kThreads) {
                const int k = ld_stream(colind + e);
                if (static_cast<unsigned>(k) >= static_cast<unsigned>(K)) {
                    flag(status, kFlagBadColind);
                    continue;
                }
                s = fmaf(ld_stream(val + e), __ldg(x + k), s);
            }
            // a fixed tree: within each warp, then over the warps' sums
#pragma unroll
            for (int off = 16; off > 0; off >>= 1) s += __shfl_xor_sync(0xffffffffu, s, off);
            if (lane == 0) red[warp] = s;
            __syncthreads();
            if (warp == 0) {
                float t = lane < kThreads / 32 ? red[lane] : 0.0f;
#pragma unroll
                for (int off = kThreads / 64; off > 0; off >>= 1) t += __shfl_xor_sync(0xffffffffu, t, off);
                if (lane == 0) y[r] = beta == 0.0f ? t : fmaf(beta, y[r], t);
            }
            __syncthreads();
        } else {
            if ((lo & 3) || (hi & 3)) lo = hi = 0;  // flagged by the row kernel
            const int n_batches = static_cast<int>(ceil_div((hi - lo) / 4, kThreads));
            // stage batch j (its blocks lo + 4 * (j * kThreads + i)) into buffer j & 1, by the
            // threads [t0, kThreads)
            auto stage = [&](int j, int t0) {
                for (int i = tid - t0; i < kThreads; i += kThreads - t0) {
                    const int b = lo + 4 * (j * kThreads + i);
                    if (b >= hi) break;
                    const int k = ld_stream(colind + b);
                    const bool ok = k >= 0 && k <= K - 4;
                    if (!ok) flag(status, kFlagBadColind);
                    const float4 v4 = __ldcs(reinterpret_cast<const float4 *>(val + b));
                    float *v = sv[j & 1] + 4 * i, *xs = sx[j & 1] + 4 * i;
                    v[0] = v4.x;
                    v[1] = v4.y;
                    v[2] = v4.z;
                    v[3] = v4.w;
#pragma unroll
                    for (int q = 0; q < 4; ++q) xs[q] = ok ? __ldg(x + k + q) : 0.0f;
                    sk[j & 1][i] = ok;
                }
            };
            float s = 0.0f;  // threads 0-3: the chain of lane position tid
            if (n_batches > 0) stage(0, 0);
            __syncthreads();
            for (int j = 0; j < n_batches; ++j) {
                if (tid >= 32) {
                    if (j + 1 < n_batches) stage(j + 1, 32);
                } else if (tid < 4) {
                    const int nb = min(kThreads, (hi - lo) / 4 - j * kThreads);
                    const float *v = sv[j & 1], *xs = sx[j & 1];
                    const int *ok = sk[j & 1];
                    int i = 0;
                    for (; i + 8 <= nb; i += 8) {  // the batch's loads before its fused steps
                        float a[8], c[8];
                        int f[8];
#pragma unroll
                        for (int u = 0; u < 8; ++u) {
                            a[u] = v[4 * (i + u) + tid];
                            c[u] = xs[4 * (i + u) + tid];
                            f[u] = ok[i + u];
                        }
#pragma unroll
                        for (int u = 0; u < 8; ++u)
                            if (f[u]) s = fmaf(a[u], c[u], s);
                    }
                    for (; i < nb; ++i)
                        if (ok[i]) s = fmaf(v[4 * i + tid], xs[4 * i + tid], s);
                }
                __syncthreads();
            }
            if (tid < 4) red[tid] = s;
            __syncthreads();
            if (tid == 0) {
                const float t = __fadd_rn(__fadd_rn(red[2], red[0]), __fadd_rn(red[3], red[1]));
                y[r] = beta == 0.0f ? t : __fadd_rn(beta * y[r], t);
            }
            __syncthreads();
        }
    }
    // the last CTA out resets the list counters and the done counter for the next call
    __syncthreads();
    if (tid == 0) {
        __threadfence();
        if (atomicAdd(counters + 1, 1u) == gridDim.x - 1) {
            counters[0] = 0;
            counters[1] = 0;
            counters[2] = 0;
            __threadfence();
        }
    }
}

// The long-row kernel after a row kernel that listed rows (programmatic dependent launch
// outside stream capture, so its CTAs are scheduled while the row kernel drains).
template <int MODE>
as_status launch_long(as_ctx *ctx, int M, int K, int nnz, const int *rowptr, const int *colind,
                      const float *val, const float *x, float *y, float beta, const int *list,
                      cudaStream_t s) {
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(s, &cap);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(static_cast<unsigned>(std::max(1, std::min(M, 4 * ctx->sms))));
    cfg.blockDim = dim3(kThreads);
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = cap == cudaStreamCaptureStatusNone ? 1 : 0;
    cudaError_t e = cudaLaunchKernelEx(&cfg, spmv_long<MODE>, M, K, nnz, rowptr, colind, val, x,
                                       y, beta, ctx->d_status, list, ctx->d_long);
    ctx->launches++;
    as_status st = check_cuda(e != cudaSuccess ? e : cudaGetLastError(), "spmv long rows launch");
    if (st != AS_OK) cudaMemsetAsync(ctx->d_long, 0, 3 * sizeof(unsigned), s);
    return st;
}

// Scratch for the long-row list when a row can exceed kLongSpmv entries: more than that many
// entries in all, and more columns (a row of distinct columns holds at most `max_row`, K or K
// rounded up to whole 1x4 blocks; a malformed row with repeated columns stays on the row
// kernel, which handles any length). Otherwise no list and no second launch, which matters
// for a small SpMV.
as_status long_list(as_ctx *ctx, int M, int nnz, long max_row, int *&list, int &thresh) {
    list = nullptr;
    thresh = INT_MAX;
    if (nnz <= kLongSpmv || M <= 0 || max_row <= kLongSpmv) return AS_OK;
    void *p = nullptr;
    as_status st = scratch(ctx, static_cast<size_t>(M) * sizeof(int), &p);
    if (st != AS_OK) return st;
    list = static_cast<int *>(p);
    thresh = kLongSpmv;
    return AS_OK;
}

}  // namespace

as_status spmv_csr_launch(as_ctx *ctx, int M, int K, int nnz, const int *rowptr,
                          const int *colind, const float *val, const float *x, float *y,
                          float beta, cudaStream_t s) {
    const double mean = M > 0 ? static_cast<double>(nnz) / M : 0.0;
    int group = 2;
    while (group < 32 && group < mean) group <<= 1;
    int *list;
    int thresh;
    as_status st = long_list(ctx, M, nnz, K, list, thresh);
    if (st != AS_OK) return st;
    const unsigned grid = static_cast<unsigned>(ceil_div(M, kThreads / group));
#define AS_SPMV_G(G)                                                                          \
    case G:                                                                                   \
        spmv_csr<G><<<grid, kThreads, 0, s>>>(M, K, nnz, rowptr, colind, val, x, y, beta,     \
                                               ctx->d_status, thresh, list, ctx->d_long);     \
        break;
    switch (group) {
        AS_SPMV_G(2) AS_SPMV_G(4) AS_SPMV_G(8) AS_SPMV_G(16)
        default: spmv_csr<32><<<grid, kThreads, 0, s>>>(M, K, nnz, rowptr, colind, val, x, y, beta,
                                                        ctx->d_status, thresh, list, ctx->d_long);
    }
#undef AS_SPMV_G
    ctx->launches++;
    st = check_cuda(cudaGetLastError(), "spmv_csr launch");
    if (st != AS_OK || !list) return st;
    return launch_long<0>(ctx, M, K, nnz, rowptr, colind, val, x, y, beta, list, s);
}

as_status spmv_vcsr4_launch(as_ctx *ctx, int M, int K, int nslots, const int *rowptr,
                            const int *colind, const float *val, const float *x, float *y,
                            float beta, cudaStream_t s) {
    if (reinterpret_cast<uintptr_t>(val) % 16)
        return fail(AS_ERR_INVALID_VALUE, "as_spmv_vcsr4_f32: val must be 16-byte aligned");
    int *list;
    int thresh;
    as_status st = long_list(ctx, M, nslots, static_cast<long>(K) + 3, list, thresh);
    if (st != AS_OK) return st;
    const unsigned grid = static_cast<unsigned>(ceil_div(static_cast<long>(M) * 4, kThreads));
    spmv_vcsr4<8><<<grid, kThreads, 0, s>>>(M, K, nslots, rowptr, colind, val, x, y, beta,
                                         ctx->d_status, thresh, list, ctx->d_long);
    ctx->launches++;
    st = check_cuda(cudaGetLastError(), "spmv_vcsr4 launch");
    if (st != AS_OK || !list) return st;
    return launch_long<1>(ctx, M, K, nslots, rowptr, colind, val, x, y, beta, list, s);
}

}  // namespace as
