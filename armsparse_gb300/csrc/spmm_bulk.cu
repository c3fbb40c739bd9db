// CSR SpMM with the gathered rows of B staged through shared memory by bulk async copies
// (sm_103a): C = A*B + beta*C, fp32 or bf16 storage, fp32 accumulation.
//
// One warp per (row, column tile). Lane 0 keeps up to STAGES entries ahead of the warp: for
// each stored entry it issues one 1-D cp.async.bulk of the B-row segment the tile needs
// (32 * LB bytes, contiguous in global memory) into the warp's ring slot, completing on the
// slot's mbarrier. All lanes wait for the slot, read their LB bytes (consecutive across lanes,
// conflict-free) and update their accumulators with fmaf in CSR order -- the same per-output
// fused-FMA chain as the reference's rowBaseSpmm3 (SDMM.cpp:90-114), so results are
// bit-identical to the row-split kernels. The ring keeps STAGES * 32 * LB bytes per warp in
// flight without holding them in registers, which is what the register-path kernels run out
// of when the dense rows are gathered from L2.
//
// (colind, val) arrive in coalesced batches of 32 (current and next batch held in lane
// registers) and are broadcast with shuffles. Every wait is bounded: a timeout sets the status
// word, lane 0 waits (bounded) for the copies it issued, and the warp leaves. The warp's wait
// for a ring slot polls at most `spin_limit` times (the context's setting, as_ctx_set_spin_limit:
// a test sets it to 0 to take the timeout path); the drain of its issued copies before it
// leaves always polls up to kSpinLimit times per copy, so no copy is in flight when it exits.
#include "common.cuh"
#include "internal.h"

namespace as {
namespace {

constexpr int kWarps = 8;
constexpr unsigned kSpinLimit = 1u << 22;

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ bool bar_try(uint32_t bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ bool bar_wait(uint32_t bar, uint32_t parity, unsigned limit = kSpinLimit) {
    for (unsigned i = 0; i < limit; ++i)
        if (bar_try(bar, parity)) return true;
    return false;
}

template <typename T, int LB>
struct Lane;
template <>
struct Lane<float, 16> {
    static constexpr int E = 4;
    __device__ static void get(const uint8_t *p, float *o) {
        const float4 v = *reinterpret_cast<const float4 *>(p);
        o[0] = v.x; o[1] = v.y; o[2] = v.z; o[3] = v.w;
    }
};
template <>
struct Lane<float, 32> {
    static constexpr int E = 8;
    __device__ static void get(const uint8_t *p, float *o) {
        Lane<float, 16>::get(p, o);
        Lane<float, 16>::get(p + 16, o + 4);
    }
};
template <>
struct Lane<uint16_t, 16> {
    static constexpr int E = 8;
    __device__ static void get(const uint8_t *p, float *o) {
        const uint4 v = *reinterpret_cast<const uint4 *>(p);
        const unsigned w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            o[2 * i] = __uint_as_float(w[i] << 16);
            o[2 * i + 1] = __uint_as_float(w[i] & 0xffff0000u);
        }
    }
};
template <>
struct Lane<uint16_t, 32> {
    static constexpr int E = 16;
    __device__ static void get(const uint8_t *p, float *o) {
        Lane<uint16_t, 16>::get(p, o);
        Lane<uint16_t, 16>::get(p + 16, o + 8);
    }
};

__device__ __forceinline__ float to_f32(float v) { return v; }
__device__ __forceinline__ float to_f32(uint16_t v) { return bf16_to_f32(v); }

template <typename T, int LB, int STAGES>
struct BulkSmem {
    static constexpr int kSlot = 32 * LB;
    static constexpr int kRing = STAGES * kSlot;
    static constexpr int kBytes = kWarps * kRing + kWarps * STAGES * 8;
};

template <typename T, int LB, int STAGES>
__global__ void __launch_bounds__(kWarps * 32)
spmm_bulk(int M, int K, int N, int nnz, const int *__restrict__ rowptr,
          const int *__restrict__ colind, const T *__restrict__ val, const T *__restrict__ B,
          long ldb, float *__restrict__ C, long ldc, float beta, unsigned *status,
          unsigned spin_limit) {
    using L = Lane<T, LB>;
    using S = BulkSmem<T, LB, STAGES>;
    constexpr int E = L::E;
    constexpr int TILE = 32 * E;
    extern __shared__ __align__(128) uint8_t smem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const long row = static_cast<long>(blockIdx.x) * kWarps + warp;
    if (row >= M) return;  // whole warp
    uint8_t *ring = smem + warp * S::kRing;
    const uint32_t bar0 = smem_u32(smem + kWarps * S::kRing) + warp * STAGES * 8;
    if (lane == 0) {
        for (int s = 0; s < STAGES; ++s)
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar0 + 8 * s));
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncwarp();

    const int tile0 = blockIdx.y * TILE;
    const int c = tile0 + lane * E;
    const bool mine = c < N;
    const int ncols = min(TILE, N - tile0);
    const uint32_t bytes = static_cast<uint32_t>(ncols * sizeof(T));
    float acc[E];
    float *crow = C + row * ldc;
#pragma unroll
    for (int i = 0; i < E; ++i) acc[i] = (beta != 0.0f && mine) ? beta * crow[c + i] : 0.0f;

    int lo, hi;
    row_range(rowptr, static_cast<int>(row), nnz, status, lo, hi);
    const int n = hi - lo;
    // batches of 32 (colind, val): current and next, lane i holds entry 32*b + i
    auto load_batch = [&](int b, int &k, float &v) {
        const int e = lo + 32 * b + lane;
        k = -1;
        v = 0.0f;
        if (e < hi) {
            k = ld_stream(colind + e);
            v = to_f32(ld_stream(val + e));
            if (static_cast<unsigned>(k) >= static_cast<unsigned>(K)) {
                flag(status, kFlagBadColind);
                k = -1;
            }
        }
    };
    int kc, kn;
    float vc, vn;
    int cb = 0;  // batch index held in (kc, vc)
    load_batch(0, kc, vc);
    load_batch(1, kn, vn);

    int issued = 0;
    bool ok = true;
    for (int done = 0; done < n; ++done) {
        while (issued < n && issued < done + STAGES) {  // warp-uniform
            const int bi = issued >> 5;
            const int src = bi == cb ? kc : kn;
            const int k = __shfl_sync(0xffffffffu, src, issued & 31);
            const int slot = issued % STAGES;
            if (lane == 0) {
                const uint32_t bar = bar0 + 8 * slot;
                if (k >= 0) {
                    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar),
                                 "r"(bytes)
                                 : "memory");
                    asm volatile(
                        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::
                            "r"(smem_u32(ring + slot * S::kSlot)),
                        "l"(B + static_cast<long>(k) * ldb + tile0), "r"(bytes), "r"(bar)
                        : "memory");
                } else {
                    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(bar) : "memory");
                }
            }
            ++issued;
        }
        const int slot = done % STAGES;
        const bool got =
            __all_sync(0xffffffffu, bar_wait(bar0 + 8 * slot, (done / STAGES) & 1, spin_limit));
        if (!got) {
            ok = false;
            break;
        }
        const int bi = done >> 5;
        const int ksrc = bi == cb ? kc : kn;
        const float vsrc = bi == cb ? vc : vn;
        const int k = __shfl_sync(0xffffffffu, ksrc, done & 31);
        const float v = __shfl_sync(0xffffffffu, vsrc, done & 31);
        if (k >= 0 && mine) {
            float b[E];
            L::get(ring + slot * S::kSlot + lane * LB, b);
#pragma unroll
            for (int i = 0; i < E; ++i) acc[i] = fmaf(b[i], v, acc[i]);
        }
        __syncwarp();
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        if ((done & 31) == 31) {  // finished batch cb: shift and fetch cb + 2
            kc = kn;
            vc = vn;
            ++cb;
            load_batch(cb + 1, kn, vn);
        }
    }
    if (!ok) {
        if (lane == 0) {
            flag(status, kFlagTimeout);
            // let every copy this warp issued land before leaving
            for (int d = max(0, issued - STAGES); d < issued; ++d)
                bar_wait(bar0 + 8 * (d % STAGES), (d / STAGES) & 1);
        }
        __syncwarp();
        return;
    }
    if (mine) {
#pragma unroll
        for (int i = 0; i < E; i += 4)
            __stcs(reinterpret_cast<float4 *>(crow + c + i),
                   make_float4(acc[i], acc[i + 1], acc[i + 2], acc[i + 3]));
    }
}

template <typename T, int LB, int STAGES>
as_status launch(as_ctx *ctx, const SpmmArgs &a, cudaStream_t s) {
    using S = BulkSmem<T, LB, STAGES>;
    constexpr int E = Lane<T, LB>::E;
    constexpr int TILE = 32 * E;
    const int esz = sizeof(T);
    // bulk copies: 16-byte aligned addresses and sizes; whole lane vectors in every tile
    if ((a.N % E) || (a.ldb * esz) % 16 || (a.ldc % 4) ||
        reinterpret_cast<uintptr_t>(a.B) % 16 || reinterpret_cast<uintptr_t>(a.C) % 16 ||
        (static_cast<long>(a.N % TILE) * esz) % 16)
        return fail(AS_ERR_UNSUPPORTED, "spmm bulk variant: layout not 16-byte aligned");
    if (ceil_div(a.N, TILE) > 65535) return fail(AS_ERR_UNSUPPORTED, "spmm bulk: N too large");
    cudaError_t e = cudaFuncSetAttribute(spmm_bulk<T, LB, STAGES>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, S::kBytes);
    if (e != cudaSuccess) return check_cuda(e, "spmm bulk: shared memory attribute");
    dim3 grid(static_cast<unsigned>(ceil_div(a.M, kWarps)), static_cast<unsigned>(ceil_div(a.N, TILE)));
    spmm_bulk<T, LB, STAGES><<<grid, kWarps * 32, S::kBytes, s>>>(
        a.M, a.K, a.N, a.nnz, a.rowptr, a.colind, static_cast<const T *>(a.val),
        static_cast<const T *>(a.B), a.ldb, a.C, a.ldc, a.beta, a.status, ctx->spin_limit);
    ctx->launches++;
    return check_cuda(cudaGetLastError(), "spmm bulk launch");
}

}  // namespace

as_status spmm_bulk_launch(as_ctx *ctx, int dtype, int lane_bytes, int stages, const SpmmArgs &a,
                           cudaStream_t s) {
    if (dtype == 0) {
        if (lane_bytes == 16 && stages == 8) return launch<float, 16, 8>(ctx, a, s);
        if (lane_bytes == 32 && stages == 8) return launch<float, 32, 8>(ctx, a, s);
        if (lane_bytes == 16 && stages == 16) return launch<float, 16, 16>(ctx, a, s);
        if (lane_bytes == 32 && stages == 4) return launch<float, 32, 4>(ctx, a, s);
    } else {
        if (lane_bytes == 16 && stages == 8) return launch<uint16_t, 16, 8>(ctx, a, s);
        if (lane_bytes == 32 && stages == 8) return launch<uint16_t, 32, 8>(ctx, a, s);
        if (lane_bytes == 16 && stages == 16) return launch<uint16_t, 16, 16>(ctx, a, s);
        if (lane_bytes == 32 && stages == 4) return launch<uint16_t, 32, 4>(ctx, a, s);
    }
    return fail(AS_ERR_UNSUPPORTED, "spmm bulk: configuration not instantiated");
}

}  // namespace as
