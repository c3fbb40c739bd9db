// Long rows of the row-split SpMM (sm_103a), bit-identical to rowBaseSpmm3 (SDMM.cpp:90-114).
//
// A row-split group walks its row's entries one after another, so one row with 10^5 entries
// (a hub of a power-law graph) keeps a single group busy long after the rest of the grid has
// finished. The row-split kernels therefore leave every row longer than a threshold to this
// kernel: they append the row number to a list (one atomic per long row) and skip it; this
// kernel, launched right after on the same stream, takes the listed rows.
//
// Each output element is still one fused-FMA chain over the row's entries in CSR order (the
// order cannot be split without changing the bits), so the speed comes from feeding the
// chains. A CTA takes one (long row, 64-byte column slice) at a time and splits its warps by
// role:
//  - warp 0 is the consumer: one lane per column of the slice runs the chain out of shared
//    memory, stage after stage, reading each entry's B segment and value from the stage's slot;
//  - warps 1-2 are producers, one thread per entry of a stage of kStage entries: the thread
//    copies its entry's B segment into the stage's ring slot with cp.async, and the entry's
//    column index for the stage kLag ahead into its own slot of a small index ring (cp.async
//    too), one commit group per stage. Before stage s it waits for its group of stage s - kLag
//    (cp.async.wait_group): that gives it stage s's index and tells it that its copies of stage
//    s - kLag have landed, which its warp then announces on that slot's `full` mbarrier (one
//    arrival per warp after __syncwarp; one lane per warp polls `empty`). The entry's
//    value it loads kLag stages ahead into a ring of kLag registers (the stage loop is unrolled
//    kLag times, so each register is named statically and none is read before its load is kLag
//    stages old) and stores it beside the B segment. A slot is refilled only after the consumer
//    arrives on its `empty` mbarrier.
// Every arrival is a synchronous one by the arriving thread (none is left pending when the CTA
// moves on).
// Every wait is bounded; a wait that gives up sets the timeout flag and an abort flag that makes
// the other role leave too; each thread waits for its own copies before the CTA moves on, and a
// row whose wait gave up is left unwritten. A malformed column index is flagged and its entry
// gets a zero segment (nothing is read for it).
//
// The list counter and a CTA-done counter live in the context's device words; the last CTA
// to finish resets both, so the next call starts from zero without a memset.
#include <algorithm>

#include "common.cuh"
#include "internal.h"

namespace as {
namespace {

constexpr int kStage = 64;                 // entries per pipeline stage
constexpr int kProducers = kStage;         // warps 1-2: one thread per entry of a stage
constexpr int kThreads = 32 + kProducers;
constexpr int kSliceBytes = 64;            // B bytes per entry per stage (16 fp32 / 32 bf16 columns)
constexpr int kStages = 24;                // B ring slots
constexpr int kLag = 12;                   // stages of copies in flight per producer thread
constexpr int kIdx = kLag + 1;             // index ring slots (a thread reads slot s, refills s + kLag)
static_assert(kLag < kStages, "a producer must announce stage s before it waits to refill its slot");
constexpr unsigned kSpinLimit = 1u << 22;  // polls of a bounded wait (a few seconds at most)
constexpr int kRingBytes = kStages * kStage * kSliceBytes;
constexpr int kIdxBytes = kIdx * kStage * 4;
constexpr int kVringBytes = kStages * kStage * 4;  // each entry's value, beside its B segment
constexpr int kSmemBytes = kRingBytes + kIdxBytes + kVringBytes + 2 * kStages * 8 + 16;

__device__ __forceinline__ float to_f32(float v) { return v; }
__device__ __forceinline__ float to_f32(uint16_t v) { return bf16_to_f32(v); }

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

template <int GB>
__device__ __forceinline__ void cp_async(uint32_t dst, const void *gmem) {
    if constexpr (GB == 16)
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(dst), "l"(gmem) : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(dst), "l"(gmem) : "memory");
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

// Bounded wait for `parity` of the mbarrier at `bar`; false when `limit` polls pass or the
// other role has given up.
__device__ __forceinline__ bool bar_wait(uint32_t bar, uint32_t parity, unsigned limit,
                                         const volatile int *abort_flag) {
    for (unsigned i = 0; i < limit; ++i) {
        if (bar_try(bar, parity)) return true;
        if (*abort_flag) return false;
    }
    return false;
}

// T: storage type of val and B (float or uint16_t = bf16); GB: cp.async size in bytes.
template <typename T, int GB>
__global__ void __launch_bounds__(kThreads)
spmm_long(int M, int K, int N, int nnz, const int *__restrict__ rowptr,
          const int *__restrict__ colind, const T *__restrict__ val, const T *__restrict__ B,
          long ldb, float *__restrict__ C, long ldc, float beta, unsigned *status,
          const int *__restrict__ list, unsigned *counters, uint16_t *__restrict__ C16,
          bool relu, unsigned spin_limit) {
    constexpr int W = kSliceBytes / static_cast<int>(sizeof(T));  // columns per slice
    extern __shared__ __align__(128) unsigned char smem[];
    unsigned char *ring = smem;                                    // [kStages][kStage][64 B]
    int *kring = reinterpret_cast<int *>(smem + kRingBytes);       // [kIdx][kStage]
    float *vring = reinterpret_cast<float *>(smem + kRingBytes + kIdxBytes);  // [kStages][kStage]
    uint64_t *full = reinterpret_cast<uint64_t *>(smem + kRingBytes + kIdxBytes + kVringBytes);
    uint64_t *empty = full + kStages;
    volatile int *abort_flag = reinterpret_cast<volatile int *>(empty + kStages);

    // launched as a programmatic dependent of the row-split kernel: wait for it to finish
    // (and its list writes to be visible) before reading the list
    asm volatile("griddepcontrol.wait;\n" ::: "memory");
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int n_long = static_cast<int>(
        min(*reinterpret_cast<volatile unsigned *>(counters), static_cast<unsigned>(M)));
    const int n_slices = static_cast<int>(ceil_div(N, W));
    const long units = static_cast<long>(n_long) * n_slices;

    // work units (long row, column slice), the slices of one row on consecutive CTAs
    for (long u = blockIdx.x; u < units; u += gridDim.x) {
        const int item = static_cast<int>(u / n_slices);
        const int slice0 = static_cast<int>(u - static_cast<long>(item) * n_slices) * W;
        const int w = min(W, N - slice0);                  // columns of this slice
        const int pieces = w * static_cast<int>(sizeof(T)) / GB;  // copy pieces per entry
        const int r = list[item];
        if (r < 0 || r >= M) continue;
        int lo, hi;
        row_range(rowptr, r, nnz, status, lo, hi);
        const int L = hi - lo;
        const int n_stages = static_cast<int>(ceil_div(L, kStage));

        if (tid == 0) {
            for (int s = 0; s < kStages; ++s) {
                asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(full + s)),
                             "r"(kProducers / 32));
                asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_u32(empty + s)));
            }
            *abort_flag = 0;
            asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        }
        __syncthreads();

        float acc = 0.0f;
        float *crow = C + static_cast<long>(r) * ldc + slice0;
        if (warp == 0) {
            // ---- consumer: the chains ----
            const int col = lane < W ? lane : lane & (W - 1);  // lanes past the slice mirror
            if (lane < w && beta != 0.0f) acc = crow[lane] * beta;
            for (int s = 0; s < n_stages; ++s) {
                const int slot = s % kStages;
                const bool ok = __all_sync(
                    0xffffffffu, bar_wait(smem_u32(full + slot), (s / kStages) & 1, spin_limit,
                                          abort_flag));
                if (!ok) {
                    if (lane == 0) {
                        flag(status, kFlagTimeout);
                        *abort_flag = 1;
                    }
                    break;
                }
                const int n = min(kStage, L - s * kStage);
                const float *vs = vring + slot * kStage;
                const T *bs = reinterpret_cast<const T *>(ring + slot * kStage * kSliceBytes) + col;
                int j = 0;
                if (n >= 8) {  // the next 8 entries' loads are in flight during this 8's chain
                    float b[8], bn[8];
                    float4 v0 = *reinterpret_cast<const float4 *>(vs);
                    float4 v1 = *reinterpret_cast<const float4 *>(vs + 4);
#pragma unroll
                    for (int i = 0; i < 8; ++i) b[i] = to_f32(bs[i * W]);
                    for (; j + 8 <= n; j += 8) {
                        const bool more = j + 16 <= n;
                        float4 n0 = v0, n1 = v1;
                        if (more) {
                            n0 = *reinterpret_cast<const float4 *>(vs + j + 8);
                            n1 = *reinterpret_cast<const float4 *>(vs + j + 12);
#pragma unroll
                            for (int i = 0; i < 8; ++i) bn[i] = to_f32(bs[(j + 8 + i) * W]);
                        }
                        acc = fmaf(b[0], v0.x, acc);
                        acc = fmaf(b[1], v0.y, acc);
                        acc = fmaf(b[2], v0.z, acc);
                        acc = fmaf(b[3], v0.w, acc);
                        acc = fmaf(b[4], v1.x, acc);
                        acc = fmaf(b[5], v1.y, acc);
                        acc = fmaf(b[6], v1.z, acc);
                        acc = fmaf(b[7], v1.w, acc);
                        if (more) {
                            v0 = n0;
                            v1 = n1;
#pragma unroll
                            for (int i = 0; i < 8; ++i) b[i] = bn[i];
                        }
                    }
                }
                for (; j < n; ++j) acc = fmaf(to_f32(bs[j * W]), vs[j], acc);
                __syncwarp();
                if (lane == 0)
                    asm volatile("mbarrier.arrive.release.cta.shared::cta.b64 _, [%0];" ::"r"(
                                     smem_u32(empty + slot))
                                 : "memory");
            }
        } else {
            // ---- producers: thread p owns entry p of every stage ----
            const int p = tid - 32;
            // the warp's copies and stores of stage st are done: __syncwarp orders every lane's
            // (each waited for its own copies) before lane 0's release arrival, one per warp
            auto announce = [&](int st) {
                __syncwarp();
                if (lane == 0)
                    asm volatile("mbarrier.arrive.release.cta.shared::cta.b64 _, [%0];" ::"r"(
                                     smem_u32(full + st % kStages))
                                 : "memory");
            };
            auto copy_index = [&](int st) {  // column index of stage st's entry p, into the ring
                const int e = st * kStage + p;
                if (st < n_stages && e < L)
                    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(
                                     smem_u32(kring + (st % kIdx) * kStage + p)),
                                 "l"(colind + lo + e)
                                 : "memory");
            };
            for (int t = 0; t < kLag; ++t) {  // the first kLag stages' indices, a group each
                copy_index(t);
                asm volatile("cp.async.commit_group;\n" ::: "memory");
            }
            // value of stage st's entry p (0 past the row)
            auto load_value = [&](int st) {
                const int e = st * kStage + p;
                return (st < n_stages && e < L) ? to_f32(ld_stream(val + lo + e)) : 0.0f;
            };
            float vr[kLag];  // vr[s % kLag]: the value of stage s, loaded at stage s - kLag
#pragma unroll
            for (int t = 0; t < kLag; ++t) vr[t] = load_value(t);
            // one stage; false when the wait for its slot gave up
            auto stage = [&](int s, float &vreg) {
                // this thread's group kLag back has landed: stage s's index, and its copies of
                // stage s - kLag (announced now)
                asm volatile("cp.async.wait_group %0;\n" ::"n"(kLag - 1) : "memory");
                if (s >= kLag) announce(s - kLag);
                const int slot = s % kStages;
                if (s >= kStages) {
                    // lane 0 waits for the consumer to free the slot; the shuffle orders the
                    // other lanes' writes after its acquire
                    int ok = 1;
                    if (lane == 0)
                        ok = bar_wait(smem_u32(empty + slot), ((s / kStages) - 1) & 1, kSpinLimit,
                                      abort_flag);
                    if (!__shfl_sync(0xffffffffu, ok, 0)) {
                        if (lane == 0 && !*abort_flag) {
                            flag(status, kFlagTimeout);
                            *abort_flag = 1;
                        }
                        return false;
                    }
                }
                const int e = s * kStage + p;
                if (e < L) {
                    const int k = kring[(s % kIdx) * kStage + p];
                    unsigned char *d = ring + (slot * kStage + p) * kSliceBytes;
                    if (static_cast<unsigned>(k) < static_cast<unsigned>(K)) {
                        const unsigned char *src = reinterpret_cast<const unsigned char *>(
                            B + static_cast<long>(k) * ldb + slice0);
                        for (int q = 0; q < pieces; ++q) cp_async<GB>(smem_u32(d + q * GB), src + q * GB);
                        vring[slot * kStage + p] = vreg;
                    } else {  // malformed: a zero segment and value, nothing read
                        flag(status, kFlagBadColind);
                        for (int q = 0; q < pieces; ++q) {
                            if constexpr (GB == 16)
                                *reinterpret_cast<uint4 *>(d + q * GB) = make_uint4(0, 0, 0, 0);
                            else
                                *reinterpret_cast<unsigned *>(d + q * GB) = 0u;
                        }
                        vring[slot * kStage + p] = 0.0f;
                    }
                }
                vreg = load_value(s + kLag);  // read again kLag stages from now
                copy_index(s + kLag);
                asm volatile("cp.async.commit_group;\n" ::: "memory");
                return true;
            };
            int issued = 0;
            bool go = true;
            for (int s0 = 0; go && s0 < n_stages; s0 += kLag) {
#pragma unroll
                for (int u = 0; u < kLag; ++u) {
                    if (s0 + u >= n_stages || !(go = stage(s0 + u, vr[u]))) break;
                    issued = s0 + u + 1;
                }
            }
            // the last stages: all copies landed (the decision is the warp's, as announce syncs it)
            if (__shfl_sync(0xffffffffu, static_cast<int>(!*abort_flag), 0)) {
                asm volatile("cp.async.wait_all;\n" ::: "memory");
                for (int st = issued > kLag ? issued - kLag : 0; st < issued; ++st) announce(st);
            }
        }
        asm volatile("cp.async.wait_all;\n" ::: "memory");  // this thread's copies have landed
        __syncthreads();
        if (warp == 0 && lane < w && !*abort_flag) {
            if (C16)
                C16[static_cast<long>(r) * ldc + slice0 + lane] = f32_to_bf16(relu_if(acc, relu));
            else
                crow[lane] = acc;
        }
        if (tid == 0) {
            for (int s = 0; s < kStages; ++s) {
                asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(full + s)));
                asm volatile("mbarrier.inval.shared::cta.b64 [%0];" ::"r"(smem_u32(empty + s)));
            }
        }
        __syncthreads();  // shared memory and barriers are reused by the next unit
    }

    // the last CTA out resets the list counter and the done counter for the next call
    __syncthreads();
    if (tid == 0) {
        __threadfence();
        const unsigned total = gridDim.x;
        if (atomicAdd(counters + 1, 1u) == total - 1) {
            counters[0] = 0;
            counters[1] = 0;
            __threadfence();
        }
    }
}

template <typename T, int GB>
as_status launch(as_ctx *ctx, const SpmmArgs &a, const int *list, cudaStream_t s) {
    auto k = spmm_long<T, GB>;
    static bool attr_set[64] = {};
    const int dev = ctx->device;
    if (dev < 0 || dev >= 64) return fail(AS_ERR_INVALID_VALUE, "spmm long rows: device index");
    if (!attr_set[dev]) {
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             kSmemBytes);
        if (e != cudaSuccess) return check_cuda(e, "spmm long rows: shared memory attribute");
        attr_set[dev] = true;
    }
    // two CTAs per multiprocessor (one wave), striding over the (row, slice) units
    const long max_units = static_cast<long>(a.M) * ceil_div(a.N, kSliceBytes / static_cast<int>(sizeof(T)));
    dim3 grid(static_cast<unsigned>(std::max(1L, std::min(max_units, 2L * ctx->sms))));
    // programmatic dependent launch (outside stream capture): the CTAs are scheduled while
    // the row-split kernel drains, hiding this launch when there are no long rows
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(s, &cap);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = dim3(kThreads);
    cfg.dynamicSmemBytes = kSmemBytes;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = cap == cudaStreamCaptureStatusNone ? 1 : 0;
    cudaError_t e = cudaLaunchKernelEx(&cfg, k, a.M, a.K, a.N, a.nnz, a.rowptr, a.colind,
                                       static_cast<const T *>(a.val), static_cast<const T *>(a.B),
                                       a.ldb, a.C, a.ldc, a.beta, a.status, list, ctx->d_long,
                                       a.C16, a.relu, ctx->spin_limit);
    ctx->launches++;
    return check_cuda(e != cudaSuccess ? e : cudaGetLastError(), "spmm long rows launch");
}

}  // namespace

int spmm_long_granule(int dtype, int N, long ldb, const void *B) {
    const int esz = dtype == 0 ? 4 : 2;
    const uintptr_t pb = reinterpret_cast<uintptr_t>(B);
    if (ceil_div(N, kSliceBytes / esz) > 65535) return 0;
    if ((static_cast<long>(N) * esz) % 16 == 0 && (ldb * esz) % 16 == 0 && pb % 16 == 0) return 16;
    if ((static_cast<long>(N) * esz) % 4 == 0 && (ldb * esz) % 4 == 0 && pb % 4 == 0) return 4;
    return 0;
}

as_status spmm_long_launch(as_ctx *ctx, int dtype, int granule, const SpmmArgs &a,
                           const int *list, cudaStream_t s) {
    if (dtype == 0)
        return granule == 16 ? launch<float, 16>(ctx, a, list, s) : launch<float, 4>(ctx, a, list, s);
    return granule == 16 ? launch<uint16_t, 16>(ctx, a, list, s) : launch<uint16_t, 4>(ctx, a, list, s);
}

}  // namespace as
