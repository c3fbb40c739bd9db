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
// chains: a CTA takes one (long row, 64-byte column slice) at a time; all 256 threads copy B
// segments
// of upcoming entries into a shared-memory ring with cp.async (kStages stages of kStage
// entries in flight), and the slice's columns -- one per consumer thread -- run their chains
// out of shared memory. Column indices and values are staged a chunk of kChunk entries ahead
// in registers (plain coalesced loads) and parked in shared memory half a chunk later.
//
// The list counter and a CTA-done counter live in the context's device words; the last CTA
// to finish resets both, so the next call starts from zero without a memset.
#include <algorithm>

#include "common.cuh"
#include "internal.h"

namespace as {
namespace {

constexpr int kThreads = 256;
constexpr int kSliceBytes = 64;   // B bytes per entry per stage (16 fp32 / 32 bf16 columns)
constexpr int kStage = 64;        // entries per pipeline stage
constexpr int kStages = 12;       // stages in the B ring: 704 entries in flight cover the
                                  // gather latency at the chain's ~4 cycles per entry
constexpr int kChunk = 2048;      // entries per (colind, val) chunk; a multiple of kStage
constexpr int kChunkPerThread = kChunk / kThreads;
constexpr int kSmemBytes = kStages * kStage * kSliceBytes + 2 * kChunk * 8;
// the next chunk's (colind, val) reach shared memory half a chunk in, before the B lookahead
// of kStages - 1 stages first needs them
static_assert(kStages - 1 < kChunk / kStage / 2, "B lookahead must not outrun the chunk staging");

__device__ __forceinline__ float to_f32(float v) { return v; }
__device__ __forceinline__ float to_f32(uint16_t v) { return bf16_to_f32(v); }

template <int GB>
__device__ __forceinline__ void cp_async(void *smem, const void *gmem) {
    const unsigned s = static_cast<unsigned>(__cvta_generic_to_shared(smem));
    if constexpr (GB == 16)
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(s), "l"(gmem) : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(s), "l"(gmem) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
template <int N>
__device__ __forceinline__ void cp_async_wait() {
    asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// T: storage type of val and B (float or uint16_t = bf16); GB: cp.async size in bytes.
template <typename T, int GB>
__global__ void __launch_bounds__(kThreads)
spmm_long(int M, int K, int N, int nnz, const int *__restrict__ rowptr,
          const int *__restrict__ colind, const T *__restrict__ val, const T *__restrict__ B,
          long ldb, float *__restrict__ C, long ldc, float beta, unsigned *status,
          const int *__restrict__ list, unsigned *counters, uint16_t *__restrict__ C16,
          bool relu) {
    constexpr int W = kSliceBytes / static_cast<int>(sizeof(T));  // columns per slice
    extern __shared__ __align__(16) unsigned char smem[];
    unsigned char *ring = smem;  // [kStages][kStage][kSliceBytes]
    int *kbuf = reinterpret_cast<int *>(smem + kStages * kStage * kSliceBytes);  // [2][kChunk]
    float *vbuf = reinterpret_cast<float *>(kbuf + 2 * kChunk);                  // [2][kChunk]

    // launched as a programmatic dependent of the row-split kernel: wait for it to finish
    // (and its list writes to be visible) before reading the list
    asm volatile("griddepcontrol.wait;\n" ::: "memory");
    const int tid = threadIdx.x;
    const int n_long = static_cast<int>(
        min(*reinterpret_cast<volatile unsigned *>(counters), static_cast<unsigned>(M)));
    const int n_slices = static_cast<int>(ceil_div(N, W));
    const long units = static_cast<long>(n_long) * n_slices;

    // work units (long row, column slice), the slices of one row on consecutive CTAs
    for (long u = blockIdx.x; u < units; u += gridDim.x) {
        const int item = static_cast<int>(u / n_slices);
        const int slice0 = static_cast<int>(u - static_cast<long>(item) * n_slices) * W;
        const int w = min(W, N - slice0);                  // columns of this slice
        const int seg = w * static_cast<int>(sizeof(T));   // bytes of B per entry in this slice
        const int pieces = seg / GB;                       // cp.async pieces per entry
        const int r = list[item];
        if (r < 0 || r >= M) continue;
        int lo, hi;
        row_range(rowptr, r, nnz, status, lo, hi);
        const int L = hi - lo;
        const int n_stages = static_cast<int>(ceil_div(L, kStage));
        const int n_chunks = static_cast<int>(ceil_div(L, kChunk));

        // chunk 0 of (colind, val), straight into shared memory
        for (int i = tid; i < kChunk; i += kThreads) {
            int k = -1;
            float v = 0.0f;
            if (i < L) {
                k = ld_stream(colind + lo + i);
                v = to_f32(ld_stream(val + lo + i));
                if (static_cast<unsigned>(k) >= static_cast<unsigned>(K)) {
                    flag(status, kFlagBadColind);
                    k = -1;
                    v = 0.0f;
                }
            }
            kbuf[i] = k;
            vbuf[i] = v;
        }
        __syncthreads();

        // B segments of stage st into ring slot st % kStages. Warp w copies entries 8w..8w+7 of
        // the stage; lane l takes piece l % P of entry l / P (P pieces per full slice), so a
        // full warp instruction moves 512 bytes (a copy instruction costs the same issue slot
        // however few lanes it carries). Entries past the row are not copied (never read); a
        // flagged entry gets zeros (its value is 0 as well).
        const int warp = tid >> 5, lane = tid & 31;
        auto issue = [&](int st) {
            if (st < n_stages) {
                const int base = st * kStage;  // first entry of the stage, relative to lo
                const int *kb = kbuf + ((base / kChunk) & 1) * kChunk + base % kChunk;
                unsigned char *dst = ring + (st % kStages) * kStage * kSliceBytes;
                constexpr int P = kSliceBytes / GB;           // pieces of a full slice (4 or 16)
                constexpr int kPerWarp = kStage / (kThreads / 32);
#pragma unroll
                for (int t = 0; t < kPerWarp * P / 32; ++t) {
                    const int p = lane + 32 * t;
                    const int j = warp * kPerWarp + p / P, q = p % P;
                    if (q >= pieces || base + j >= L) continue;
                    const int k = kb[j];
                    unsigned char *d = dst + j * kSliceBytes + q * GB;
                    if (k >= 0) {
                        const unsigned char *src = reinterpret_cast<const unsigned char *>(
                            B + static_cast<long>(k) * ldb + slice0);
                        cp_async<GB>(d, src + q * GB);
                    } else if constexpr (GB == 16) {
                        *reinterpret_cast<uint4 *>(d) = make_uint4(0, 0, 0, 0);
                    } else {
                        *reinterpret_cast<unsigned *>(d) = 0u;
                    }
                }
            }
            cp_async_commit();  // one group per stage, empty or not, to keep the counting uniform
        };

        float acc = 0.0f;
        float *crow = C + static_cast<long>(r) * ldc + slice0;
        if (tid < w && beta != 0.0f) acc = crow[tid] * beta;

        for (int st = 0; st < kStages - 1; ++st) issue(st);

        int kreg[kChunkPerThread];
        float vreg[kChunkPerThread];
        for (int st = 0; st < n_stages; ++st) {
            const int c = st / (kChunk / kStage), sc = st % (kChunk / kStage);
            // stage the next chunk: registers at its start, shared memory at its middle
            if (sc == 0 && c + 1 < n_chunks) {
#pragma unroll
                for (int i = 0; i < kChunkPerThread; ++i) {
                    const int e = (c + 1) * kChunk + i * kThreads + tid;
                    kreg[i] = -1;
                    vreg[i] = 0.0f;
                    if (e < L) {
                        kreg[i] = ld_stream(colind + lo + e);
                        vreg[i] = to_f32(ld_stream(val + lo + e));
                    }
                }
            }
            if (sc == kChunk / kStage / 2 && c + 1 < n_chunks) {
                int *kd = kbuf + ((c + 1) & 1) * kChunk;
                float *vd = vbuf + ((c + 1) & 1) * kChunk;
#pragma unroll
                for (int i = 0; i < kChunkPerThread; ++i) {
                    int k = kreg[i];
                    float v = vreg[i];
                    if (k != -1 && static_cast<unsigned>(k) >= static_cast<unsigned>(K)) {
                        flag(status, kFlagBadColind);
                        k = -1;
                        v = 0.0f;
                    }
                    kd[i * kThreads + tid] = k;
                    vd[i * kThreads + tid] = v;
                }
            }
            __syncthreads();  // slot (st - 1) % kStages is free; staged (colind, val) visible
            issue(st + kStages - 1);
            cp_async_wait<kStages - 1>();  // stage st has landed (this thread's copies)
            __syncthreads();               // ... and every thread's
            if (tid < w) {
                const int base = st * kStage;
                const int n = min(kStage, L - base);
                const float *vs = vbuf + ((base / kChunk) & 1) * kChunk + base % kChunk;
                const T *bs = reinterpret_cast<const T *>(ring + (st % kStages) * kStage * kSliceBytes) + tid;
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
            }
        }
        cp_async_wait<0>();
        if (tid < w) {
            if (C16)
                C16[static_cast<long>(r) * ldc + slice0 + tid] = f32_to_bf16(relu_if(acc, relu));
            else
                crow[tid] = acc;
        }
        __syncthreads();  // shared memory is reused by the next row
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
                                       a.C16, a.relu);
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
