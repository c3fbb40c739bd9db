// Long rows of the row-split SpMM (sm_103a), bit-identical to rowBaseSpmm3 (SDMM.cpp:90-114).
//
// A row-split group walks its row's entries one after another, so one row with 10^5 entries
// (a hub of a power-law graph) keeps a single group busy long after the rest of the grid has
// finished. The row-split kernels therefore leave every row longer than a threshold to this
// kernel: they append the row number to a list (one atomic per long row) and skip it; this
// kernel, launched right after on the same stream, takes the listed rows. Rows longer than
// kHugeRow entries are listed from the other end of the list and taken first, so the longest
// chains start at once instead of behind shorter rows.
//
// The same kernel takes the long rows of the other row-oriented SpMMs, with their own chain
// step (OP below): the reduce aggregations (spmm_reduce.cu), the 1x4-blocked layout
// (spmm_vcsr4.cu) and the row-pair layout (spmm_rowpair.cu: a listed pair gives a unit per
// row, whose chain runs over the entries a per-stage include mask keeps).
//
// Each output element is still one chain over the row's entries in CSR order (the order
// cannot be split without changing the bits), so the speed comes from feeding the chains. A
// CTA takes one (long row, 64-column slice) at a time; its warps split by role:
//  - warp 0 is the consumer: lane l runs the chains of columns 2l and 2l+1 of the slice out of
//    shared memory, stage after stage (kStage entries per stage), reading each entry's two B
//    values with one 64-bit (fp32) or 32-bit (bf16) load and the entry's value from the
//    stage's value slot. It waits for a stage on the slot's `full` flag (an acquire load of a
//    shared word) and frees the slot by a release store to its `empty` flag;
//  - eight producer warps take the stages in turn (warp p owns stages p, p + 8, ..., all in
//    slot p). For its stage a warp waits for the slot's `empty` flag, stores the entries'
//    values (loaded into registers one turn earlier) into the value slot, and copies each
//    entry's B segment into the ring slot with cp.async, eight lanes per entry; the entries'
//    column indices, also loaded one turn earlier, reach those lanes by shuffle. It then waits
//    for its own copies (cp.async.wait_group 0; its next stage is a whole turn away) and
//    lane 0 publishes the stage with a release store to the slot's `full` flag after
//    __syncwarp.
// The consumer warp sits alone on its SM sub-partition (warps 4 and 8 are idle): the chains
// issue one FMA every few cycles and lose a large share of that rate when two busy producer
// warps share its scheduler.
//
// Every wait is bounded; a wait that gives up sets the timeout flag and an abort flag that makes
// the other role leave too. No copy is ever in flight when a warp leaves (a stage is published
// only after its copies landed); a row whose wait gave up is left unwritten. A malformed column
// index is flagged and its entry gets a zero segment (nothing is read for it).
//
// The list counters and a CTA-done counter live in the context's device words; the last CTA
// to finish resets them, so the next call starts from zero without a memset.
#include <algorithm>

#include "common.cuh"
#include "internal.h"

namespace as {
namespace {

constexpr int kCols = 64;                   // columns per slice (two per consumer lane)
constexpr int kStage = 64;                  // entries per pipeline stage
constexpr int kStages = 8;                  // ring slots
constexpr int kProducers = 8;               // producer warps, one stage each in turn
constexpr int kWarps = 12;                  // warp 0 consumer; 4, 8 and 11 idle
constexpr int kThreads = 32 * kWarps;
constexpr unsigned kSpinLimit = 1u << 22;   // polls of a bounded wait (a few seconds at most)
static_assert(kStages % kProducers == 0, "a slot is always refilled by the same producer warp");
static_assert(kStage == 64, "each producer lane holds two entries' index and value");

template <typename T>
struct Layout {
    static constexpr int kSlice = kCols * static_cast<int>(sizeof(T));  // B bytes per entry
    static constexpr int kRing = kStages * kStage * kSlice;
    static constexpr int kVals = kStages * kStage * 4;                  // values as fp32
    static constexpr int kMasks = kStages * 8;  // row-pair mode: the stage's include bits
    static constexpr int kBytes = kRing + kVals + kMasks + 2 * kStages * 4 + 16;
};

// producer index (0-7) of a warp, or -1 for the consumer and the idle warps
__device__ __forceinline__ int producer_of(int warp) {
    return (warp & 3) != 0 && warp <= 10 ? warp - 1 - (warp >> 2) : -1;
}

__device__ __forceinline__ float to_f32(float v) { return v; }
__device__ __forceinline__ float to_f32(uint16_t v) { return bf16_to_f32(v); }

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ int ld_acquire(uint32_t a) {
    int v;
    asm volatile("ld.acquire.cta.shared::cta.b32 %0, [%1];" : "=r"(v) : "r"(a) : "memory");
    return v;
}
__device__ __forceinline__ void st_release(uint32_t a, int v) {
    asm volatile("st.release.cta.shared::cta.b32 [%0], %1;" ::"r"(a), "r"(v) : "memory");
}
// Bounded wait until the flag at `a` reaches `target`; false when `limit` polls pass or the
// other role has given up. `nap` > 0 sleeps that many ns between polls (producers, which are
// ahead and must not take issue slots from the consumer).
__device__ __forceinline__ bool wait_seq(uint32_t a, int target, unsigned limit,
                                         const volatile int *abort_flag, unsigned nap = 0) {
    for (unsigned i = 0; i < limit; ++i) {
        if (ld_acquire(a) >= target) return true;
        if (*abort_flag) return false;
        if (nap) __nanosleep(nap);
    }
    return false;
}

// Two consecutive B columns of one entry from shared memory, as fp32.
__device__ __forceinline__ float2 lds_pair(uint32_t a, float) {
    float2 r;
    asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];" : "=f"(r.x), "=f"(r.y) : "r"(a));
    return r;
}
__device__ __forceinline__ float2 lds_pair(uint32_t a, uint16_t) {
    uint32_t u;
    asm volatile("ld.shared.u32 %0, [%1];" : "=r"(u) : "r"(a));
    return make_float2(__uint_as_float(u << 16), __uint_as_float(u & 0xffff0000u));
}
__device__ __forceinline__ float4 lds_vals(uint32_t a) {
    float4 r;
    asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];"
                 : "=f"(r.x), "=f"(r.y), "=f"(r.z), "=f"(r.w)
                 : "r"(a));
    return r;
}

template <int GB>
__device__ __forceinline__ void cp_async_zfill(uint32_t dst, const void *gmem, int src_bytes) {
    if constexpr (GB == 16)
        asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(gmem),
                     "r"(src_bytes)
                     : "memory");
    else
        asm volatile("cp.async.ca.shared.global [%0], [%1], 4, %2;\n" ::"r"(dst), "l"(gmem),
                     "r"(src_bytes)
                     : "memory");
}

// The per-entry step of a chain: OP 0 the SpMM's fused multiply-add (acc = fma(b, v, acc)),
// 1 the unweighted copy-sum (acc + b), 2 max from -inf (fmaxf(acc, v * b)), 3 the DGL max
// (acc > v * b ? acc : v * b), 4 the fused multiply-add skipping zero values (the 1x4-blocked
// layout's empty slots), 5 the fused multiply-add over the entries a row-pair unit includes
// (the include mask is applied by the consumer); the max forms use b alone when the row has
// no values.
template <int OP>
__device__ __forceinline__ float step(float acc, float b, float v, bool weighted) {
    if constexpr (OP == 0) return fmaf(b, v, acc);
    if constexpr (OP == 1) return __fadd_rn(acc, b);
    if constexpr (OP == 4) return v != 0.0f ? fmaf(b, v, acc) : acc;
    if constexpr (OP == 5) return fmaf(b, v, acc);
    const float x = weighted ? __fmul_rn(v, b) : b;
    if constexpr (OP == 2) return fmaxf(acc, x);
    return acc > x ? acc : x;
}

// T: storage type of val and B (float or uint16_t = bf16); GB: cp.async size in bytes; OP: the
// chain step above (the steps other than 0 take fp32 only). pair_flag: the row-pair layout's
// flags (OP 5 only).
template <typename T, int GB, int OP>
__global__ void __launch_bounds__(kThreads, 1)
spmm_long(int M, int K, int N, int nnz, const int *__restrict__ rowptr,
          const int *__restrict__ colind, const T *__restrict__ val, const T *__restrict__ B,
          long ldb, float *__restrict__ C, long ldc, float beta, unsigned *status,
          const int *__restrict__ list, unsigned *counters, uint16_t *__restrict__ C16,
          bool relu, unsigned spin_limit, const uint8_t *__restrict__ pair_flag) {
    using Lay = Layout<T>;
    constexpr int kSlice = Lay::kSlice;
    constexpr int kEsz = static_cast<int>(sizeof(T));
    constexpr unsigned kAll = 0xffffffffu;
    extern __shared__ __align__(1024) unsigned char smem[];
    unsigned char *ring = smem;                                  // [kStages][kStage][kSlice]
    float *vals = reinterpret_cast<float *>(smem + Lay::kRing);  // [kStages][kStage]
    unsigned long long *masks = reinterpret_cast<unsigned long long *>(smem + Lay::kRing + Lay::kVals);
    int *full_seq = reinterpret_cast<int *>(smem + Lay::kRing + Lay::kVals + Lay::kMasks);  // stage filled + 1
    int *empty_seq = full_seq + kStages;                                       // stage consumed + 1
    volatile int *abort_flag = reinterpret_cast<volatile int *>(empty_seq + kStages);

    // launched as a programmatic dependent of the row-split kernel: wait for it to finish
    // (and its list writes to be visible) before reading the list
    asm volatile("griddepcontrol.wait;\n" ::: "memory");
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const unsigned cap = static_cast<unsigned>(M);
    const int n_long = static_cast<int>(min(*reinterpret_cast<volatile unsigned *>(counters), cap));
    const int n_huge =
        static_cast<int>(min(*reinterpret_cast<volatile unsigned *>(counters + 2), cap));
    // row-pair mode: a listed item is a pair's even row; each pair gives two rows' units
    constexpr int kRowsPerItem = OP == 5 ? 2 : 1;
    const int n_slices = static_cast<int>(ceil_div(N, kCols)) * kRowsPerItem;
    const long units_huge = static_cast<long>(n_huge) * n_slices;
    const long units = units_huge + static_cast<long>(n_long) * n_slices;
    const int pw = producer_of(warp);

    // work units (row, column slice): the huge rows (listed from the end) first, the slices of
    // one row on consecutive CTAs
    for (long u = blockIdx.x; u < units; u += gridDim.x) {
        const bool huge = u < units_huge;
        const long v = huge ? u : u - units_huge;
        const int item = static_cast<int>(v / n_slices);
        const int sub_unit = static_cast<int>(v - static_cast<long>(item) * n_slices);
        const int which = sub_unit % kRowsPerItem;   // row-pair mode: 0 the even row, 1 the odd
        const int slice0 = sub_unit / kRowsPerItem * kCols;
        const int w = min(kCols, N - slice0);        // columns of this slice
        const int pieces = w * kEsz / GB;            // copy pieces per entry
        const int r0 = huge ? list[M - 1 - item] : list[item];
        const int r = r0 + which;                    // the output row
        if (r0 < 0 || r >= M) continue;
        int lo, hi;
        row_range(rowptr, r0, nnz, status, lo, hi);
        // Row-pair mode: the even row chains over its segment's unflagged entries (all of them
        // when it has no partner); the odd row over the even segment's flagged entries, then
        // over its own segment (entries at positions L1.. map to [lo1, hi1)).
        int L1 = hi - lo, lo1 = 0, hi1 = 0;
        const bool partner = OP == 5 && r0 + 1 < M;
        if (OP == 5 && which == 1) row_range(rowptr, r0 + 1, nnz, status, lo1, hi1);
        const int L = L1 + (hi1 - lo1);
        const int n_stages = static_cast<int>(ceil_div(L, kStage));

        if (tid == 0) {
            for (int s = 0; s < kStages; ++s) {
                full_seq[s] = 0;
                empty_seq[s] = 0;
            }
            *abort_flag = 0;
        }
        __syncthreads();

        constexpr float kInit = OP == 2 ? -INFINITY : OP == 3 ? -10000.0f : 0.0f;
        const bool weighted = val != nullptr;
        float acc0 = kInit, acc1 = kInit;
        const int c0 = 2 * lane;  // this lane's first column within the slice
        float *crow = C + static_cast<long>(r) * ldc + slice0;  // r: this unit's output row
        if (warp == 0) {
            // ---- consumer: the chains of columns c0 and c0 + 1 ----
            if (beta != 0.0f) {
                if (c0 < w) acc0 = crow[c0] * beta;
                if (c0 + 1 < w) acc1 = crow[c0 + 1] * beta;
            }
            for (int s = 0; s < n_stages; ++s) {
                const int slot = s % kStages;
                const bool ok = __all_sync(kAll, wait_seq(smem_u32(full_seq + slot), s + 1,
                                                          spin_limit, abort_flag));
                if (!ok) {
                    if (lane == 0) {
                        flag(status, kFlagTimeout);
                        *abort_flag = 1;
                    }
                    break;
                }
                const int n = min(kStage, L - s * kStage);
                const uint32_t bs = smem_u32(ring + slot * kStage * kSlice) + c0 * kEsz;
                const uint32_t vs = smem_u32(vals + slot * kStage);
                // row-pair mode: entry j of the stage counts when bit j is set
                const unsigned long long mask = OP == 5 ? masks[slot] : ~0ull;
                auto st = [&](float acc, float b, float x, int j) {
                    if constexpr (OP == 5) return ((mask >> j) & 1ull) ? fmaf(b, x, acc) : acc;
                    return step<OP>(acc, b, x, weighted);
                };
                if (n == kStage) {
#pragma unroll
                    for (int q = 0; q < kStage; q += 16) {
                        float2 b[16];
                        float4 v[4];
#pragma unroll
                        for (int i = 0; i < 16; ++i) b[i] = lds_pair(bs + (q + i) * kSlice, T());
#pragma unroll
                        for (int i = 0; i < 4; ++i) v[i] = lds_vals(vs + (q + 4 * i) * 4);
#pragma unroll
                        for (int i = 0; i < 4; ++i) {
                            const int j = q + 4 * i;
                            acc0 = st(acc0, b[4 * i].x, v[i].x, j);
                            acc1 = st(acc1, b[4 * i].y, v[i].x, j);
                            acc0 = st(acc0, b[4 * i + 1].x, v[i].y, j + 1);
                            acc1 = st(acc1, b[4 * i + 1].y, v[i].y, j + 1);
                            acc0 = st(acc0, b[4 * i + 2].x, v[i].z, j + 2);
                            acc1 = st(acc1, b[4 * i + 2].y, v[i].z, j + 2);
                            acc0 = st(acc0, b[4 * i + 3].x, v[i].w, j + 3);
                            acc1 = st(acc1, b[4 * i + 3].y, v[i].w, j + 3);
                        }
                    }
                } else {
                    for (int j = 0; j < n; ++j) {
                        const float2 b = lds_pair(bs + j * kSlice, T());
                        const float x = vals[slot * kStage + j];
                        acc0 = st(acc0, b.x, x, j);
                        acc1 = st(acc1, b.y, x, j);
                    }
                }
                __syncwarp();
                if (lane == 0) st_release(smem_u32(empty_seq + slot), s + 1);
            }
        } else if (pw >= 0) {
            // ---- producer pw: stages pw, pw + kProducers, ... (all in slot pw % kStages) ----
            const int sub = lane >> 3, pl = lane & 7;  // entry of a group of four, lane in it
            // column index and value of this lane's entries (lane, lane + 32) of stage st
            // entry position e of the unit -> index in the arrays, and whether it counts
            // (row-pair mode; every entry counts otherwise)
            auto entry = [&](int e, int &idx, int &inc) {
                idx = lo + e;
                inc = 1;
                if constexpr (OP == 5) {
                    if (e >= L1) {
                        idx = lo1 + (e - L1);
                    } else if (partner) {
                        inc = (__ldg(pair_flag + idx) != 0) == (which == 1);
                    }
                }
            };
            auto load = [&](int st, int &k0, int &k1, float &x0, float &x1, int &f0, int &f1) {
                k0 = k1 = 0;
                x0 = x1 = 0.0f;
                f0 = f1 = 0;
                const int e0 = st * kStage + lane, e1 = e0 + 32;
                int i0, i1;
                if (st < n_stages && e0 < L) {
                    entry(e0, i0, f0);
                    k0 = ld_stream(colind + i0);
                    x0 = weighted ? to_f32(ld_stream(val + i0)) : 1.0f;
                }
                if (st < n_stages && e1 < L) {
                    entry(e1, i1, f1);
                    k1 = ld_stream(colind + i1);
                    x1 = weighted ? to_f32(ld_stream(val + i1)) : 1.0f;
                }
            };
            int k0, k1, f0, f1;
            float x0, x1;
            load(pw, k0, k1, x0, x1, f0, f1);
            for (int s = pw; s < n_stages; s += kProducers) {
                const int slot = s % kStages;
                if (s >= kStages) {  // the consumer is done with stage s - kStages
                    int ok = 1;
                    if (lane == 0)
                        ok = wait_seq(smem_u32(empty_seq + slot), s - kStages + 1, kSpinLimit,
                                      abort_flag, 64);
                    if (!__shfl_sync(kAll, ok, 0)) break;
                }
                int nk0, nk1, nf0, nf1;
                float nx0, nx1;
                load(s + kProducers, nk0, nk1, nx0, nx1, nf0, nf1);  // the next turn's, in flight meanwhile
                vals[slot * kStage + lane] = x0;
                vals[slot * kStage + lane + 32] = x1;
                if constexpr (OP == 5) {
                    const unsigned long long m =
                        __ballot_sync(kAll, f0) | (static_cast<unsigned long long>(__ballot_sync(kAll, f1)) << 32);
                    if (lane == 0) masks[slot] = m;
                }
                const uint32_t dst0 = smem_u32(ring + slot * kStage * kSlice);
#pragma unroll 4
                for (int g = 0; g < kStage / 4; ++g) {
                    const int j = 4 * g + sub;
                    int k = __shfl_sync(kAll, g < 8 ? k0 : k1, j & 31);
                    // OP 4: an empty slot (value 0) may point past K; only a filled one is bad.
                    // OP 5: an entry the unit leaves out is neither checked nor copied.
                    bool filled = true;
                    if constexpr (OP == 4) filled = __shfl_sync(kAll, g < 8 ? x0 : x1, j & 31) != 0.0f;
                    if constexpr (OP == 5) filled = __shfl_sync(kAll, g < 8 ? f0 : f1, j & 31) != 0;
                    if (s * kStage + j < L && (OP != 5 || filled)) {
                        const bool bad = static_cast<unsigned>(k) >= static_cast<unsigned>(K);
                        if (bad) {
                            if (filled) flag(status, kFlagBadColind);
                            k = 0;
                        }
                        const unsigned char *src = reinterpret_cast<const unsigned char *>(
                            B + static_cast<long>(k) * ldb + slice0);
                        const uint32_t dst = dst0 + j * kSlice;
#pragma unroll
                        for (int q = 0; q < kSlice / GB / 8; ++q) {
                            const int piece = pl + 8 * q;
                            if (piece < pieces)
                                cp_async_zfill<GB>(dst + piece * GB, src + piece * GB, bad ? 0 : GB);
                        }
                    }
                }
                // the slot is full once every lane's copies have landed
                asm volatile("cp.async.commit_group;\n" ::: "memory");
                asm volatile("cp.async.wait_group 0;\n" ::: "memory");
                __syncwarp();
                if (lane == 0) st_release(smem_u32(full_seq + slot), s + 1);
                k0 = nk0;
                k1 = nk1;
                x0 = nx0;
                x1 = nx1;
                f0 = nf0;
                f1 = nf1;
            }
            asm volatile("cp.async.wait_all;\n" ::: "memory");
            __syncwarp();
        }
        __syncthreads();
        if (warp == 0 && !*abort_flag) {
            if (C16) {
                uint16_t *orow = C16 + static_cast<long>(r) * ldc + slice0;
                if (c0 < w) orow[c0] = f32_to_bf16(relu_if(acc0, relu));
                if (c0 + 1 < w) orow[c0 + 1] = f32_to_bf16(relu_if(acc1, relu));
            } else {
                if (c0 < w) crow[c0] = acc0;
                if (c0 + 1 < w) crow[c0 + 1] = acc1;
            }
        }
        __syncthreads();  // shared memory and flags are reused by the next unit
    }

    // the last CTA out resets the list counters and the done counter for the next call
    __syncthreads();
    if (tid == 0) {
        __threadfence();
        const unsigned total = gridDim.x;
        if (atomicAdd(counters + 1, 1u) == total - 1) {
            counters[0] = 0;
            counters[1] = 0;
            counters[2] = 0;
            __threadfence();
        }
    }
}

template <typename T, int GB, int OP = 0>
as_status launch(as_ctx *ctx, const SpmmArgs &a, const int *list, cudaStream_t s,
                 const uint8_t *pair_flag = nullptr) {
    auto k = spmm_long<T, GB, OP>;
    constexpr int kBytes = Layout<T>::kBytes;
    static int per_sm[64] = {};  // resident CTAs per multiprocessor, per device
    const int dev = ctx->device;
    if (dev < 0 || dev >= 64) return fail(AS_ERR_INVALID_VALUE, "spmm long rows: device index");
    if (!per_sm[dev]) {
        cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, kBytes);
        if (e != cudaSuccess) return check_cuda(e, "spmm long rows: shared memory attribute");
        int n = 0;
        e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k, kThreads, kBytes);
        if (e != cudaSuccess) return check_cuda(e, "spmm long rows: occupancy");
        per_sm[dev] = std::max(1, n);
    }
    // one wave of CTAs striding over the (row, slice) units
    const long max_units = static_cast<long>(a.M) * ceil_div(a.N, kCols) * (OP == 5 ? 2 : 1);
    dim3 grid(static_cast<unsigned>(
        std::max(1L, std::min(max_units, static_cast<long>(per_sm[dev]) * ctx->sms))));
    // programmatic dependent launch (outside stream capture): the CTAs are scheduled while
    // the row-split kernel drains, hiding this launch when there are no long rows
    cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
    cudaStreamIsCapturing(s, &cap);
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = grid;
    cfg.blockDim = dim3(kThreads);
    cfg.dynamicSmemBytes = kBytes;
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    attr[0].val.programmaticStreamSerializationAllowed = 1;
    cfg.attrs = attr;
    cfg.numAttrs = cap == cudaStreamCaptureStatusNone ? 1 : 0;
    cudaError_t e = cudaLaunchKernelEx(&cfg, k, a.M, a.K, a.N, a.nnz, a.rowptr, a.colind,
                                       static_cast<const T *>(a.val), static_cast<const T *>(a.B),
                                       a.ldb, a.C, a.ldc, a.beta, a.status, list, ctx->d_long,
                                       a.C16, a.relu, ctx->spin_limit, pair_flag);
    ctx->launches++;
    return check_cuda(e != cudaSuccess ? e : cudaGetLastError(), "spmm long rows launch");
}

}  // namespace

int spmm_long_granule(int dtype, int N, long ldb, const void *B) {
    const int esz = dtype == 0 ? 4 : 2;
    const uintptr_t pb = reinterpret_cast<uintptr_t>(B);
    if ((static_cast<long>(N) * esz) % 16 == 0 && (ldb * esz) % 16 == 0 && pb % 16 == 0) return 16;
    if ((static_cast<long>(N) * esz) % 4 == 0 && (ldb * esz) % 4 == 0 && pb % 4 == 0) return 4;
    return 0;
}

as_status spmm_long_launch(as_ctx *ctx, int dtype, int granule, const SpmmArgs &a,
                           const int *list, cudaStream_t s, int op, const uint8_t *pair_flag) {
    if (op != 0) {  // the reductions and the 1x4-blocked layout: fp32
        if (dtype != 0) return fail(AS_ERR_UNSUPPORTED, "spmm long rows: this step takes fp32");
        switch (op) {
            case 1: return granule == 16 ? launch<float, 16, 1>(ctx, a, list, s) : launch<float, 4, 1>(ctx, a, list, s);
            case 2: return granule == 16 ? launch<float, 16, 2>(ctx, a, list, s) : launch<float, 4, 2>(ctx, a, list, s);
            case 3: return granule == 16 ? launch<float, 16, 3>(ctx, a, list, s) : launch<float, 4, 3>(ctx, a, list, s);
            case 4: return granule == 16 ? launch<float, 16, 4>(ctx, a, list, s) : launch<float, 4, 4>(ctx, a, list, s);
            case 5:
                if (!pair_flag) return fail(AS_ERR_INVALID_VALUE, "spmm long rows: row pairs need their flags");
                return granule == 16 ? launch<float, 16, 5>(ctx, a, list, s, pair_flag)
                                     : launch<float, 4, 5>(ctx, a, list, s, pair_flag);
        }
        return fail(AS_ERR_INVALID_VALUE, "spmm long rows: unknown reduction");
    }
    if (dtype == 0)
        return granule == 16 ? launch<float, 16>(ctx, a, list, s) : launch<float, 4>(ctx, a, list, s);
    return granule == 16 ? launch<uint16_t, 16>(ctx, a, list, s) : launch<uint16_t, 4>(ctx, a, list, s);
}

}  // namespace as
