// Tensor-core SDDMM on sm_103a: out[e] = s_e * <X[row(e)], Y[col(e)]> with split-bf16
// operands, FP32 accumulation in tensor memory.
//
// 1. split:  X -> Xhi, Xlo and Y -> Yhi, Ylo in bf16 (hi = bf16(x), lo = bf16(x - hi)),
//    K zero-padded to a multiple of 64, so that x*y ~= hi*hi + hi*lo + lo*hi (the dropped
//    lo*lo term and the rounding of lo are ~2^-16 relative).
// 2. tiles:  one CTA per 128 x BN tile of X * Y^T that holds at least one pattern entry
//    (tiles without entries exit before touching tensor memory). Warp roles:
//      warp 0  TMA producer: per 64-wide K block, four 2-D tiled bulk copies (Xhi, Xlo of the
//              tile's 128 rows; Yhi, Ylo of its BN rows) into 128B-swizzled shared memory,
//              completing on the stage's mbarrier;
//      warp 1  allocates BN columns of tensor memory; one lane issues, per K block, 12
//              tcgen05.mma.kind::f16 (M=128, N=BN, K=16; bf16 x bf16 -> f32) -- Xhi.Yhi,
//              Xhi.Ylo, Xlo.Yhi for four 16-wide K steps -- and tcgen05.commit frees the
//              stage; a final commit marks the accumulator ready;
//      warps 2-5 epilogue: each thread owns one tile row (its TMEM lane), reads the
//              accumulator 32 columns at a time (tcgen05.ld 32x32b.x32), stages them in its
//              own shared-memory row and writes the sampled entries of that row in CSR order
//              (a row's entries inside the tile are contiguous because columns ascend).
//    Every mbarrier wait is bounded; a timeout sets the status word, makes the other roles
//    leave, and the CTA still frees its tensor memory.
// Requires columns ascending within each row (checked on the device; a violation sets the
// status word).
#include <cuda.h>
#include <cudaTypedefs.h>

#include "common.cuh"
#include "internal.h"

namespace as {
namespace {

constexpr int kBM = 128;
constexpr int kBK = 64;  // bf16 elements per K block = 128 bytes = one swizzle row
constexpr int kThreads = 192;
constexpr unsigned kSpinLimit = 1u << 22;  // a few seconds of try_wait at most

__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t parity) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

// Bounded wait; false on timeout or when another role gave up.
__device__ __forceinline__ bool mbar_wait(uint64_t *bar, uint32_t parity, volatile int *abort_flag,
                                          unsigned *status) {
    for (unsigned i = 0; i < kSpinLimit; ++i) {
        if (mbar_try_wait(bar, parity)) return true;
        if ((i & 63) == 63 && *abort_flag) return false;
    }
    *abort_flag = 1;
    flag(status, kFlagTimeout);
    return false;
}

__device__ __forceinline__ void tma_load_2d(void *dst, const CUtensorMap *map, uint64_t *bar, int x,
                                            int y) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%3, %4}], [%2];" ::
            "r"(smem_u32(dst)),
        "l"(map), "r"(smem_u32(bar)), "r"(x), "r"(y)
        : "memory");
}

__device__ __forceinline__ void tc_fence_before() {
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
}
__device__ __forceinline__ void tc_fence_after() {
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
}

// Shared-memory matrix descriptor: K-major operand, 128-byte swizzle, 8-row groups 1024 B
// apart (SBO), descriptor version 1, base offset 0 (tiles are 1024-byte aligned).
__device__ __forceinline__ uint64_t desc_sw128(uint32_t saddr) {
    uint64_t d = 0;
    d |= static_cast<uint64_t>((saddr >> 4) & 0x3FFFu);
    d |= static_cast<uint64_t>(1) << 16;             // LBO (unused for swizzled K-major)
    d |= static_cast<uint64_t>(1024 >> 4) << 32;     // SBO
    d |= static_cast<uint64_t>(1) << 46;             // version
    d |= static_cast<uint64_t>(2) << 61;             // 128B swizzle
    return d;
}

// Instruction descriptor, kind::f16: D f32, A and B bf16, both K-major, M x N.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | (static_cast<uint32_t>(N >> 3) << 17) |
           (static_cast<uint32_t>(M >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t dt, uint64_t a, uint64_t b, uint32_t idesc,
                                         uint32_t acc) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(dt),
        "l"(a), "l"(b), "r"(idesc), "r"(acc));
}

__device__ __forceinline__ void mma_commit(uint64_t *bar) {
    asm volatile(
        "tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(
            smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&r)[32]) {
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 "
        "{%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, %15, "
        "%16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]),
          "=r"(r[7]), "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]),
          "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]), "=r"(r[17]), "=r"(r[18]),
          "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
          "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]),
          "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
}

template <int BN>
struct Smem {
    static constexpr int kStages = BN >= 256 ? 2 : 3;
    static constexpr int kTileA = kBM * kBK * 2;  // bytes of one A (X) tile
    static constexpr int kTileB = BN * kBK * 2;   // bytes of one B (Y) tile
    static constexpr int kStage = 2 * kTileA + 2 * kTileB;
    static constexpr int kStageRow = 33;          // floats per staged epilogue row
    static constexpr int kStaging = 128 * kStageRow * 4;
    static constexpr int kBytes = 1024 /*alignment slack*/ + kStages * kStage + kStaging + 256;
};

template <int BN>
__global__ void __launch_bounds__(kThreads, 1)
sddmm_tc_kernel(const __grid_constant__ CUtensorMap tmXhi, const __grid_constant__ CUtensorMap tmXlo,
                const __grid_constant__ CUtensorMap tmYhi, const __grid_constant__ CUtensorMap tmYlo,
                int M, int N, int nkb, int nnz, const int *__restrict__ rowptr,
                const int *__restrict__ colind, const float *__restrict__ aval,
                float *__restrict__ out, unsigned *status) {
    using L = Smem<BN>;
    extern __shared__ uint8_t smem_raw[];
    const uint32_t raw = smem_u32(smem_raw);
    uint8_t *smem = smem_raw + ((1024 - (raw & 1023)) & 1023);
    uint8_t *stages = smem;
    float *staging = reinterpret_cast<float *>(smem + L::kStages * L::kStage);
    uint8_t *tail = smem + L::kStages * L::kStage + L::kStaging;
    uint64_t *full = reinterpret_cast<uint64_t *>(tail);
    uint64_t *empty = full + L::kStages;
    uint64_t *accum = empty + L::kStages;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(accum + 1);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int r0 = blockIdx.y * kBM, c0 = blockIdx.x * BN;

    // Epilogue threads find where their row's entries of this tile start.
    int row = -1, e = 0, hi = 0;
    bool mine = false;
    if (warp >= 2) {
        row = r0 + 32 * (warp & 3) + lane;
        if (row < M) {
            int lo;
            row_range(rowptr, row, nnz, status, lo, hi);
            int a = lo, b = hi;  // lower_bound of c0 in colind[lo, hi)
            while (a < b) {
                const int m = (a + b) >> 1;
                if (__ldg(colind + m) < c0)
                    a = m + 1;
                else
                    b = m;
            }
            e = a;
            mine = e < hi && __ldg(colind + e) < c0 + BN;
        }
    }
    if (!__syncthreads_or(mine)) return;  // no pattern entry in this tile

    if (threadIdx.x == 0) {
        for (int s = 0; s < L::kStages; ++s) {
            mbar_init(&full[s], 1);
            mbar_init(&empty[s], 1);
        }
        mbar_init(accum, 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(tmem_slot)),
                     "r"(BN)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) {
            int issued = 0;
            for (int kb = 0; kb < nkb; ++kb) {
                const int s = kb % L::kStages;
                const int round = kb / L::kStages;
                if (round > 0 && !mbar_wait(&empty[s], (round - 1) & 1, abort_flag, status)) break;
                uint8_t *st = stages + s * L::kStage;
                mbar_expect_tx(&full[s], L::kStage);
                const int k0 = kb * kBK;
                tma_load_2d(st, &tmXhi, &full[s], k0, r0);
                tma_load_2d(st + L::kTileA, &tmXlo, &full[s], k0, r0);
                tma_load_2d(st + 2 * L::kTileA, &tmYhi, &full[s], k0, c0);
                tma_load_2d(st + 2 * L::kTileA + L::kTileB, &tmYlo, &full[s], k0, c0);
                issued = kb + 1;
            }
            // Leave only after the last copies landed (they complete even if no MMA reads
            // them), so no bulk copy targets this CTA's shared memory after it exits.
            for (int kb = issued - L::kStages > 0 ? issued - L::kStages : 0; kb < issued; ++kb) {
                const int s = kb % L::kStages;
                for (unsigned i = 0; i < kSpinLimit; ++i)
                    if (mbar_try_wait(&full[s], (kb / L::kStages) & 1)) break;
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {
            constexpr uint32_t idesc = idesc_bf16(kBM, BN);
            bool ok = true;
            for (int kb = 0; kb < nkb && ok; ++kb) {
                const int s = kb % L::kStages;
                const int round = kb / L::kStages;
                if (!mbar_wait(&full[s], round & 1, abort_flag, status)) {
                    ok = false;
                    break;
                }
                tc_fence_after();
                const uint32_t base = smem_u32(stages + s * L::kStage);
                const uint64_t ahi = desc_sw128(base), alo = desc_sw128(base + L::kTileA);
                const uint64_t bhi = desc_sw128(base + 2 * L::kTileA);
                const uint64_t blo = desc_sw128(base + 2 * L::kTileA + L::kTileB);
#pragma unroll
                for (int j = 0; j < kBK / 16; ++j) {
                    const uint64_t adv = static_cast<uint64_t>(j * 32 >> 4);  // 32 bytes per K step
                    mma_bf16(tmem, ahi + adv, bhi + adv, idesc, (kb | j) != 0);
                    mma_bf16(tmem, ahi + adv, blo + adv, idesc, 1u);
                    mma_bf16(tmem, alo + adv, bhi + adv, idesc, 1u);
                }
                mma_commit(&empty[s]);
            }
            if (ok) mma_commit(accum);
        }
    } else {
        // epilogue: 4 warps, thread = tile row (TMEM lane 32*(warp%4) + lane)
        const bool ready = __all_sync(0xffffffffu, mbar_wait(accum, 0, abort_flag, status));
        tc_fence_after();
        float *my = staging + (32 * (warp & 3) + lane) * L::kStageRow;
        const uint32_t lane_addr = tmem + (static_cast<uint32_t>(32 * (warp & 3)) << 16);
        if (ready) {
            int prev = -1;
#pragma unroll 1
            for (int j = 0; j < BN / 32; ++j) {
                uint32_t v[32];
                tmem_ld32(lane_addr + 32 * j, v);
                if (!mine) continue;
#pragma unroll
                for (int t = 0; t < 32; ++t) my[t] = __uint_as_float(v[t]);
                const int cend = c0 + 32 * (j + 1);
                while (e < hi) {
                    const int c = __ldg(colind + e);
                    if (c >= cend) break;
                    if (c <= prev || c >= N) {
                        flag(status, kFlagBadColind);
                        out[e] = 0.0f;
                    } else {
                        const float d = my[c - (cend - 32)];
                        out[e] = aval ? __ldg(aval + e) * d : d;
                    }
                    prev = c;
                    ++e;
                }
            }
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(BN)
                     : "memory");
    }
}

// ---- persistent form --------------------------------------------------------------------
// One CTA per SM walks the tiles (grouped order: 16 row tiles at a time across all column
// tiles, for L2 reuse of the operand panels) and skips tiles without pattern entries (a
// pre-pass marks them). Two accumulators in tensor memory (2 x BN columns): the epilogue
// warps drain tile j from one while the MMA thread accumulates tile j+1 in the other. BK is
// the K width of a pipeline stage: 64 (128-byte swizzle, 2 stages of 96 KB) or 32 (64-byte
// swizzle, 4 stages of 48 KB).
template <int BN, int BK>
struct PSmem {
    static constexpr int kTileA = kBM * BK * 2;
    static constexpr int kTileB = BN * BK * 2;
    static constexpr int kStage = 2 * kTileA + 2 * kTileB;
    static constexpr int kStages = BK == 32 ? 4 : 2;
    static constexpr int kStaging = 128 * 33 * 4;
    static constexpr int kBytes = 1024 + kStages * kStage + kStaging + 512;
    static constexpr int kLayout = BK == 32 ? 4 : 2;  // descriptor swizzle: 64B / 128B
    static constexpr int kSBO = 8 * BK * 2;           // bytes between 8-row core groups
};
constexpr int kGroupM = 16;

__device__ __forceinline__ uint64_t desc_kmajor(uint32_t saddr, int sbo, int layout) {
    uint64_t d = 0;
    d |= static_cast<uint64_t>((saddr >> 4) & 0x3FFFu);
    d |= static_cast<uint64_t>(1) << 16;
    d |= static_cast<uint64_t>((sbo >> 4) & 0x3FFF) << 32;
    d |= static_cast<uint64_t>(1) << 46;
    d |= static_cast<uint64_t>(layout) << 61;
    return d;
}

__device__ __forceinline__ void tile_coords(int t, int tiles_m, int tiles_n, int &tm, int &tn) {
    const int per = kGroupM * tiles_n;
    const int g = t / per, r = t - g * per;
    const int rows = min(kGroupM, tiles_m - g * kGroupM);
    tm = g * kGroupM + r % rows;
    tn = r / rows;
}

template <int BN, int BK>
__global__ void __launch_bounds__(kThreads, 1)
sddmm_tc_persistent(const __grid_constant__ CUtensorMap tmXhi, const __grid_constant__ CUtensorMap tmXlo,
                    const __grid_constant__ CUtensorMap tmYhi, const __grid_constant__ CUtensorMap tmYlo,
                    int M, int N, int nkb, int nnz, const int *__restrict__ rowptr,
                    const int *__restrict__ colind, const float *__restrict__ aval,
                    float *__restrict__ out, const unsigned char *__restrict__ occ, int tiles_m,
                    int tiles_n, unsigned *status) {
    using L = PSmem<BN, BK>;
    extern __shared__ uint8_t smem_raw[];
    const uint32_t raw = smem_u32(smem_raw);
    uint8_t *smem = smem_raw + ((1024 - (raw & 1023)) & 1023);
    uint8_t *stages = smem;
    float *staging = reinterpret_cast<float *>(smem + L::kStages * L::kStage);
    uint64_t *full = reinterpret_cast<uint64_t *>(smem + L::kStages * L::kStage + L::kStaging);
    uint64_t *empty = full + L::kStages;
    uint64_t *accf = empty + L::kStages;
    uint64_t *acce = accf + 2;
    uint64_t *done = acce + 2;
    uint32_t *tmem_slot = reinterpret_cast<uint32_t *>(done + 1);
    volatile int *abort_flag = reinterpret_cast<volatile int *>(tmem_slot + 1);
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int ntiles = tiles_m * tiles_n;

    if (threadIdx.x == 0) {
        for (int i = 0; i < L::kStages; ++i) {
            mbar_init(&full[i], 1);
            mbar_init(&empty[i], 1);
        }
        mbar_init(&accf[0], 1);
        mbar_init(&accf[1], 1);
        mbar_init(&acce[0], 128);
        mbar_init(&acce[1], 128);
        mbar_init(done, 1);
        *abort_flag = 0;
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(
                         smem_u32(tmem_slot)),
                     "r"(2 * BN)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *tmem_slot;

    if (warp == 0) {
        if (lane == 0) {
            int it = 0;
            bool ok = true;
            for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
                int tm, tn;
                tile_coords(t, tiles_m, tiles_n, tm, tn);
                if (!occ[static_cast<long>(tm) * tiles_n + tn]) continue;
                for (int kb = 0; kb < nkb; ++kb, ++it) {
                    const int s = it % L::kStages, r = it / L::kStages;
                    if (r > 0 && !mbar_wait(&empty[s], (r - 1) & 1, abort_flag, status)) {
                        ok = false;
                        break;
                    }
                    uint8_t *st = stages + s * L::kStage;
                    mbar_expect_tx(&full[s], L::kStage);
                    tma_load_2d(st, &tmXhi, &full[s], kb * BK, tm * kBM);
                    tma_load_2d(st + L::kTileA, &tmXlo, &full[s], kb * BK, tm * kBM);
                    tma_load_2d(st + 2 * L::kTileA, &tmYhi, &full[s], kb * BK, tn * BN);
                    tma_load_2d(st + 2 * L::kTileA + L::kTileB, &tmYlo, &full[s], kb * BK, tn * BN);
                }
            }
            for (int d = it - L::kStages > 0 ? it - L::kStages : 0; d < it; ++d)
                for (unsigned i = 0; i < kSpinLimit; ++i)
                    if (mbar_try_wait(&full[d % L::kStages], (d / L::kStages) & 1)) break;
        }
    } else if (warp == 1) {
        if (lane == 0) {
            constexpr uint32_t idesc = idesc_bf16(kBM, BN);
            int it = 0, j = 0;
            bool ok = true;
            for (int t = blockIdx.x; t < ntiles && ok; t += gridDim.x) {
                int tm, tn;
                tile_coords(t, tiles_m, tiles_n, tm, tn);
                if (!occ[static_cast<long>(tm) * tiles_n + tn]) continue;
                const int buf = j & 1, use = j >> 1;
                if (use > 0 && !mbar_wait(&acce[buf], (use - 1) & 1, abort_flag, status)) break;
                tc_fence_after();
                const uint32_t d = tmem + buf * BN;
                for (int kb = 0; kb < nkb; ++kb, ++it) {
                    const int s = it % L::kStages, r = it / L::kStages;
                    if (!mbar_wait(&full[s], r & 1, abort_flag, status)) {
                        ok = false;
                        break;
                    }
                    tc_fence_after();
                    const uint32_t base = smem_u32(stages + s * L::kStage);
                    const uint64_t ahi = desc_kmajor(base, L::kSBO, L::kLayout);
                    const uint64_t alo = desc_kmajor(base + L::kTileA, L::kSBO, L::kLayout);
                    const uint64_t bhi = desc_kmajor(base + 2 * L::kTileA, L::kSBO, L::kLayout);
                    const uint64_t blo = desc_kmajor(base + 2 * L::kTileA + L::kTileB, L::kSBO, L::kLayout);
#pragma unroll
                    for (int k = 0; k < BK / 16; ++k) {
                        const uint64_t adv = static_cast<uint64_t>(k * 32 >> 4);
                        mma_bf16(d, ahi + adv, bhi + adv, idesc, (kb | k) != 0);
                        mma_bf16(d, ahi + adv, blo + adv, idesc, 1u);
                        mma_bf16(d, alo + adv, bhi + adv, idesc, 1u);
                    }
                    mma_commit(&empty[s]);
                }
                if (!ok) break;
                mma_commit(&accf[buf]);
                ++j;
            }
            // every MMA this thread issued has completed once `done` flips
            mma_commit(done);
            for (unsigned i = 0; i < kSpinLimit; ++i)
                if (mbar_try_wait(done, 0)) break;
        }
    } else {
        const int q = warp & 3;
        float *my = staging + (32 * q + lane) * 33;
        const uint32_t lane_addr = tmem + (static_cast<uint32_t>(32 * q) << 16);
        int j = 0;
        for (int t = blockIdx.x; t < ntiles; t += gridDim.x) {
            int tm, tn;
            tile_coords(t, tiles_m, tiles_n, tm, tn);
            if (!occ[static_cast<long>(tm) * tiles_n + tn]) continue;
            const int buf = j & 1, use = j >> 1;
            const int c0 = tn * BN;
            const int row = tm * kBM + 32 * q + lane;
            int e = 0, hi = 0;
            if (row < M) {
                int lo;
                row_range(rowptr, row, nnz, status, lo, hi);
                int a = lo, b = hi;
                while (a < b) {
                    const int m = (a + b) >> 1;
                    if (__ldg(colind + m) < c0) a = m + 1; else b = m;
                }
                e = a;
            }
            const bool ready = __all_sync(0xffffffffu, mbar_wait(&accf[buf], use & 1, abort_flag, status));
            if (!ready) break;
            tc_fence_after();
            int prev = -1;
#pragma unroll 1
            for (int jj = 0; jj < BN / 32; ++jj) {
                uint32_t v[32];
                tmem_ld32(lane_addr + buf * BN + 32 * jj, v);
                const int cend = c0 + 32 * (jj + 1);
                if (e < hi && __ldg(colind + e) < cend) {
#pragma unroll
                    for (int u = 0; u < 32; ++u) my[u] = __uint_as_float(v[u]);
                    while (e < hi) {
                        const int c = __ldg(colind + e);
                        if (c >= cend) break;
                        if (c <= prev || c >= N) {
                            flag(status, kFlagBadColind);
                            out[e] = 0.0f;
                        } else {
                            const float dv = my[c - (cend - 32)];
                            out[e] = aval ? __ldg(aval + e) * dv : dv;
                        }
                        prev = c;
                        ++e;
                    }
                }
            }
            tc_fence_before();
            asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(&acce[buf])) : "memory");
            ++j;
        }
    }
    tc_fence_before();
    __syncthreads();
    if (warp == 1) {
        tc_fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * BN)
                     : "memory");
    }
}

// One warp per row: flags rows whose columns do not ascend (or leave [0, N)), and sets
// occ[tm * tiles_n + tn] = 1 for every output tile holding a pattern entry -- one mark per
// (row, tile) since the columns ascend (the first entry of the row in each tile marks). Each
// lane issues four column loads before using them; a lane's predecessor column comes from
// the lane below (lane 0: the last column of the previous batch). SHARED: the CTA's 8 rows
// (all in one 128-row band) mark a shared copy of the band's flags, which the CTA then writes
// out once -- the 128 rows of a band otherwise store to the same few bytes, and those stores
// serialise in L2.
constexpr int kMarkSharedTiles = 16384;  // tiles per band held in shared memory

template <bool SHARED>
__global__ void __launch_bounds__(256)
check_and_mark(int M, int N, int nnz, const int *__restrict__ rowptr,
               const int *__restrict__ colind, int BN, int tiles_n, unsigned char *__restrict__ occ,
               unsigned *status) {
    extern __shared__ unsigned char sflag[];  // SHARED: tiles_n bytes
    const long w = (static_cast<long>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    const long band = (static_cast<long>(blockIdx.x) * (blockDim.x >> 5)) / kBM;
    if (SHARED) {
        for (int t = threadIdx.x; t < tiles_n; t += blockDim.x) sflag[t] = 0;
        __syncthreads();
    }
    unsigned char *rowocc = SHARED ? sflag : occ + (w / kBM) * static_cast<long>(tiles_n);
    bool bad = false;
    if (w < M) {
        int lo, hi;
        row_range(rowptr, static_cast<int>(w), nnz, status, lo, hi);
        int carry = -1;  // column of the entry before this batch (-1 before the row's first)
        for (int base = lo; base < hi; base += 128) {
            int c[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int e = base + 32 * q + lane;
                c[q] = e < hi ? __ldg(colind + e) : 0;
            }
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int e = base + 32 * q + lane;
                const int up = __shfl_up_sync(0xffffffffu, c[q], 1);
                const int last = __shfl_sync(0xffffffffu, c[q], 31);
                const int prev = lane == 0 ? carry : up;
                if (e < hi) {
                    if (c[q] < 0 || c[q] >= N || prev >= c[q])
                        bad = true;
                    else if (prev < 0 || prev / BN != c[q] / BN)
                        rowocc[c[q] / BN] = 1;
                }
                carry = last;
            }
        }
        if (__any_sync(0xffffffffu, bad) && lane == 0) flag(status, kFlagBadColind);
    }
    if (SHARED) {
        __syncthreads();
        unsigned char *bandocc = occ + band * static_cast<long>(tiles_n);
        for (int t = threadIdx.x; t < tiles_n; t += blockDim.x)
            if (sflag[t]) bandocc[t] = 1;
    }
}

// X's rows then Y's rows -> bf16 hi/lo planes: hi = bf16(x), lo = bf16(x - hi), columns
// [K, Kp) zero. A block takes (row, 4096-column segment) items; each thread issues its four
// 16-byte loads before converting, so a block keeps 16 KB of loads in flight.
__global__ void __launch_bounds__(256)
split_xy(long M, long N, int K, int Kp, const float *__restrict__ X, long ldx, bool vx,
         const float *__restrict__ Y, long ldy, bool vy, uint16_t *__restrict__ xhi,
         uint16_t *__restrict__ xlo, uint16_t *__restrict__ yhi, uint16_t *__restrict__ ylo) {
    constexpr int kSeg = 4096;
    const long segs = (Kp + kSeg - 1) / kSeg;
    const long items = (M + N) * segs;
    for (long item = blockIdx.x; item < items; item += gridDim.x) {
        const long row = item / segs;
        const int base = static_cast<int>(item - row * segs) * kSeg;
        const bool isx = row < M;
        const long r = isx ? row : row - M;
        const float *x = isx ? X + r * ldx : Y + r * ldy;
        const bool vec = isx ? vx : vy;
        uint16_t *hi = (isx ? xhi : yhi) + r * Kp, *lo = (isx ? xlo : ylo) + r * Kp;
        float v[4][4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int k = base + (u * 256 + static_cast<int>(threadIdx.x)) * 4;
            if (vec && k + 4 <= K) {
                const float4 t = __ldcs(reinterpret_cast<const float4 *>(x + k));
                v[u][0] = t.x; v[u][1] = t.y; v[u][2] = t.z; v[u][3] = t.w;
            } else {
#pragma unroll
                for (int i = 0; i < 4; ++i) v[u][i] = k + i < K ? __ldcs(x + k + i) : 0.0f;
            }
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            const int k = base + (u * 256 + static_cast<int>(threadIdx.x)) * 4;
            if (k >= Kp) continue;
            uint16_t h[4], l[4];
#pragma unroll
            for (int i = 0; i < 4; ++i) {
                h[i] = f32_to_bf16(v[u][i]);
                l[i] = f32_to_bf16(v[u][i] - bf16_to_f32(h[i]));
            }
            *reinterpret_cast<uint2 *>(hi + k) =
                make_uint2(h[0] | (unsigned(h[1]) << 16), h[2] | (unsigned(h[3]) << 16));
            *reinterpret_cast<uint2 *>(lo + k) =
                make_uint2(l[0] | (unsigned(l[1]) << 16), l[2] | (unsigned(l[3]) << 16));
        }
    }
}

// hi = bf16(x), lo = bf16(x - hi); columns [K, Kp) are zero. Blocks stride over rows,
// threads over groups of four columns.

// Columns must ascend within rows for the tile walk; flag rows that break it (one warp per
// row, coalesced).
__global__ void __launch_bounds__(256)
check_sorted_rows(int M, int N, int nnz, const int *__restrict__ rowptr,
                  const int *__restrict__ colind, unsigned *status) {
    const long w = (static_cast<long>(blockIdx.x) * blockDim.x + threadIdx.x) >> 5;
    const int lane = threadIdx.x & 31;
    if (w >= M) return;
    int lo, hi;
    row_range(rowptr, static_cast<int>(w), nnz, status, lo, hi);
    bool bad = false;
    for (int e = lo + lane; e < hi; e += 32) {
        const int c = __ldg(colind + e);
        if (c < 0 || c >= N || (e > lo && __ldg(colind + e - 1) >= c)) bad = true;
    }
    if (__any_sync(0xffffffffu, bad) && lane == 0) flag(status, kFlagBadColind);
}

__global__ void fill_zero(float *p, long n) {
    for (long i = static_cast<long>(blockIdx.x) * blockDim.x + threadIdx.x; i < n;
         i += static_cast<long>(gridDim.x) * blockDim.x)
        p[i] = 0.0f;
}

PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        void *p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault,
                                             &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }
    return fn;
}

// 2-D bf16 tensor map: rows x Kp (row-major), box = box_rows x box_k, swizzle = box_k * 2 bytes.
bool make_map(CUtensorMap *m, const uint16_t *base, long rows, int Kp, int box_rows,
              int box_k = kBK) {
    auto enc = encode_fn();
    if (!enc) return false;
    cuuint64_t dims[2] = {static_cast<cuuint64_t>(Kp), static_cast<cuuint64_t>(rows)};
    cuuint64_t strides[1] = {static_cast<cuuint64_t>(Kp) * 2};
    cuuint32_t box[2] = {static_cast<cuuint32_t>(box_k), static_cast<cuuint32_t>(box_rows)};
    cuuint32_t estr[2] = {1, 1};
    return enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<uint16_t *>(base), dims, strides,
               box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
               box_k == 32 ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_128B,
               CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int BN>
as_status launch_tiles(as_ctx *ctx, int M, int N, int Kp, int nnz, const int *rowptr,
                       const int *colind, const float *aval, float *out, const uint16_t *xhi,
                       const uint16_t *xlo, const uint16_t *yhi, const uint16_t *ylo,
                       cudaStream_t s) {
    CUtensorMap mxh, mxl, myh, myl;
    if (!make_map(&mxh, xhi, M, Kp, kBM) || !make_map(&mxl, xlo, M, Kp, kBM) ||
        !make_map(&myh, yhi, N, Kp, BN) || !make_map(&myl, ylo, N, Kp, BN))
        return fail(AS_ERR_CUDA, "sddmm_bf16x3: cuTensorMapEncodeTiled failed");
    const int smem = Smem<BN>::kBytes;
    cudaError_t e = cudaFuncSetAttribute(sddmm_tc_kernel<BN>,
                                         cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return check_cuda(e, "sddmm_bf16x3: shared memory attribute");
    dim3 grid(static_cast<unsigned>(ceil_div(N, BN)), static_cast<unsigned>(ceil_div(M, kBM)));
    sddmm_tc_kernel<BN><<<grid, kThreads, smem, s>>>(mxh, mxl, myh, myl, M, N, Kp / kBK, nnz,
                                                     rowptr, colind, aval, out, ctx->d_status);
    ctx->launches++;
    return check_cuda(cudaGetLastError(), "sddmm_bf16x3 launch");
}

int sm_count() {
    int dev = 0, n = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev);
    return n > 0 ? n : 148;
}

template <int BN, int BK>
as_status launch_persistent(as_ctx *ctx, int M, int N, int Kp, int nnz, const int *rowptr,
                            const int *colind, const float *aval, float *out, const uint16_t *xhi,
                            const uint16_t *xlo, const uint16_t *yhi, const uint16_t *ylo,
                            unsigned char *occ, cudaStream_t s) {
    CUtensorMap mxh, mxl, myh, myl;
    if (!make_map(&mxh, xhi, M, Kp, kBM, BK) || !make_map(&mxl, xlo, M, Kp, kBM, BK) ||
        !make_map(&myh, yhi, N, Kp, BN, BK) || !make_map(&myl, ylo, N, Kp, BN, BK))
        return fail(AS_ERR_CUDA, "sddmm_bf16x3: cuTensorMapEncodeTiled failed");
    const int tiles_m = static_cast<int>(ceil_div(M, kBM)), tiles_n = static_cast<int>(ceil_div(N, BN));
    const int smem = PSmem<BN, BK>::kBytes;
    cudaError_t e = cudaFuncSetAttribute(sddmm_tc_persistent<BN, BK>,
                             cudaFuncAttributeMaxDynamicSharedMemorySize, smem);
    if (e != cudaSuccess) return check_cuda(e, "sddmm_bf16x3: shared memory attribute");
    const long ntiles = static_cast<long>(tiles_m) * tiles_n;
    const int grid = static_cast<int>(ntiles < sm_count() ? ntiles : sm_count());
    sddmm_tc_persistent<BN, BK><<<grid, kThreads, smem, s>>>(
        mxh, mxl, myh, myl, M, N, Kp / BK, nnz, rowptr, colind, aval, out, occ, tiles_m, tiles_n,
        ctx->d_status);
    ctx->launches++;
    return check_cuda(cudaGetLastError(), "sddmm_bf16x3 persistent launch");
}

}  // namespace

int sddmm_tc_variant_count() { return 3; }

// variant: 1 = one tile per CTA (K block 64), 2 = persistent, K block 64, 3 = persistent,
// K block 32 (deeper pipeline); 0 = library choice.
as_status sddmm_bf16x3_launch(as_ctx *ctx, int M, int N, int K, int nnz, const int *rowptr,
                              const int *colind, const float *aval, const float *X, long ldx,
                              const float *Y, long ldy, float *out, int variant, cudaStream_t s) {
    if (variant == 0) variant = 3;  // persistent, 4-stage pipeline: fastest on GB300
    if (M == 0) return fail(AS_ERR_INVALID_CSR, "sddmm: nnz > 0 with zero rows");
    const int BN = 256;
    const int Kp = static_cast<int>(ceil_div(K, kBK) * kBK);
    const size_t xs = static_cast<size_t>(M) * Kp * 2, ys = static_cast<size_t>(N) * Kp * 2;
    auto al = [](size_t b) { return (b + 1023) & ~size_t(1023); };
    const int tiles_m = static_cast<int>(ceil_div(M, kBM)), tiles_n = static_cast<int>(ceil_div(N, BN));
    const size_t occ_bytes = static_cast<size_t>(tiles_m) * tiles_n;
    void *w = nullptr;
    as_status st = scratch(ctx, 2 * al(xs) + 2 * al(ys) + al(occ_bytes), &w);
    if (st != AS_OK) return st;
    uint8_t *p = static_cast<uint8_t *>(w);
    unsigned char *occ = p + 2 * al(xs) + 2 * al(ys);
    const unsigned rows_grid = static_cast<unsigned>(ceil_div(static_cast<long>(M) * 32, 256));
    if (variant == 1 || K == 0) {
        check_sorted_rows<<<rows_grid, 256, 0, s>>>(M, N, nnz, rowptr, colind, ctx->d_status);
    } else {
        cudaError_t e = cudaMemsetAsync(occ, 0, occ_bytes, s);
        if (e != cudaSuccess) return check_cuda(e, "sddmm_bf16x3: occupancy clear");
        if (tiles_n <= kMarkSharedTiles)
            check_and_mark<true><<<rows_grid, 256, static_cast<size_t>(tiles_n), s>>>(
                M, N, nnz, rowptr, colind, BN, tiles_n, occ, ctx->d_status);
        else
            check_and_mark<false><<<rows_grid, 256, 0, s>>>(M, N, nnz, rowptr, colind, BN,
                                                            tiles_n, occ, ctx->d_status);
    }
    ctx->launches++;
    if (K == 0) {
        fill_zero<<<static_cast<unsigned>(ceil_div(nnz, 256) < 4096 ? ceil_div(nnz, 256) : 4096), 256, 0, s>>>(out, nnz);
        ctx->launches++;
        return check_cuda(cudaGetLastError(), "sddmm_bf16x3 fill");
    }
    uint16_t *xhi = reinterpret_cast<uint16_t *>(p);
    uint16_t *xlo = reinterpret_cast<uint16_t *>(p + al(xs));
    uint16_t *yhi = reinterpret_cast<uint16_t *>(p + 2 * al(xs));
    uint16_t *ylo = reinterpret_cast<uint16_t *>(p + 2 * al(xs) + al(ys));
    const bool vx = ldx % 4 == 0 && reinterpret_cast<uintptr_t>(X) % 16 == 0;
    const bool vy = ldy % 4 == 0 && reinterpret_cast<uintptr_t>(Y) % 16 == 0;
    const long items = (static_cast<long>(M) + N) * ceil_div(Kp, 4096);
    const unsigned sg = static_cast<unsigned>(items < 152L * 8 ? items : 152L * 8);
    split_xy<<<sg, 256, 0, s>>>(M, N, K, Kp, X, ldx, vx, Y, ldy, vy, xhi, xlo, yhi, ylo);
    ctx->launches++;
    st = check_cuda(cudaGetLastError(), "sddmm_bf16x3 split");
    if (st != AS_OK) return st;
    if (variant == 2)
        return launch_persistent<256, 64>(ctx, M, N, Kp, nnz, rowptr, colind, aval, out, xhi, xlo,
                                          yhi, ylo, occ, s);
    if (variant == 3)
        return launch_persistent<256, 32>(ctx, M, N, Kp, nnz, rowptr, colind, aval, out, xhi, xlo,
                                          yhi, ylo, occ, s);
    return launch_tiles<256>(ctx, M, N, Kp, nnz, rowptr, colind, aval, out, xhi, xlo, yhi, ylo, s);
}

}  // namespace as
