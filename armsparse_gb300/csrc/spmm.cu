// CSR SpMM, C = A*B + beta*C, fp32 or bf16 storage with fp32 accumulation (sm_103a).
//
// Row-split family (bit-identical to the reference's rowBaseSpmm3, SDMM.cpp:90-114):
//   A group of GROUP lanes (1..32, a power of two) owns one row of A and a tile of
//   GROUP*ELEMS*CPL output columns. Lane g of the group holds CPL vectors of ELEMS
//   consecutive columns (16/8/4/2-byte loads of B rows: 128-bit when the layout allows).
//   The group fetches GROUP (colind, val) pairs of its row per step with one coalesced
//   load and broadcasts them with width-GROUP shuffles; every lane then walks the entries
//   in CSR order and updates its accumulators with fmaf(b, v, acc). Each output element is
//   therefore exactly the reference's fused-FMA chain. Blocks are 256 threads; blockIdx.x
//   runs over row blocks and blockIdx.y over column tiles, so the CTAs resident at any
//   moment share one column tile of B, which stays in L2. Rows with more than kLongRow
//   entries are skipped here and computed by the long-row kernel (spmm_long.cu), which keeps
//   the same chains.
#include <limits.h>
#include <stdio.h>

#include "common.cuh"
#include "internal.h"
#include "spmm_vec.cuh"

namespace as {
namespace {

template <int E>
__device__ __forceinline__ void store_c(float *p, const float *v) {
    if constexpr (E % 4 == 0) {
#pragma unroll
        for (int i = 0; i < E; i += 4)
            __stcs(reinterpret_cast<float4 *>(p + i), make_float4(v[i], v[i + 1], v[i + 2], v[i + 3]));
    } else if constexpr (E == 2) {
        __stcs(reinterpret_cast<float2 *>(p), make_float2(v[0], v[1]));
    } else {
#pragma unroll
        for (int i = 0; i < E; ++i) __stcs(p + i, v[i]);
    }
}

template <int E>
__device__ __forceinline__ void load_c(const float *p, float *v) {
    if constexpr (E % 4 == 0) {
#pragma unroll
        for (int i = 0; i < E; i += 4) {
            float4 t = *reinterpret_cast<const float4 *>(p + i);
            v[i] = t.x; v[i + 1] = t.y; v[i + 2] = t.z; v[i + 3] = t.w;
        }
    } else if constexpr (E == 2) {
        float2 t = *reinterpret_cast<const float2 *>(p);
        v[0] = t.x; v[1] = t.y;
    } else {
#pragma unroll
        for (int i = 0; i < E; ++i) v[i] = p[i];
    }
}

constexpr int kThreads = 256;

template <typename T, int VB, int GROUP, int CPL, int U, bool PF>
__global__ void __launch_bounds__(kThreads, PF ? 4 : 1)
spmm_rowsplit(int M, int K, int N, int nnz, const int *__restrict__ rowptr,
              const int *__restrict__ colind, const T *__restrict__ val,
              const T *__restrict__ B, long ldb, float *__restrict__ C, long ldc, float beta,
              unsigned *status, int long_thresh, int *long_list, unsigned *long_count,
              uint16_t *__restrict__ C16, bool relu) {
    using V = Vec<T, VB>;
    constexpr int E = V::E;
    constexpr int TILE = GROUP * E * CPL;
    const int lane = threadIdx.x & 31;
    const int g = threadIdx.x % GROUP;
    const unsigned gmask =
        GROUP == 32 ? 0xffffffffu : (((1u << GROUP) - 1u) << (lane & ~(GROUP - 1)));
    // let a programmatic dependent (the long-row kernel) be scheduled early; it waits for
    // this grid to complete before it reads anything
    asm volatile("griddepcontrol.launch_dependents;\n" ::: "memory");
    const long row = static_cast<long>(blockIdx.x) * (kThreads / GROUP) + threadIdx.x / GROUP;
    if (row >= M) return;  // the whole group leaves together
    int lo, hi;
    row_range(rowptr, static_cast<int>(row), nnz, status, lo, hi);
    if (hi - lo > long_thresh) {  // left to the long-row kernel (spmm_long.cu)
        if (blockIdx.y == 0 && g == 0) list_long_row(row, hi - lo, M, long_list, long_count, status);
        return;
    }

    const int tile0 = blockIdx.y * TILE;
    float acc[CPL][E];
    float *crow = C + row * ldc;
#pragma unroll
    for (int j = 0; j < CPL; ++j) {
        const int c = tile0 + (j * GROUP + g) * E;
        if (beta != 0.0f && c < N) {
            load_c<E>(crow + c, acc[j]);
#pragma unroll
            for (int i = 0; i < E; ++i) acc[j][i] *= beta;
        } else {
#pragma unroll
            for (int i = 0; i < E; ++i) acc[j][i] = 0.0f;
        }
    }

    // (colind, val) of GROUP entries per batch, one per lane. PF: the next batch is loaded while
    // the current one is consumed (registers capped so that four CTAs stay resident)
    auto load_entry = [&](int e, int &k, float &v) {
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
    int kn = -1;
    float vn = 0.0f;
    if (PF) load_entry(lo + g, kn, vn);
    for (int base = lo; base < hi; base += GROUP) {
        int k;
        float v;
        if (PF) {
            k = kn;
            v = vn;
            load_entry(base + GROUP + g, kn, vn);
        } else {
            load_entry(base + g, k, v);
        }
        const int cnt = min(GROUP, hi - base);
        int t = 0;
        // U entries per step: their B loads are issued before the FMAs, which then run in
        // CSR order. fp32 keeps per-load predicates (measured faster on GB300); bf16 loads
        // branch-free into packed registers (an idle lane or a flagged entry reads an
        // in-bounds element that contributes nothing) and unpacks at the FMA, which halves the
        // registers held per load and lets more loads be in flight.
        for (; t + U <= cnt; t += U) {
            int kk[U];
            float vv[U];
#pragma unroll
            for (int u = 0; u < U; ++u) {
                kk[u] = __shfl_sync(gmask, k, t + u, GROUP);
                vv[u] = __shfl_sync(gmask, v, t + u, GROUP);
            }
            if constexpr (sizeof(T) == 4) {
                float b[U][CPL][E];
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    const T *brow = B + static_cast<long>(kk[u] < 0 ? 0 : kk[u]) * ldb;
#pragma unroll
                    for (int j = 0; j < CPL; ++j) {
                        const int c = tile0 + (j * GROUP + g) * E;
                        if (c < N && kk[u] >= 0) {
                            V::load(brow + c, b[u][j]);
                        } else {
#pragma unroll
                            for (int i = 0; i < E; ++i) b[u][j][i] = 0.0f;
                        }
                    }
                }
#pragma unroll
                for (int u = 0; u < U; ++u)
#pragma unroll
                    for (int j = 0; j < CPL; ++j) fma_vec_f32<E>(b[u][j], vv[u], acc[j]);
            } else {
                typename V::Raw b[U][CPL];
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    const T *brow = B + static_cast<long>(kk[u] < 0 ? 0 : kk[u]) * ldb;
#pragma unroll
                    for (int j = 0; j < CPL; ++j) {
                        const int c = tile0 + (j * GROUP + g) * E;
                        b[u][j] = V::raw(brow + (c < N ? c : 0));
                    }
                }
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    // v came from bf16, so its fp32 bits are the bf16 bits followed by zeros
                    const unsigned short vu = kk[u] < 0
                        ? static_cast<unsigned short>(0)
                        : static_cast<unsigned short>(__float_as_uint(vv[u]) >> 16);
#pragma unroll
                    for (int j = 0; j < CPL; ++j) V::fma(b[u][j], vu, acc[j]);
                }
            }
        }
        for (; t < cnt; ++t) {
            const int kk = __shfl_sync(gmask, k, t, GROUP);
            const float vv = __shfl_sync(gmask, v, t, GROUP);
            if (kk < 0) continue;
            const T *brow = B + static_cast<long>(kk) * ldb;
#pragma unroll
            for (int j = 0; j < CPL; ++j) {
                const int c = tile0 + (j * GROUP + g) * E;
                if (c < N) {
                    float b[E];
                    V::load(brow + c, b);
#pragma unroll
                    for (int i = 0; i < E; ++i) acc[j][i] = fmaf(b[i], vv, acc[j][i]);
                }
            }
        }
    }

#pragma unroll
    for (int j = 0; j < CPL; ++j) {
        const int c = tile0 + (j * GROUP + g) * E;
        if (c < N) {
            if (C16)
                store_bf16<E>(C16 + row * ldc + c, acc[j], relu);
            else
                store_c<E>(crow + c, acc[j]);
        }
    }
}

// ---- variant table --------------------------------------------------------------------------
struct Variant {
    int vb, group, cpl, unroll;
    const char *name;
    int kind;  // 0 = row-split (registers), 1 = bulk-copy staged (spmm_bulk.cu: vb = bytes per
               // lane, unroll = ring stages), 2 = nnz-split (spmm_nnz.cu: unroll = chunk size,
               // steps = entries per load batch), 3 = multi-entry nnz-split (spmm_nnz.cu, a warp
               // per chunk in 32 / group sub-groups; unroll = chunk size)
    int steps = 4;
    int pf = 0;  // row-split: 1 = next index batch prefetched (64 registers at most)
};

#define AS_V(vb, g, c, u) {vb, g, c, u, "rowsplit_v" #vb "_g" #g "_c" #c "_u" #u, 0}
#define AS_VPF(vb, g, c, u) {vb, g, c, u, "rowsplit_v" #vb "_g" #g "_c" #c "_u" #u "_pf", 0, 4, 1}
#define AS_VPFS AS_VPF(8, 32, 4, 4), AS_VPF(16, 32, 2, 4), AS_VPF(16, 32, 4, 4)
#define AS_BULK(lb, st) {lb, 32, 1, st, "bulk_lb" #lb "_s" #st, 1}
#define AS_BULKS AS_BULK(16, 8), AS_BULK(32, 8), AS_BULK(16, 16), AS_BULK(32, 4)
#define AS_NNZ(vb, g, c, ch) {vb, g, c, ch, "nnzsplit_v" #vb "_g" #g "_c" #c "_ch" #ch, 2}
#define AS_NNZ8(vb, g, c, ch) {vb, g, c, ch, "nnzsplit_v" #vb "_g" #g "_c" #c "_ch" #ch "_u8", 2, 8}
#define AS_NNZS8(ch) AS_NNZ8(16, 16, 1, ch), AS_NNZ8(16, 32, 1, ch), AS_NNZ8(16, 32, 2, ch), \
    AS_NNZ8(4, 32, 1, ch), AS_NNZ8(4, 32, 2, ch)
#define AS_NNZS(ch) AS_NNZ(16, 8, 1, ch), AS_NNZ(16, 16, 1, ch), AS_NNZ(16, 32, 1, ch), \
    AS_NNZ(16, 32, 2, ch), AS_NNZ(4, 32, 1, ch), AS_NNZ(4, 32, 2, ch)
#define AS_NNZS_BF16_SCALAR(ch) AS_NNZ(2, 32, 1, ch), AS_NNZ(2, 32, 2, ch)
#define AS_VG(vb, g) AS_V(vb, g, 1, 4), AS_V(vb, g, 2, 4), AS_V(vb, g, 4, 4), AS_V(vb, g, 1, 8), \
    AS_V(vb, g, 2, 8)
#define AS_VROW(vb) AS_VG(vb, 1), AS_VG(vb, 2), AS_VG(vb, 4), AS_VG(vb, 8), AS_VG(vb, 16), AS_VG(vb, 32)

// 32-entry chunks: many short chains for small graphs (N <= kSmallChunkMaxN: their carry
// scratch, 2 x nnz/32 x N floats, stays modest)
#define AS_NNZS32 AS_NNZ(4, 32, 1, 32), AS_NNZ(4, 32, 2, 32), AS_NNZ(16, 32, 1, 32)
// multi-entry chunks for narrow rows of B (a row of B spans fewer than 32 lanes' vectors)
#define AS_ME(vb, g, ch) {vb, g, 1, ch, "nnzme_v" #vb "_g" #g "_ch" #ch, 3}
#define AS_MES AS_ME(16, 8, 256), AS_ME(16, 8, 1024), AS_ME(16, 16, 1024), AS_ME(8, 8, 1024), \
    AS_ME(8, 16, 1024)
constexpr int kSmallChunk = 32;
constexpr int kSmallChunkMaxN = 64;
const Variant kF32[] = {AS_VROW(16), AS_VROW(8), AS_VROW(4), AS_BULKS, AS_NNZS(128),
                        AS_NNZS(1024), AS_NNZS8(256), AS_NNZS8(1024), AS_NNZS32, AS_MES,
                        AS_VPFS};
const Variant kBF16[] = {AS_VROW(16), AS_VROW(8), AS_VROW(4), AS_VROW(2), AS_BULKS,
                         AS_NNZS(128), AS_NNZS(1024), AS_NNZS_BF16_SCALAR(128),
                         AS_NNZS_BF16_SCALAR(1024), AS_NNZS8(256), AS_NNZS8(1024),
                         AS_NNZ8(2, 32, 2, 256), AS_NNZ8(2, 32, 2, 1024), AS_NNZS32, AS_MES,
                         AS_VPFS};
constexpr int kNF32 = sizeof(kF32) / sizeof(kF32[0]);
constexpr int kNBF16 = sizeof(kBF16) / sizeof(kBF16[0]);

struct LongRows {
    int thresh;       // rows with more entries go to the long-row kernel (INT_MAX: none)
    int *list;        // their row numbers (scratch, M entries)
    unsigned *count;  // list length (context device word)
};

template <typename T, int VB, int G, int CPL, int U, bool PF = false>
void launch_one(const SpmmArgs &a, const LongRows &lr, cudaStream_t s) {
    constexpr int E = Vec<T, VB>::E;
    constexpr int TILE = G * E * CPL;
    dim3 grid(static_cast<unsigned>(ceil_div(a.M, kThreads / G)),
              static_cast<unsigned>(ceil_div(a.N, TILE)));
    spmm_rowsplit<T, VB, G, CPL, U, PF><<<grid, kThreads, 0, s>>>(
        a.M, a.K, a.N, a.nnz, a.rowptr, a.colind, static_cast<const T *>(a.val),
        static_cast<const T *>(a.B), a.ldb, a.C, a.ldc, a.beta, a.status, lr.thresh, lr.list,
        lr.count, a.C16, a.relu);
}

template <typename T, int VB, int G>
bool dispatch_cpl(int cpl, int u, const SpmmArgs &a, const LongRows &lr, cudaStream_t s) {
    if (u == 4) {
        switch (cpl) {
            case 1: launch_one<T, VB, G, 1, 4>(a, lr, s); return true;
            case 2: launch_one<T, VB, G, 2, 4>(a, lr, s); return true;
            case 4: launch_one<T, VB, G, 4, 4>(a, lr, s); return true;
        }
    } else if (u == 8) {
        switch (cpl) {
            case 1: launch_one<T, VB, G, 1, 8>(a, lr, s); return true;
            case 2: launch_one<T, VB, G, 2, 8>(a, lr, s); return true;
        }
    }
    return false;
}

// the prefetching row-split kernels: full warps, four entries per step
template <typename T>
bool dispatch_pf(int vb, int cpl, const SpmmArgs &a, const LongRows &lr, cudaStream_t s) {
    if (vb == 8 && cpl == 4) { launch_one<T, 8, 32, 4, 4, true>(a, lr, s); return true; }
    if (vb == 16 && cpl == 2) { launch_one<T, 16, 32, 2, 4, true>(a, lr, s); return true; }
    if (vb == 16 && cpl == 4) { launch_one<T, 16, 32, 4, 4, true>(a, lr, s); return true; }
    return false;
}

template <typename T, int VB>
bool dispatch_group(int g, int cpl, int u, const SpmmArgs &a, const LongRows &lr,
                    cudaStream_t s) {
    switch (g) {
        case 1: return dispatch_cpl<T, VB, 1>(cpl, u, a, lr, s);
        case 2: return dispatch_cpl<T, VB, 2>(cpl, u, a, lr, s);
        case 4: return dispatch_cpl<T, VB, 4>(cpl, u, a, lr, s);
        case 8: return dispatch_cpl<T, VB, 8>(cpl, u, a, lr, s);
        case 16: return dispatch_cpl<T, VB, 16>(cpl, u, a, lr, s);
        case 32: return dispatch_cpl<T, VB, 32>(cpl, u, a, lr, s);
    }
    return false;
}

bool aligned(const void *p, int bytes) { return reinterpret_cast<uintptr_t>(p) % bytes == 0; }

// Can vector width `vb` bytes serve these arguments?
bool vb_ok(int dtype, int vb, int N, long ldb, long ldc, const void *B, const void *C) {
    const int esz = dtype == 0 ? 4 : 2;
    const int e = vb / esz;
    if (e < 1) return false;
    if (N % e || ldb % e || ldc % e) return false;
    if (!aligned(B, vb)) return false;
    // C is fp32: its vectors hold e floats
    if (!aligned(C, 4 * e > 16 ? 16 : 4 * e)) return false;
    return true;
}

}  // namespace

int spmm_variant_count(int dtype) { return dtype == 0 ? kNF32 : kNBF16; }

const char *spmm_variant_name(int dtype, int variant) {
    const int n = spmm_variant_count(dtype);
    if (variant < 1 || variant > n) return "unknown";
    return dtype == 0 ? kF32[variant - 1].name : kBF16[variant - 1].name;
}

static int find_variant(int dtype, int vb, int g, int cpl, int u, int pf = 0) {
    const Variant *t = dtype == 0 ? kF32 : kBF16;
    const int n = spmm_variant_count(dtype);
    for (int i = 0; i < n; ++i)
        if (t[i].kind == 0 && t[i].pf == pf && t[i].vb == vb && t[i].group == g && t[i].cpl == cpl &&
            t[i].unroll == u)
            return i + 1;
    return 0;
}

// Library choice among the bit-identical row-split kernels, from variant sweeps on GB300 (a
// uniform 100k x 100k matrix with 2M entries and a power-law 200k one, N from 16 to 384, and
// the 4096-square C1 matrix): the fastest kernel's column tile matches the width of B, with
// 16- or 8-byte vectors, and the one tile of a wide row wants full warps with two or four
// vectors per lane (fp32: float4 x 2 with the next index batch prefetched, then float2 x 4;
// bf16: 8 x bf16 x 2). Each width class lists its pick first, then narrower vectors for B and
// C layouts the wider ones cannot serve. The entry-balanced kernels, which win on skewed rows,
// are not picked here: they change the summation order of rows that cross a chunk, and the
// library cannot see the row lengths without reading rowptr (the learned selector does that on
// the host).
int spmm_default_variant(int dtype, int M, int K, int N, int nnz, long ldb, long ldc,
                         const void *B, const void *C) {
    (void)M; (void)K; (void)nnz;
    const int esz = dtype == 0 ? 4 : 2;
    struct Pick { int vb, g, cpl, u, pf; };
    struct Class { int max_n; Pick picks[4]; int n; };
    // fp32 (tile = vb / 4 * g * cpl columns)
    static const Class f32[] = {
        {16, {{16, 2, 2, 4, 0}, {8, 4, 2, 4, 0}, {4, 8, 2, 4, 0}}, 3},
        {32, {{16, 4, 2, 8, 0}, {8, 8, 2, 4, 0}, {4, 16, 2, 4, 0}}, 3},
        {64, {{8, 16, 2, 4, 0}, {4, 16, 4, 4, 0}, {4, 32, 2, 8, 0}}, 3},
        {128, {{8, 32, 2, 4, 0}, {4, 32, 4, 4, 0}, {4, 32, 2, 8, 0}}, 3},
        {256, {{16, 32, 2, 4, 1}, {8, 32, 4, 4, 1}, {8, 32, 2, 4, 0}, {4, 32, 4, 4, 0}}, 4},
        {511, {{8, 32, 2, 4, 0}, {4, 32, 4, 4, 0}, {4, 32, 2, 8, 0}}, 3},
        {INT_MAX, {{16, 32, 2, 4, 1}, {8, 32, 4, 4, 0}, {16, 32, 2, 4, 0}, {4, 32, 2, 8, 0}}, 4},
    };
    // bf16 (tile = vb / 2 * g * cpl columns)
    static const Class bf16[] = {
        {16, {{8, 4, 1, 4, 0}, {4, 8, 1, 4, 0}, {2, 16, 1, 4, 0}}, 3},
        {32, {{16, 4, 1, 4, 0}, {8, 8, 1, 4, 0}, {4, 16, 1, 4, 0}}, 3},
        {64, {{16, 8, 1, 4, 0}, {8, 16, 1, 4, 0}, {4, 16, 2, 4, 0}}, 3},
        {128, {{16, 8, 2, 4, 0}, {8, 16, 2, 4, 0}, {4, 32, 2, 4, 0}}, 3},
        {256, {{16, 32, 1, 4, 0}, {16, 16, 2, 4, 0}, {8, 32, 2, 4, 0}, {4, 32, 4, 4, 0}}, 4},
        {511, {{16, 32, 2, 4, 1}, {16, 32, 2, 4, 0}, {8, 32, 2, 4, 0}, {4, 32, 4, 4, 0}}, 4},
        {INT_MAX, {{16, 32, 2, 4, 0}, {8, 32, 2, 4, 0}, {4, 32, 4, 4, 0}, {2, 32, 2, 8, 0}}, 4},
    };
    // bf16 rows wider than one 512-column tile that do not fill whole tiles: the 256-column
    // tile (no half-empty last tile; 0.313 against 0.385 ms at N = 768 on the sweep matrix)
    if (dtype == 1 && N > 511 && N % 512 != 0 && vb_ok(dtype, 16, N, ldb, ldc, B, C)) {
        const int v = find_variant(dtype, 16, 32, 1, 4, 0);
        if (v) return v;
    }
    const Class *cls = dtype == 0 ? f32 : bf16;
    while (N > cls->max_n) ++cls;
    for (int i = 0; i < cls->n; ++i) {
        const Pick &p = cls->picks[i];
        if (!vb_ok(dtype, p.vb, N, ldb, ldc, B, C)) continue;
        const int v = find_variant(dtype, p.vb, p.g, p.cpl, p.u, p.pf);
        if (v) return v;
    }
    // any layout: scalar lanes
    return find_variant(dtype, esz, 32, N > 32 ? 2 : 1, 8);
}

// Whether `variant` can serve this layout (the launch would not return AS_ERR_UNSUPPORTED).
bool spmm_variant_supported(int dtype, int variant, int N, long ldb, long ldc, const void *B,
                            const void *C) {
    if (variant < 1 || variant > spmm_variant_count(dtype)) return false;
    const Variant &v = dtype == 0 ? kF32[variant - 1] : kBF16[variant - 1];
    const int esz = dtype == 0 ? 4 : 2;
    const uintptr_t pb = reinterpret_cast<uintptr_t>(B), pc = reinterpret_cast<uintptr_t>(C);
    if (v.kind == 0) {
        const int tile = (v.vb / esz) * v.group * v.cpl;
        return vb_ok(dtype, v.vb, N, ldb, ldc, B, C) && ceil_div(N, tile) <= 65535;
    }
    if (v.kind == 1) {  // bulk: E = lane bytes / esz, tile = 32 * E
        const int E = v.vb / esz, tile = 32 * E;
        return N % E == 0 && (ldb * esz) % 16 == 0 && ldc % 4 == 0 && pb % 16 == 0 &&
               pc % 16 == 0 && (static_cast<long>(N % tile) * esz) % 16 == 0 &&
               ceil_div(N, tile) <= 65535;
    }
    const int E = v.vb / esz;  // nnz-split and multi-entry
    if (v.kind == 2 && v.unroll == kSmallChunk && N > kSmallChunkMaxN) return false;
    return N % E == 0 && ldb % E == 0 && pb % (E * esz) == 0 &&
           ceil_div(N, E * v.group * v.cpl) <= 65535 && ceil_div(N, 32) <= 65535;
}

// A bf16 output (a.C16) in vectors of e elements: aligned to min(2e, 16) bytes, rows of e.
static bool c16_ok(int e, long ldc, const void *C16) {
    return ldc % e == 0 && aligned(C16, 2 * e > 16 ? 16 : 2 * e);
}

as_status spmm_launch(as_ctx *ctx, int dtype, int variant, const SpmmArgs &a, cudaStream_t s) {
    const Variant &v = dtype == 0 ? kF32[variant - 1] : kBF16[variant - 1];
    if (a.C16) {
        const int e = v.vb / (dtype == 0 ? 4 : 2);
        if (v.kind == 1)
            return fail(AS_ERR_UNSUPPORTED, std::string("spmm: variant ") + v.name +
                                                " has no bf16 output");
        if (a.beta != 0.0f) return fail(AS_ERR_INVALID_VALUE, "spmm: bf16 output needs beta = 0");
        if (!c16_ok(e, a.ldc, a.C16))
            return fail(AS_ERR_UNSUPPORTED, std::string("spmm: variant ") + v.name +
                                                " needs the bf16 C aligned to its vectors");
    }
    if (v.kind == 1) return spmm_bulk_launch(ctx, dtype, v.vb, v.unroll, a, s);
    if (v.kind == 3) return spmm_nnzme_launch(ctx, dtype, v.vb, v.group, v.unroll, a, s);
    if (v.kind == 2) {
        if (v.unroll == kSmallChunk && a.N > kSmallChunkMaxN)
            return fail(AS_ERR_UNSUPPORTED, std::string("spmm: variant ") + v.name +
                                                " serves N <= 64 only");
        return spmm_nnz_launch(ctx, dtype, v.vb, v.group, v.cpl, v.unroll, v.steps, a, s);
    }
    if (!vb_ok(dtype, v.vb, a.N, a.ldb, a.ldc, a.B, a.C16 ? nullptr : a.C))
        return fail(AS_ERR_UNSUPPORTED, std::string("spmm: variant ") + v.name +
                                            " needs N, ldb, ldc and pointer alignment to match its vector width");
    if (ceil_div(a.N, (v.vb / (dtype == 0 ? 4 : 2)) * v.group * v.cpl) > 65535)
        return fail(AS_ERR_UNSUPPORTED, "spmm: N too large for this variant's column tile");
    // rows longer than kLongRow entries go to the long-row kernel when its copies can serve
    // the layout (a matrix with nnz <= kLongRow has none)
    LongRows lr{INT_MAX, nullptr, ctx->d_long};
    const int granule = a.nnz > kLongRow && a.M > 0 ? spmm_long_granule(dtype, a.N, a.ldb, a.B) : 0;
    if (granule) {
        void *p = nullptr;
        as_status st = scratch(ctx, static_cast<size_t>(a.M) * sizeof(int), &p);
        if (st != AS_OK) return st;
        lr.thresh = kLongRow;
        lr.list = static_cast<int *>(p);
    }
    bool ok = false;
    if (v.pf) {
        ok = dtype == 0 ? dispatch_pf<float>(v.vb, v.cpl, a, lr, s)
                        : dispatch_pf<uint16_t>(v.vb, v.cpl, a, lr, s);
    } else if (dtype == 0) {
        switch (v.vb) {
            case 16: ok = dispatch_group<float, 16>(v.group, v.cpl, v.unroll, a, lr, s); break;
            case 8: ok = dispatch_group<float, 8>(v.group, v.cpl, v.unroll, a, lr, s); break;
            case 4: ok = dispatch_group<float, 4>(v.group, v.cpl, v.unroll, a, lr, s); break;
        }
    } else {
        switch (v.vb) {
            case 16: ok = dispatch_group<uint16_t, 16>(v.group, v.cpl, v.unroll, a, lr, s); break;
            case 8: ok = dispatch_group<uint16_t, 8>(v.group, v.cpl, v.unroll, a, lr, s); break;
            case 4: ok = dispatch_group<uint16_t, 4>(v.group, v.cpl, v.unroll, a, lr, s); break;
            case 2: ok = dispatch_group<uint16_t, 2>(v.group, v.cpl, v.unroll, a, lr, s); break;
        }
    }
    if (!ok) return fail(AS_ERR_UNSUPPORTED, "spmm: variant not instantiated");
    ctx->launches++;
    as_status st = check_cuda(cudaGetLastError(), "spmm launch");
    if (st != AS_OK || !granule) return st;
    st = spmm_long_launch(ctx, dtype, granule, a, lr.list, s);
    if (st != AS_OK) cudaMemsetAsync(ctx->d_long, 0, 3 * sizeof(unsigned), s);
    return st;
}

// The SpMM with the SDDMM fused in (spmm_nnz.cu): nnz-split variants only, one column tile.
// Library choice: the narrowest full-warp tile that covers N (chunks of 1024 entries, four
// entries per load batch -- the variants the autotuner picks for the power-law GCN layers).
as_status spmm_sddmm_launch(as_ctx *ctx, int dtype, int variant, const SpmmArgs &a,
                            const SddmmFuse &f, cudaStream_t s) {
    const int esz = dtype == 0 ? 4 : 2;
    const Variant *t = dtype == 0 ? kF32 : kBF16;
    const int n = spmm_variant_count(dtype);
    auto tile = [&](const Variant &v) { return (v.vb / esz) * v.group * v.cpl; };
    if (variant == 0) {
        const int picks[][3] = {{4, 32, 1}, {16, 32, 1}, {16, 32, 2}};  // vb, group, cpl
        for (const auto &pk : picks) {
            for (int i = 0; i < n && variant == 0; ++i)
                if (t[i].kind == 2 && t[i].vb == pk[0] && t[i].group == pk[1] &&
                    t[i].cpl == pk[2] && t[i].unroll == 1024 && t[i].steps == 4 &&
                    tile(t[i]) >= a.N &&
                    spmm_variant_supported(dtype, i + 1, a.N, a.ldb, a.ldc, a.B, a.C))
                    variant = i + 1;
            if (variant) break;
        }
        if (variant == 0)
            return fail(AS_ERR_UNSUPPORTED, "spmm+sddmm: no variant covers this N and layout");
    }
    const Variant &v = t[variant - 1];
    if (v.kind != 2 && v.kind != 3)
        return fail(AS_ERR_UNSUPPORTED, std::string("spmm+sddmm: variant ") + v.name +
                                            " is not an nnz-split variant");
    if (tile(v) < a.N)
        return fail(AS_ERR_UNSUPPORTED, std::string("spmm+sddmm: variant ") + v.name +
                                            " covers fewer than N columns");
    if (v.kind == 3) return spmm_nnzme_launch(ctx, dtype, v.vb, v.group, v.unroll, a, s, &f);
    if (v.unroll == kSmallChunk && a.N > kSmallChunkMaxN)
        return fail(AS_ERR_UNSUPPORTED, std::string("spmm+sddmm: variant ") + v.name +
                                            " serves N <= 64 only");
    return spmm_nnz_launch(ctx, dtype, v.vb, v.group, v.cpl, v.unroll, v.steps, a, s, &f);
}

}  // namespace as
