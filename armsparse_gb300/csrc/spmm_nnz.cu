// CSR SpMM balanced by entries (sm_103a): C = A*B + beta*C for matrices whose row lengths are
// skewed (power-law graphs), where one long row would serialise a row-per-group kernel.
//
// Pass 1 (spmm_nnzsplit): the entries are cut into chunks of CH consecutive entries; a group
//   of GROUP lanes takes one chunk and one column tile, walks the chunk's row segments in CSR
//   order and accumulates each segment with fmaf like the row-split kernels. A row that lies
//   entirely inside the chunk is written to C directly (bit-identical to rowBaseSpmm3,
//   SDMM.cpp:90-114). A row that crosses a chunk boundary leaves its segment's partial sum in
//   a carry slot: slot 0 when the segment starts the chunk, slot 1 otherwise.
// Pass 2 (spmm_nnz_fixup): for every row that ends inside chunk c after starting in an earlier
//   chunk, chunk c's warp (a whole CTA for a long span) adds that row's partial sums (in chunk
//   order when the row spans at most 8 chunks, else runs of chunks and then the runs in order;
//   then beta * C): a fixed order, so the result is deterministic run to run (not
//   bit-identical to a single chain for those rows).
// Pass 3 (spmm_empty_rows): rows without entries get beta * C (zeros when beta == 0).
//
// Fused form (FUSE): pass 1 also computes, for every entry e (row r, column k), the dot product
// dA[perm[e]] = <B[k, :], F[r, :]> from the B row it has just loaded for the SpMM and F's row r
// (loaded once per row segment): the SDDMM that the backward of a product with trainable
// values needs, without a second gather of B. Each lane chains over its own
// columns of the row (its E-element slices j = 0..CPL-1, in order), then the GROUP lanes are
// summed by a butterfly (lane l adds lane l ^ off, off = GROUP/2 .. 1) -- for a step of U
// entries the butterflies of all U run interleaved (each lane hands half of its values to its
// partner at the first log2(U) steps), which pairs the same lanes in the same order, so each
// dot product is the single-entry butterfly's bit for bit. One column tile only (TILE >= N).
#include "common.cuh"
#include "internal.h"
#include "spmm_vec.cuh"

namespace as {
namespace {

constexpr int kThreads = 256;

__device__ __forceinline__ int find_row(const int *__restrict__ rowptr, int M, int e) {
    int lo = 0, hi = M;  // largest r with rowptr[r] <= e
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(rowptr + mid) <= e)
            lo = mid;
        else
            hi = mid;
    }
    return lo;
}

// Sum of each of the U values d[0..U) over the GROUP lanes of a group (U <= GROUP, both powers
// of two). While a lane holds more than one value, it keeps one half and sends the other to its
// partner lane ^ off; then plain butterfly steps. Lane g ends with the total of value
// g / (GROUP / U); the pairing tree is the single-value butterfly's.
template <int U, int GROUP>
__device__ __forceinline__ float reduce_entries(float (&d)[U], unsigned gmask, int g) {
    static_assert(U <= GROUP && (U & (U - 1)) == 0 && (GROUP & (GROUP - 1)) == 0, "shape");
#pragma unroll
    for (int h = U / 2, off = GROUP / 2; h >= 1; h >>= 1, off >>= 1) {
        const bool up = (g & off) != 0;
#pragma unroll
        for (int i = 0; i < h; ++i) {
            const float send = up ? d[i] : d[i + h];
            const float keep = up ? d[i + h] : d[i];
            d[i] = keep + __shfl_xor_sync(gmask, send, off, GROUP);
        }
    }
#pragma unroll
    for (int off = GROUP / (2 * U); off >= 1; off >>= 1)
        d[0] += __shfl_xor_sync(gmask, d[0], off, GROUP);
    return d[0];
}

// dA[perm[e]] (dA[e] without perm) = v, skipping and flagging a position outside [0, nnz).
__device__ __forceinline__ void store_dot(int e, float v, int nnz, const int *__restrict__ perm,
                                          float *__restrict__ dA, unsigned *status) {
    const int p = perm ? __ldg(perm + e) : e;
    if (static_cast<unsigned>(p) < static_cast<unsigned>(nnz))
        dA[p] = v;
    else
        flag(status, kFlagBadPerm);
}

// The U dot products of a step (entries e0 .. e0 + U - 1) reduced over the group and stored
// at their CSR positions; an entry with an out-of-range column (kk < 0, already flagged) is
// left unwritten.
template <int U, int GROUP>
__device__ __forceinline__ void write_dots(float (&d)[U], const int (&kk)[U], unsigned gmask,
                                           int g, int e0, int nnz, const int *__restrict__ perm,
                                           float *__restrict__ dA, unsigned *status) {
    unsigned ok = 0;
#pragma unroll
    for (int u = 0; u < U; ++u) ok |= (kk[u] >= 0 ? 1u : 0u) << u;
    const float sum = reduce_entries<U, GROUP>(d, gmask, g);
    constexpr int SUB = GROUP / U;
    const int u = g / SUB;
    if (g % SUB == 0 && ((ok >> u) & 1u)) store_dot(e0 + u, sum, nnz, perm, dA, status);
}

template <typename T, int VB, int GROUP, int CPL, int U, bool FUSE>
__global__ void __launch_bounds__(kThreads)
spmm_nnzsplit(int M, int K, int N, int nnz, int CH, const int *__restrict__ rowptr,
              const int *__restrict__ colind, const T *__restrict__ val,
              const T *__restrict__ B, long ldb, float *__restrict__ C, long ldc, float beta,
              float *__restrict__ carry, int *__restrict__ fix, unsigned *status,
              const T *__restrict__ F, long ldf, const int *__restrict__ perm,
              float *__restrict__ dA, uint16_t *__restrict__ C16, bool relu) {
    using V = Vec<T, VB>;
    constexpr int E = V::E;
    constexpr int TILE = GROUP * E * CPL;
    const int lane = threadIdx.x & 31;
    const int g = threadIdx.x % GROUP;
    const unsigned gmask =
        GROUP == 32 ? 0xffffffffu : (((1u << GROUP) - 1u) << (lane & ~(GROUP - 1)));
    const long chunk = static_cast<long>(blockIdx.x) * (kThreads / GROUP) + threadIdx.x / GROUP;
    const long e0l = chunk * CH;
    if (e0l >= nnz) return;
    const int e0 = static_cast<int>(e0l);
    const int e1 = static_cast<int>(e0l + CH < nnz ? e0l + CH : nnz);
    const int tile0 = blockIdx.y * TILE;
    int r = find_row(rowptr, M, e0);
    int e = e0;
    int fix_row = -1;  // the row that started in an earlier chunk and ends in this one
    while (e < e1 && r < M) {
        const int rs = __ldg(rowptr + r), re = __ldg(rowptr + r + 1);
        if (re <= e || rs > e) {  // empty row before e, or malformed pointers
            if (rs > e || re < rs) {
                flag(status, kFlagBadRowptr);
                break;
            }
            ++r;
            continue;
        }
        const int se = re < e1 ? re : e1;
        const bool split = rs < e0 || re > e1;
        if (rs < e0 && re <= e1) fix_row = r;
        typename V::Raw fr[CPL];  // FUSE: this row's slices of F
        if constexpr (FUSE) {
#pragma unroll
            for (int j = 0; j < CPL; ++j) {
                const int cc = tile0 + (j * GROUP + g) * E;
                fr[j] = V::raw(F + static_cast<long>(r) * ldf + (cc < N ? cc : 0));
            }
        }
        float acc[CPL][E];
#pragma unroll
        for (int j = 0; j < CPL; ++j) {
            const int cc = tile0 + (j * GROUP + g) * E;
#pragma unroll
            for (int i = 0; i < E; ++i)
                acc[j][i] = (!split && beta != 0.0f && cc < N) ? beta * C[r * ldc + cc + i] : 0.0f;
        }
        for (int base = e; base < se; base += GROUP) {
            const int ee = base + g;
            int k = -1;
            float v = 0.0f;
            if (ee < se) {
                k = ld_stream(colind + ee);
                v = to_f32(ld_stream(val + ee));
                if (static_cast<unsigned>(k) >= static_cast<unsigned>(K)) {
                    flag(status, kFlagBadColind);
                    k = -1;
                }
            }
            const int cnt = min(GROUP, se - base);
            int t = 0;
            // U entries per step, loads before FMAs (as in the row-split kernels: fp32 with
            // per-load predicates, bf16 packed until the mixed-precision FMA)
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
                            const int cc = tile0 + (j * GROUP + g) * E;
                            if (cc < N && kk[u] >= 0) {
                                V::load(brow + cc, b[u][j]);
                            } else {
#pragma unroll
                                for (int i = 0; i < E; ++i) b[u][j][i] = 0.0f;
                            }
                        }
                    }
#pragma unroll
                    for (int u = 0; u < U; ++u)
                        if (kk[u] >= 0)
#pragma unroll
                            for (int j = 0; j < CPL; ++j) fma_vec_f32<E>(b[u][j], vv[u], acc[j]);
                    if constexpr (FUSE) {
                        float d[U];
#pragma unroll
                        for (int u = 0; u < U; ++u) {
                            d[u] = 0.0f;
#pragma unroll
                            for (int j = 0; j < CPL; ++j)
                                if (tile0 + (j * GROUP + g) * E < N)
#pragma unroll
                                    for (int i = 0; i < E; ++i)
                                        d[u] = fmaf(b[u][j][i], V::at(fr[j], i), d[u]);
                        }
                        write_dots<U, GROUP>(d, kk, gmask, g, base + t, nnz, perm, dA, status);
                    }
                } else {
                    typename V::Raw b[U][CPL];
#pragma unroll
                    for (int u = 0; u < U; ++u) {
                        const T *brow = B + static_cast<long>(kk[u] < 0 ? 0 : kk[u]) * ldb;
#pragma unroll
                        for (int j = 0; j < CPL; ++j) {
                            const int cc = tile0 + (j * GROUP + g) * E;
                            b[u][j] = V::raw(brow + (cc < N ? cc : 0));
                        }
                    }
#pragma unroll
                    for (int u = 0; u < U; ++u) {
                        if (kk[u] < 0) continue;
                        const unsigned short vu = static_cast<unsigned short>(__float_as_uint(vv[u]) >> 16);
#pragma unroll
                        for (int j = 0; j < CPL; ++j) V::fma(b[u][j], vu, acc[j]);
                    }
                    if constexpr (FUSE) {
                        float d[U];
#pragma unroll
                        for (int u = 0; u < U; ++u) {
                            d[u] = 0.0f;
#pragma unroll
                            for (int j = 0; j < CPL; ++j)
                                if (tile0 + (j * GROUP + g) * E < N) V::dot(b[u][j], fr[j], d[u]);
                        }
                        write_dots<U, GROUP>(d, kk, gmask, g, base + t, nnz, perm, dA, status);
                    }
                }
            }
            for (; t < cnt; ++t) {
                const int kk = __shfl_sync(gmask, k, t, GROUP);
                const float vv = __shfl_sync(gmask, v, t, GROUP);
                if (kk < 0) continue;
                float d = 0.0f;
#pragma unroll
                for (int j = 0; j < CPL; ++j) {
                    const int cc = tile0 + (j * GROUP + g) * E;
                    if (cc < N) {
                        float b[E];
                        V::load(B + static_cast<long>(kk) * ldb + cc, b);
#pragma unroll
                        for (int i = 0; i < E; ++i) acc[j][i] = fmaf(b[i], vv, acc[j][i]);
                        if constexpr (FUSE) {
#pragma unroll
                            for (int i = 0; i < E; ++i) d = fmaf(b[i], V::at(fr[j], i), d);
                        }
                    }
                }
                if constexpr (FUSE) {
#pragma unroll
                    for (int off = GROUP / 2; off >= 1; off >>= 1)
                        d += __shfl_xor_sync(gmask, d, off, GROUP);
                    if (g == 0) store_dot(base + t, d, nnz, perm, dA, status);
                }
            }
        }
        float *dst = split ? carry + (2 * chunk + (e == e0 ? 0 : 1)) * static_cast<long>(N)
                           : C + r * ldc;
#pragma unroll
        for (int j = 0; j < CPL; ++j) {
            const int cc = tile0 + (j * GROUP + g) * E;
            if (cc < N) {
                if (!split && C16) {
                    store_bf16<E>(C16 + r * ldc + cc, acc[j], relu);
                } else {
#pragma unroll
                    for (int i = 0; i < E; ++i) dst[cc + i] = acc[j][i];
                }
            }
        }
        e = se;
        ++r;
    }
    if (blockIdx.y == 0 && g == 0) fix[chunk] = fix_row;
}

// Multi-entry form, for narrow rows of B (GROUP * E < 32 lanes' worth): a warp takes a chunk,
// and its S = 32 / GROUP sub-groups of GROUP lanes take every S-th entry of each row segment
// (sub-group s: entries s, s + S, s + 2S, ... of each 32-entry block), so one load
// instruction brings S entries' rows and the broadcasts, addresses and loop control are shared
// by S entries. A sub-group chains its entries in CSR order; at the segment's end the S partial
// sums are added by a butterfly over the sub-groups (lane l adds lane l ^ off, off = GROUP ..
// 16), then beta * C. Deterministic, but not the single CSR chain of the other kernels. Carry
// slots, fix-up and empty rows as in spmm_nnzsplit; FUSE as there (each dot product over one
// sub-group's GROUP lanes), with one column tile.
template <int U, int GROUP>
__device__ __forceinline__ void write_dots_me(float (&d)[U], const int (&kk)[U], unsigned gmask,
                                              int g, int e0, int stride, int nnz,
                                              const int *__restrict__ perm, float *__restrict__ dA,
                                              unsigned *status) {
    unsigned ok = 0;
#pragma unroll
    for (int u = 0; u < U; ++u) ok |= (kk[u] >= 0 ? 1u : 0u) << u;
    const float sum = reduce_entries<U, GROUP>(d, gmask, g);
    constexpr int SUB = GROUP / U;
    const int u = g / SUB;
    if (g % SUB == 0 && ((ok >> u) & 1u)) store_dot(e0 + stride * u, sum, nnz, perm, dA, status);
}

template <typename T, int VB, int GROUP, int U, bool FUSE>
__global__ void __launch_bounds__(kThreads)
spmm_nnzme(int M, int K, int N, int nnz, int CH, const int *__restrict__ rowptr,
           const int *__restrict__ colind, const T *__restrict__ val, const T *__restrict__ B,
           long ldb, float *__restrict__ C, long ldc, float beta, float *__restrict__ carry,
           int *__restrict__ fix, unsigned *status, const T *__restrict__ F, long ldf,
           const int *__restrict__ perm, float *__restrict__ dA, uint16_t *__restrict__ C16,
           bool relu) {
    using V = Vec<T, VB>;
    constexpr int E = V::E;
    constexpr int S = 32 / GROUP;
    constexpr int TILE = GROUP * E;
    static_assert(S >= 1 && U <= GROUP, "shape");
    const int lane = threadIdx.x & 31;
    const int g = lane % GROUP, sg = lane / GROUP;
    const unsigned gmask =
        GROUP == 32 ? 0xffffffffu : (((1u << GROUP) - 1u) << (lane & ~(GROUP - 1)));
    const long chunk = static_cast<long>(blockIdx.x) * (kThreads / 32) + threadIdx.x / 32;
    const long e0l = chunk * CH;
    if (e0l >= nnz) return;  // the whole warp leaves together
    const int e0 = static_cast<int>(e0l);
    const int e1 = static_cast<int>(e0l + CH < nnz ? e0l + CH : nnz);
    const int cc = blockIdx.y * TILE + g * E;  // this lane's columns
    const bool col_ok = cc < N;
    int r = find_row(rowptr, M, e0);
    int e = e0;
    int fix_row = -1;
    while (e < e1 && r < M) {  // uniform across the warp
        const int rs = __ldg(rowptr + r), re = __ldg(rowptr + r + 1);
        if (re <= e || rs > e) {
            if (rs > e || re < rs) {
                flag(status, kFlagBadRowptr);
                break;
            }
            ++r;
            continue;
        }
        const int se = re < e1 ? re : e1;
        const bool split = rs < e0 || re > e1;
        if (rs < e0 && re <= e1) fix_row = r;
        typename V::Raw fr;  // FUSE: this row's slice of F
        if constexpr (FUSE) fr = V::raw(F + static_cast<long>(r) * ldf + (col_ok ? cc : 0));
        float acc[E];
#pragma unroll
        for (int i = 0; i < E; ++i) acc[i] = 0.0f;
        for (int base = e; base < se; base += 32) {
            const int ee = base + lane;
            int k = -1;
            float v = 0.0f;
            if (ee < se) {
                k = ld_stream(colind + ee);
                v = to_f32(ld_stream(val + ee));
                if (static_cast<unsigned>(k) >= static_cast<unsigned>(K)) {
                    flag(status, kFlagBadColind);
                    k = -1;
                }
            }
            const int cnt = min(32, se - base);
            for (int t = 0; t < cnt; t += S * U) {  // sub-group sg: entries t + sg + S*u
                int kk[U];
                float vv[U];
#pragma unroll
                for (int u = 0; u < U; ++u) {
                    const int j = t + sg + S * u;
                    kk[u] = __shfl_sync(0xffffffffu, k, j & 31);
                    vv[u] = __shfl_sync(0xffffffffu, v, j & 31);
                    if (j >= cnt) kk[u] = -1;
                }
                if constexpr (sizeof(T) == 4) {
                    float b[U][E];
#pragma unroll
                    for (int u = 0; u < U; ++u) {
                        if (col_ok && kk[u] >= 0) {
                            V::load(B + static_cast<long>(kk[u]) * ldb + cc, b[u]);
                        } else {
#pragma unroll
                            for (int i = 0; i < E; ++i) b[u][i] = 0.0f;
                        }
                    }
#pragma unroll
                    for (int u = 0; u < U; ++u)
                        if (kk[u] >= 0) fma_vec_f32<E>(b[u], vv[u], acc);
                    if constexpr (FUSE) {
                        float d[U];
#pragma unroll
                        for (int u = 0; u < U; ++u) {
                            d[u] = 0.0f;
                            if (col_ok)
#pragma unroll
                                for (int i = 0; i < E; ++i) d[u] = fmaf(b[u][i], V::at(fr, i), d[u]);
                        }
                        write_dots_me<U, GROUP>(d, kk, gmask, g, base + t + sg, S, nnz, perm, dA,
                                                status);
                    }
                } else {
                    typename V::Raw b[U];
#pragma unroll
                    for (int u = 0; u < U; ++u)  // branch-free: a skipped entry reads row 0
                        b[u] = V::raw(B + static_cast<long>(kk[u] < 0 ? 0 : kk[u]) * ldb +
                                      (col_ok ? cc : 0));
#pragma unroll
                    for (int u = 0; u < U; ++u) {
                        if (kk[u] < 0) continue;
                        const unsigned short vu =
                            static_cast<unsigned short>(__float_as_uint(vv[u]) >> 16);
                        V::fma(b[u], vu, acc);
                    }
                    if constexpr (FUSE) {
                        float d[U];
#pragma unroll
                        for (int u = 0; u < U; ++u) {
                            d[u] = 0.0f;
                            if (col_ok) V::dot(b[u], fr, d[u]);
                        }
                        write_dots_me<U, GROUP>(d, kk, gmask, g, base + t + sg, S, nnz, perm, dA,
                                                status);
                    }
                }
            }
        }
#pragma unroll
        for (int off = GROUP; off < 32; off <<= 1)  // the sub-groups' partial sums
#pragma unroll
            for (int i = 0; i < E; ++i) acc[i] += __shfl_xor_sync(0xffffffffu, acc[i], off);
        if (sg == 0 && col_ok) {
            if (split) {
                float *dst = carry + (2 * chunk + (e == e0 ? 0 : 1)) * static_cast<long>(N) + cc;
#pragma unroll
                for (int i = 0; i < E; ++i) dst[i] = acc[i];
            } else if (C16) {
                store_bf16<E>(C16 + r * ldc + cc, acc, relu);
            } else {
                float *dst = C + r * ldc + cc;
#pragma unroll
                for (int i = 0; i < E; ++i) dst[i] = beta != 0.0f ? fmaf(beta, dst[i], acc[i]) : acc[i];
            }
        }
        e = se;
        ++r;
    }
    if (blockIdx.y == 0 && lane == 0) fix[chunk] = fix_row;
}

constexpr int kShortSpan = 8;  // rows over at most this many chunks: the one-pass fix-up
constexpr int kFixBatch = 8;  // partial loads in flight per thread on a long span (16 measured slower)

template <int VW>
struct Lanes;  // VW consecutive fp32 columns of a carry row, one load
template <>
struct Lanes<4> {
    __device__ static void load(const float *p, float *v) {
        const float4 t = *reinterpret_cast<const float4 *>(p);
        v[0] = t.x; v[1] = t.y; v[2] = t.z; v[3] = t.w;
    }
};
template <>
struct Lanes<1> {
    __device__ static void load(const float *p, float *v) { v[0] = *p; }
};

// Rows that end in chunk c after starting in an earlier chunk: sum their partials. A CTA takes
// kFixChunks consecutive chunks, one per warp.
//  - A row over at most kShortSpan chunks (nearly all of them): the chunk's warp alone, each
//    lane VW columns at a time, the chunks' partials loaded together and added in chunk order.
//  - A longer row, afterwards with the whole CTA: the threads split into R consecutive runs of
//    the row's chunks times groups of VW columns (R = threads / column groups, so all threads
//    load at once); each sums its run in chunk order, kFixBatch loads in flight, and the runs
//    are then added in run order.
// Both orders are fixed by the row's span and N, so the result is deterministic. (One row of a
// power-law graph can span thousands of chunks: that CTA is the fix-up's critical path. One
// CTA per chunk made the many short fix-ups cost more in CTA launches than in loads.)
constexpr int kFixChunks = kThreads / 32;

template <int VW>
__device__ __forceinline__ void store_out(float *C, uint16_t *C16, long off, float beta, float v,
                                          bool relu) {
    if (C16)
        C16[off] = f32_to_bf16(relu_if(v, relu));
    else
        C[off] = beta == 0.0f ? v : fmaf(beta, C[off], v);
}

template <int VW>
__global__ void __launch_bounds__(kThreads)
spmm_nnz_fixup(int M, int N, long nchunks, int CH, const int *__restrict__ rowptr,
               const float *__restrict__ carry, const int *__restrict__ fix,
               float *__restrict__ C, long ldc, float beta, uint16_t *__restrict__ C16,
               bool relu) {
    __shared__ float part[kThreads * VW];
    __shared__ int long_rows[kFixChunks];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // the chunk's row to fix (-1: none) and its span
    auto span = [&](long chunk, int &r, int &rs, long &c_first, long &n) {
        r = chunk < nchunks ? fix[chunk] : -1;  // recorded by the first pass
        if (r < 0 || r >= M) {
            r = -1;
            return;
        }
        rs = __ldg(rowptr + r);
        c_first = rs / CH;
        n = chunk - c_first + 1;
    };
    // slot 1 holds the first chunk's partial when the row starts inside that chunk
    auto row_of = [&](long cc, long c_first, int rs) {
        return (2 * cc + ((cc == c_first && static_cast<long>(rs) != cc * CH) ? 1 : 0)) *
               static_cast<long>(N);
    };
    {
        int r, rs = 0;
        long c_first = 0, n = 0;
        span(static_cast<long>(blockIdx.x) * kFixChunks + warp, r, rs, c_first, n);
        if (lane == 0) long_rows[warp] = r >= 0 && n > kShortSpan;
        if (r >= 0 && n <= kShortSpan) {
            for (int col = lane * VW; col < N; col += 32 * VW) {
                float v[kShortSpan][VW];
#pragma unroll
                for (int i = 0; i < kShortSpan; ++i) {
                    if (i < n) {
                        Lanes<VW>::load(carry + row_of(c_first + i, c_first, rs) + col, v[i]);
                    } else {
#pragma unroll
                        for (int j = 0; j < VW; ++j) v[i][j] = 0.0f;
                    }
                }
#pragma unroll
                for (int j = 0; j < VW; ++j) {
                    float acc = v[0][j];
#pragma unroll
                    for (int i = 1; i < kShortSpan; ++i)
                        if (i < n) acc += v[i][j];
                    store_out<VW>(C, C16, r * ldc + col + j, beta, acc, relu);
                }
            }
        }
    }
    __syncthreads();
    for (int w = 0; w < kFixChunks; ++w) {
        if (!long_rows[w]) continue;  // shared: the same for the whole CTA
        int r, rs = 0;
        long c_first = 0, n = 0;
        span(static_cast<long>(blockIdx.x) * kFixChunks + w, r, rs, c_first, n);
        const int ncg = N / VW;  // column groups (the launcher guarantees N % VW == 0)
        for (int cg0 = 0; cg0 < ncg; cg0 += kThreads) {
            const int cgs = min(kThreads, ncg - cg0);
            const int R = kThreads / cgs;
            const int run = threadIdx.x / cgs, gi = threadIdx.x % cgs;
            const int col = (cg0 + gi) * VW;
            float acc[VW];
#pragma unroll
            for (int j = 0; j < VW; ++j) acc[j] = 0.0f;
            if (run < R) {
                const long b0 = c_first + n * run / R, b1 = c_first + n * (run + 1) / R;
                for (long cc = b0; cc < b1; cc += kFixBatch) {
                    float v[kFixBatch][VW];
#pragma unroll
                    for (int i = 0; i < kFixBatch; ++i) {
                        if (cc + i < b1) {
                            Lanes<VW>::load(carry + row_of(cc + i, c_first, rs) + col, v[i]);
                        } else {
#pragma unroll
                            for (int j = 0; j < VW; ++j) v[i][j] = 0.0f;
                        }
                    }
#pragma unroll
                    for (int i = 0; i < kFixBatch; ++i)
                        if (cc + i < b1)
#pragma unroll
                            for (int j = 0; j < VW; ++j) acc[j] += v[i][j];
                }
#pragma unroll
                for (int j = 0; j < VW; ++j) part[(run * cgs + gi) * VW + j] = acc[j];
            }
            __syncthreads();
            if (run == 0) {
#pragma unroll
                for (int j = 0; j < VW; ++j) {
                    float t = part[gi * VW + j];
                    for (int q = 1; q < R; ++q) t += part[(q * cgs + gi) * VW + j];
                    store_out<VW>(C, C16, r * ldc + col + j, beta, t, relu);
                }
            }
            __syncthreads();  // part[] is reused by the next column block or row
        }
    }
}

// Rows without entries get beta * C. A warp checks 32 consecutive rows with one load each and
// writes only the empty ones, 32 columns at a time.
__global__ void __launch_bounds__(kThreads)
spmm_empty_rows(int M, int N, const int *__restrict__ rowptr, float *__restrict__ C, long ldc,
                float beta, uint16_t *__restrict__ C16) {
    const long base = (static_cast<long>(blockIdx.x) * (kThreads / 32) + (threadIdx.x >> 5)) * 32;
    const int lane = threadIdx.x & 31;
    if (base >= M) return;  // the same for the whole warp
    const long r = base + lane;
    const bool empty = r < M && __ldg(rowptr + r) == __ldg(rowptr + r + 1);
    for (unsigned m = __ballot_sync(0xffffffffu, empty); m; m &= m - 1) {
        const long rr = base + (__ffs(m) - 1);
        for (int col = lane; col < N; col += 32) {
            if (C16)
                C16[rr * ldc + col] = 0;
            else
                C[rr * ldc + col] = beta == 0.0f ? 0.0f : beta * C[rr * ldc + col];
        }
    }
}

// ME: the multi-entry kernel (spmm_nnzme, CPL 1); else spmm_nnzsplit.
template <typename T, int VB, int G, int CPL, int U, bool FUSE, bool ME = false>
as_status launch(as_ctx *ctx, const SpmmArgs &a, int CH, const SddmmFuse *fu, cudaStream_t s) {
    static_assert(!ME || CPL == 1, "multi-entry kernels hold one vector per lane");
    constexpr int E = Vec<T, VB>::E;
    constexpr int TILE = G * E * CPL;
    const int esz = sizeof(T);
    if ((a.N % E) || (a.ldb % E) || (reinterpret_cast<uintptr_t>(a.B) % (E * esz)))
        return fail(AS_ERR_UNSUPPORTED, "spmm nnz-split: layout does not fit the vector width");
    if (ceil_div(a.N, TILE) > 65535 || ceil_div(a.N, 32) > 65535)
        return fail(AS_ERR_UNSUPPORTED, "spmm nnz-split: N too large");
    if (a.C16 && (a.beta != 0.0f || (a.ldc % E) ||
                  (reinterpret_cast<uintptr_t>(a.C16) % (2 * E > 16 ? 16 : 2 * E))))
        return fail(AS_ERR_UNSUPPORTED,
                    "spmm nnz-split: bf16 output needs beta = 0 and C aligned to the vectors");
    if (FUSE && (a.N > TILE || (fu->ldf % E) || (reinterpret_cast<uintptr_t>(fu->F) % (E * esz))))
        return fail(AS_ERR_UNSUPPORTED,
                    "spmm+sddmm: the variant's column tile must cover N, F aligned to its vectors");
    const long nchunks = ceil_div(a.nnz, CH);
    void *w = nullptr;
    const size_t carry_bytes = (sizeof(float) * static_cast<size_t>(2 * nchunks) * a.N + 255) & ~size_t(255);
    as_status st = scratch(ctx, carry_bytes + sizeof(int) * static_cast<size_t>(nchunks), &w);
    if (st != AS_OK) return st;
    float *carry = static_cast<float *>(w);
    int *fix = reinterpret_cast<int *>(static_cast<char *>(w) + carry_bytes);
    if (nchunks > 0) {
        if constexpr (ME) {
            dim3 g1(static_cast<unsigned>(ceil_div(nchunks, kThreads / 32)),
                    static_cast<unsigned>(ceil_div(a.N, TILE)));
            spmm_nnzme<T, VB, G, U, FUSE><<<g1, kThreads, 0, s>>>(
                a.M, a.K, a.N, a.nnz, CH, a.rowptr, a.colind, static_cast<const T *>(a.val),
                static_cast<const T *>(a.B), a.ldb, a.C, a.ldc, a.beta, carry, fix, a.status,
                FUSE ? static_cast<const T *>(fu->F) : nullptr, FUSE ? fu->ldf : 0,
                FUSE ? fu->perm : nullptr, FUSE ? fu->dA : nullptr, a.C16, a.relu);
        } else {
            dim3 g1(static_cast<unsigned>(ceil_div(nchunks, kThreads / G)),
                    static_cast<unsigned>(ceil_div(a.N, TILE)));
            spmm_nnzsplit<T, VB, G, CPL, U, FUSE><<<g1, kThreads, 0, s>>>(
                a.M, a.K, a.N, a.nnz, CH, a.rowptr, a.colind, static_cast<const T *>(a.val),
                static_cast<const T *>(a.B), a.ldb, a.C, a.ldc, a.beta, carry, fix, a.status,
                FUSE ? static_cast<const T *>(fu->F) : nullptr, FUSE ? fu->ldf : 0,
                FUSE ? fu->perm : nullptr, FUSE ? fu->dA : nullptr, a.C16, a.relu);
        }
        dim3 g2(static_cast<unsigned>(ceil_div(nchunks, kFixChunks)));
        if (a.N % 4 == 0)  // carry rows are 16-byte aligned: whole-vector loads
            spmm_nnz_fixup<4><<<g2, kThreads, 0, s>>>(a.M, a.N, nchunks, CH, a.rowptr, carry, fix,
                                                      a.C, a.ldc, a.beta, a.C16, a.relu);
        else
            spmm_nnz_fixup<1><<<g2, kThreads, 0, s>>>(a.M, a.N, nchunks, CH, a.rowptr, carry, fix,
                                                      a.C, a.ldc, a.beta, a.C16, a.relu);
        ctx->launches += 2;
    }
    spmm_empty_rows<<<static_cast<unsigned>(ceil_div(a.M, kThreads)), kThreads, 0, s>>>(
        a.M, a.N, a.rowptr, a.C, a.ldc, a.beta, a.C16);
    ctx->launches++;
    return check_cuda(cudaGetLastError(), "spmm nnz-split launch");
}

template <typename T, int VB, int G, int CPL>
as_status launch_u(as_ctx *ctx, const SpmmArgs &a, int CH, int unroll, const SddmmFuse *fu,
                   cudaStream_t s) {
    if (fu)
        return unroll == 8 ? launch<T, VB, G, CPL, 8, true>(ctx, a, CH, fu, s)
                           : launch<T, VB, G, CPL, 4, true>(ctx, a, CH, fu, s);
    return unroll == 8 ? launch<T, VB, G, CPL, 8, false>(ctx, a, CH, fu, s)
                       : launch<T, VB, G, CPL, 4, false>(ctx, a, CH, fu, s);
}

template <typename T, int VB, int G>
as_status launch_me(as_ctx *ctx, const SpmmArgs &a, int CH, const SddmmFuse *fu, cudaStream_t s) {
    return fu ? launch<T, VB, G, 1, 4, true, true>(ctx, a, CH, fu, s)
              : launch<T, VB, G, 1, 4, false, true>(ctx, a, CH, fu, s);
}

}  // namespace

as_status spmm_nnzme_launch(as_ctx *ctx, int dtype, int vb, int group, int chunk,
                            const SpmmArgs &a, cudaStream_t s, const SddmmFuse *fuse) {
#define AS_ME_CASE(T, VBV, G) \
    if (vb == VBV && group == G) return launch_me<T, VBV, G>(ctx, a, chunk, fuse, s);
    if (dtype == 0) {
        AS_ME_CASE(float, 16, 8) AS_ME_CASE(float, 16, 16) AS_ME_CASE(float, 8, 8)
        AS_ME_CASE(float, 8, 16)
    } else {
        AS_ME_CASE(uint16_t, 16, 8) AS_ME_CASE(uint16_t, 16, 16) AS_ME_CASE(uint16_t, 8, 8)
        AS_ME_CASE(uint16_t, 8, 16)
    }
#undef AS_ME_CASE
    return fail(AS_ERR_UNSUPPORTED, "spmm multi-entry: configuration not instantiated");
}

as_status spmm_nnz_launch(as_ctx *ctx, int dtype, int vb, int group, int cpl, int chunk,
                          int unroll, const SpmmArgs &a, cudaStream_t s, const SddmmFuse *fuse) {
#define AS_NNZ_CASE(T, VBV, G, C)            \
    if (vb == VBV && group == G && cpl == C) \
        return launch_u<T, VBV, G, C>(ctx, a, chunk, unroll, fuse, s);
    if (dtype == 0) {
        AS_NNZ_CASE(float, 16, 8, 1) AS_NNZ_CASE(float, 16, 16, 1) AS_NNZ_CASE(float, 16, 32, 1)
        AS_NNZ_CASE(float, 16, 32, 2) AS_NNZ_CASE(float, 4, 32, 1) AS_NNZ_CASE(float, 4, 32, 2)
    } else {
        AS_NNZ_CASE(uint16_t, 16, 8, 1) AS_NNZ_CASE(uint16_t, 16, 16, 1)
        AS_NNZ_CASE(uint16_t, 16, 32, 1) AS_NNZ_CASE(uint16_t, 16, 32, 2)
        AS_NNZ_CASE(uint16_t, 4, 32, 1) AS_NNZ_CASE(uint16_t, 4, 32, 2)
        AS_NNZ_CASE(uint16_t, 2, 32, 1) AS_NNZ_CASE(uint16_t, 2, 32, 2)
    }
#undef AS_NNZ_CASE
    return fail(AS_ERR_UNSUPPORTED, "spmm nnz-split: configuration not instantiated");
}

}  // namespace as
