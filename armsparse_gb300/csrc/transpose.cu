// CSR -> CSC transpose, CSR validation and small conversion kernels (sm_103a).
//
// Transpose = stable sort of the CSR entries by column. The CSR order is already
// row-ascending, so a stable sort by column leaves rows ascending inside every column:
// exactly the canonical CSC that scipy's tocsc() builds on the reference's GCN path
// (gcn/pytorch-custom/gcn_custom.py:52), and the order the reference's counting transpose
// (sparseTranspose.cpp:95-142) gives when its scatter runs in order. The sort is an LSD
// radix sort over 8-bit digits of the column id, ceil(log2 N / 8) passes, each pass:
//   1. tile histogram   -- each CTA counts the digits of its tile of kTile entries into
//                          hist[digit * tiles + tile] (shared-memory atomics on counts:
//                          the counts, unlike positions, do not depend on ordering);
//   2. exclusive scan   -- over hist in (digit, tile) order, giving every (digit, tile) its
//                          first output slot;
//   3. stable scatter   -- each CTA re-reads its tile in rounds of 256 entries and ranks
//                          every entry among equal digits that precede it (warp
//                          __match_any_sync + per-warp counts + a running per-digit count),
//                          parks the tile in shared memory sorted by digit, then writes
//                          key, row and value out in that order, so each digit's entries
//                          leave as one coalesced run.
// No position depends on timing, so the output is identical run to run. colptr comes
// from the sorted keys (first slot of every column). All indices stay inside their
// buffers for any input; malformed input sets the status word instead of faulting.
#include "common.cuh"
#include "internal.h"

namespace as {
namespace {

constexpr int kThreads = 256;
constexpr int kRounds = 8;
constexpr int kTile = kThreads * kRounds;  // entries per tile
constexpr int kBins = 256;
constexpr int kWarps = kThreads / 32;

// ---- exclusive scan of int32 (three phases, no cross-CTA waits) ---------------------------
constexpr int kScanItems = 8;
constexpr int kScanChunk = kThreads * kScanItems;  // 2048 per CTA

__device__ __forceinline__ int block_exclusive_scan(int v, int *smem_warp, int &total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) smem_warp[warp] = x;
    __syncthreads();
    if (warp == 0) {
        int w = lane < kWarps ? smem_warp[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, w, o);
            if (lane >= o) w += y;
        }
        if (lane < kWarps) smem_warp[lane] = w;  // inclusive warp totals
    }
    __syncthreads();
    total = smem_warp[kWarps - 1];
    const int before = warp ? smem_warp[warp - 1] : 0;
    __syncthreads();
    return before + x - v;
}

__global__ void __launch_bounds__(kThreads)
scan_reduce(const int *__restrict__ in, long n, int *__restrict__ block_sums) {
    __shared__ int sw[kWarps];
    const long base = static_cast<long>(blockIdx.x) * kScanChunk;
    int s = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        const long idx = base + static_cast<long>(i) * kThreads + threadIdx.x;
        if (idx < n) s += in[idx];
    }
    int total;
    block_exclusive_scan(s, sw, total);
    if (threadIdx.x == 0) block_sums[blockIdx.x] = total;
}

// Single CTA: exclusive scan of the block sums in place (any count, chunked).
__global__ void __launch_bounds__(kThreads) scan_block_sums(int *sums, int nb) {
    __shared__ int sw[kWarps];
    int carry = 0;
    for (int base = 0; base < nb; base += kThreads) {
        const int idx = base + threadIdx.x;
        const int v = idx < nb ? sums[idx] : 0;
        int total;
        const int ex = block_exclusive_scan(v, sw, total);
        if (idx < nb) sums[idx] = carry + ex;
        carry += total;
    }
}

__global__ void __launch_bounds__(kThreads)
scan_downsweep(const int *__restrict__ in, long n, const int *__restrict__ block_sums,
               int *__restrict__ out) {
    __shared__ int sw[kWarps];
    const long base = static_cast<long>(blockIdx.x) * kScanChunk;
    // blocked layout: thread t owns items [t*kScanItems, (t+1)*kScanItems)
    int v[kScanItems];
    int s = 0;
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        const long idx = base + static_cast<long>(threadIdx.x) * kScanItems + i;
        v[i] = idx < n ? in[idx] : 0;
        s += v[i];
    }
    int total;
    int run = block_exclusive_scan(s, sw, total) + block_sums[blockIdx.x];
#pragma unroll
    for (int i = 0; i < kScanItems; ++i) {
        const long idx = base + static_cast<long>(threadIdx.x) * kScanItems + i;
        if (idx < n) out[idx] = run;
        run += v[i];
    }
}

// ---- transpose kernels -----------------------------------------------------------------
// rowidx[e] = row of entry e. Each thread takes kExpand consecutive entries: one binary
// search over rowptr for its first entry, then it steps the row forward -- so one row with
// millions of entries is spread over many threads. An entry that no well-formed row holds
// (malformed pointers) is flagged and given row 0, so every row index written stays in [0, M)
// and no slot keeps data from an earlier call.
constexpr int kExpand = 8;
__global__ void __launch_bounds__(kThreads)
expand_rows(int M, int nnz, const int *__restrict__ rowptr, int *__restrict__ rowidx,
            unsigned *status) {
    const long e0 = (static_cast<long>(blockIdx.x) * kThreads + threadIdx.x) * kExpand;
    if (e0 >= nnz) return;
    int lo = 0, hi = M;  // largest r with rowptr[r] <= e0 (rowptr monotone for valid input)
    while (hi - lo > 1) {
        const int mid = (lo + hi) >> 1;
        if (__ldg(rowptr + mid) <= e0)
            lo = mid;
        else
            hi = mid;
    }
    int r = lo;
    int rs = __ldg(rowptr + r), re = __ldg(rowptr + r + 1);
    const long e1 = e0 + kExpand < nnz ? e0 + kExpand : nnz;
    for (long e = e0; e < e1; ++e) {
        while (e >= re && r + 1 < M) {  // advance to the row that holds e
            ++r;
            rs = re;
            re = __ldg(rowptr + r + 1);
        }
        if (rs < 0 || re < rs || re > nnz || e < rs || e >= re) {
            flag(status, kFlagBadRowptr);
            rowidx[e] = 0;  // malformed pointers: an in-range row, never stale scratch
            continue;
        }
        rowidx[e] = r;
    }
}

__global__ void __launch_bounds__(kThreads)
check_rowptr_ends(int M, int nnz, const int *__restrict__ rowptr, int *__restrict__ rowidx,
                  unsigned *status) {
    // rowptr[0] must be 0 and rowptr[M] == nnz; otherwise some rowidx slots would be stale:
    // zero them so the sort reads defined data, and flag.
    const int first = __ldg(rowptr), last = __ldg(rowptr + M);
    if (first != 0 || last != nnz) {
        if (blockIdx.x == 0 && threadIdx.x == 0) flag(status, kFlagBadRowptr);
        for (long e = static_cast<long>(blockIdx.x) * kThreads + threadIdx.x; e < nnz;
             e += static_cast<long>(gridDim.x) * kThreads)
            rowidx[e] = 0;
    }
}

__global__ void __launch_bounds__(kThreads)
radix_histogram(const int *__restrict__ keys, int nnz, int shift, int tiles, int N,
                int *__restrict__ hist, unsigned *status, int check_range) {
    __shared__ int h[kBins];
    h[threadIdx.x] = 0;
    __syncthreads();
    const long base = static_cast<long>(blockIdx.x) * kTile;
    int kv[kRounds];  // all of this thread's keys are loaded before any is counted
#pragma unroll
    for (int i = 0; i < kRounds; ++i) {
        const long idx = base + static_cast<long>(i) * kThreads + threadIdx.x;
        kv[i] = idx < nnz ? keys[idx] : 0;
    }
#pragma unroll
    for (int i = 0; i < kRounds; ++i) {
        const long idx = base + static_cast<long>(i) * kThreads + threadIdx.x;
        if (idx < nnz) {
            const int k = kv[i];
            if (check_range && static_cast<unsigned>(k) >= static_cast<unsigned>(N))
                flag(status, kFlagBadColind);
            atomicAdd(&h[(static_cast<unsigned>(k) >> shift) & (kBins - 1)], 1);
        }
    }
    __syncthreads();
    hist[static_cast<long>(threadIdx.x) * tiles + blockIdx.x] = h[threadIdx.x];
}

__global__ void __launch_bounds__(kThreads)
radix_scatter(const int *__restrict__ keys, const int *__restrict__ rows,
              const unsigned *__restrict__ vals, bool iota, int nnz, int shift, int tiles,
              const int *__restrict__ offsets, int *__restrict__ okeys, int *__restrict__ orows,
              unsigned *__restrict__ ovals) {
    static_assert(kBins == kThreads, "one digit per thread");
    __shared__ int run[kBins];            // running local slot per digit inside this tile
    __shared__ int start[kBins];          // first local slot of each digit in this tile
    __shared__ int goff[kBins];           // first global slot of each digit for this tile
    __shared__ int wcnt[kWarps][kBins];   // per-warp counts of the current round
    __shared__ int sw[kWarps];
    __shared__ int sk[kTile];             // the tile, sorted by digit (stable)
    __shared__ int sr[kTile];
    __shared__ unsigned sv[kTile];  // the payload: value bits or entry index
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const long base = static_cast<long>(blockIdx.x) * kTile;
    const int n_tile = static_cast<int>(nnz - base < kTile ? nnz - base : kTile);
    {   // this tile's digit counts from the scanned (digit, tile) offsets; local starts
        const long idx = static_cast<long>(threadIdx.x) * tiles + blockIdx.x;
        const int off = offsets[idx];
        const int nxt = idx + 1 < static_cast<long>(kBins) * tiles ? offsets[idx + 1] : nnz;
        int total;
        const int st = block_exclusive_scan(nxt - off, sw, total);
        goff[threadIdx.x] = off;
        start[threadIdx.x] = st;
        run[threadIdx.x] = st;
    }
    const unsigned lt_mask = (1u << lane) - 1u;
    int kr[kRounds], rr[kRounds];  // the thread's entries, loaded before the ranking rounds
    unsigned vr[kRounds];
#pragma unroll
    for (int i = 0; i < kRounds; ++i) {
        const int li = i * kThreads + threadIdx.x;
        kr[i] = 0;
        rr[i] = 0;
        vr[i] = 0u;
        if (li < n_tile) {
            kr[i] = keys[base + li];
            rr[i] = rows[base + li];
            if (vals)
                vr[i] = vals[base + li];
            else if (iota)
                vr[i] = static_cast<unsigned>(base + li);  // the entry's CSR position
        }
    }
#pragma unroll
    for (int i = 0; i < kRounds; ++i) {
        const int li = i * kThreads + threadIdx.x;
        const bool valid = li < n_tile;
        const int k = kr[i], r = rr[i];
        const unsigned v = vr[i];
        const int d = valid ? static_cast<int>((static_cast<unsigned>(k) >> shift) & (kBins - 1))
                            : kBins;  // invalid lanes get a digit of their own
#pragma unroll
        for (int w = 0; w < kWarps; ++w) wcnt[w][threadIdx.x] = 0;
        __syncthreads();
        const unsigned peers = __match_any_sync(0xffffffffu, d);
        const int rank = __popc(peers & lt_mask);
        if (valid && rank == 0) wcnt[warp][d] = __popc(peers);
        __syncthreads();
        {   // per digit: exclusive prefix over warps, then advance the running count
            const int dd = threadIdx.x;
            int acc = run[dd];
#pragma unroll
            for (int w = 0; w < kWarps; ++w) {
                const int c = wcnt[w][dd];
                wcnt[w][dd] = acc;
                acc += c;
            }
            run[dd] = acc;
        }
        __syncthreads();
        if (valid) {
            const int pos = wcnt[warp][d] + rank;
            sk[pos] = k;
            sr[pos] = r;
            sv[pos] = v;
        }
        __syncthreads();  // wcnt is cleared by the next round
    }
    // write out in local (digit-sorted) order: a digit's entries go to consecutive global
    // slots, so neighbouring threads write neighbouring addresses
    for (int p = threadIdx.x; p < n_tile; p += kThreads) {
        const int k = sk[p];
        const int d = static_cast<int>((static_cast<unsigned>(k) >> shift) & (kBins - 1));
        const int g = goff[d] + (p - start[d]);
        okeys[g] = k;
        orows[g] = sr[p];
        if (ovals) ovals[g] = sv[p];
    }
}

// colptr[c] = first slot whose key >= c, from the sorted keys.
__global__ void __launch_bounds__(kThreads)
colptr_from_keys(const int *__restrict__ skeys, int nnz, int N, int *__restrict__ colptr) {
    const long p = static_cast<long>(blockIdx.x) * kThreads + threadIdx.x;
    if (p > nnz) return;
    long kprev = p == 0 ? -1 : skeys[p - 1];
    long kcur = p == nnz ? N : skeys[p];
    if (kprev < -1) kprev = -1;
    if (kcur > N) kcur = N;
    for (long c = kprev + 1; c <= kcur; ++c) colptr[c] = static_cast<int>(p);
}

// ---- validation --------------------------------------------------------------------------
__global__ void __launch_bounds__(kThreads)
csr_validate(int n_rows, int n_cols, int nnz, const int *__restrict__ rowptr,
             const int *__restrict__ colind, int require_sorted, unsigned *result) {
    const long r = static_cast<long>(blockIdx.x) * kThreads + threadIdx.x;
    if (r == 0 && (__ldg(rowptr) != 0 || __ldg(rowptr + n_rows) != nnz)) atomicOr(result, 1u);
    if (r >= n_rows) return;
    int lo = __ldg(rowptr + r), hi = __ldg(rowptr + r + 1);
    if (hi < lo || lo < 0 || hi > nnz) {
        atomicOr(result, 2u);
        return;
    }
    int prev = -1;
    for (int e = lo; e < hi; ++e) {
        const int c = __ldg(colind + e);
        if (static_cast<unsigned>(c) >= static_cast<unsigned>(n_cols)) atomicOr(result, 4u);
        if (require_sorted && c <= prev) atomicOr(result, 8u);
        prev = c;
    }
}

__global__ void __launch_bounds__(kThreads)
f32_to_bf16_kernel(long n, const float *__restrict__ src, uint16_t *__restrict__ dst) {
    for (long i = static_cast<long>(blockIdx.x) * kThreads + threadIdx.x; i < n;
         i += static_cast<long>(gridDim.x) * kThreads)
        dst[i] = f32_to_bf16(src[i]);
}

__global__ void zero_u32(unsigned *p) { *p = 0u; }

int radix_passes(int N) {
    int bits = 0;
    while (bits < 31 && (1L << bits) < N) ++bits;
    return bits <= 8 ? 1 : (bits + 7) / 8;
}

size_t align256(size_t b) { return (b + 255) & ~size_t(255); }

}  // namespace

// Exclusive scan of n ints (in may equal out); `work` holds ceil(n / 2048) ints.
static as_status exclusive_scan(as_ctx *ctx, const int *in, int *out, long n, int *work,
                                cudaStream_t s) {
    const long nb = ceil_div(n, kScanChunk);
    if (nb == 0) return AS_OK;
    scan_reduce<<<static_cast<unsigned>(nb), kThreads, 0, s>>>(in, n, work);
    scan_block_sums<<<1, kThreads, 0, s>>>(work, static_cast<int>(nb));
    scan_downsweep<<<static_cast<unsigned>(nb), kThreads, 0, s>>>(in, n, work, out);
    ctx->launches += 3;
    return check_cuda(cudaGetLastError(), "scan launch");
}

as_status exclusive_scan_i32(as_ctx *ctx, const int *in, int *out, long n, cudaStream_t s) {
    void *w = nullptr;
    as_status st = scratch(ctx, sizeof(int) * static_cast<size_t>(ceil_div(n, kScanChunk) + 1), &w);
    if (st != AS_OK) return st;
    return exclusive_scan(ctx, in, out, n, static_cast<int *>(w), s);
}

size_t csr2csc_scratch_bytes(int nnz, int N, bool with_val) {
    const long tiles = ceil_div(nnz, kTile);
    const long hist = tiles * kBins;
    size_t b = 0;
    b += align256(sizeof(int) * static_cast<size_t>(nnz));        // rowidx
    b += 2 * align256(sizeof(int) * static_cast<size_t>(nnz));    // keys ping-pong
    b += align256(sizeof(int) * static_cast<size_t>(nnz));        // rows (intermediate)
    if (with_val) b += align256(sizeof(float) * static_cast<size_t>(nnz));
    b += align256(sizeof(int) * static_cast<size_t>(hist));       // histogram / offsets
    b += align256(sizeof(int) * static_cast<size_t>(ceil_div(hist, kScanChunk) + 1));
    (void)N;
    return b;
}

as_status csr2csc_launch(as_ctx *ctx, int M, int N, int nnz, const int *rowptr,
                         const int *colind, const float *val, int *colptr, int *rowind,
                         float *cscval, void *work, cudaStream_t s, int *perm) {
    if (nnz == 0) {
        if (cudaMemsetAsync(colptr, 0, sizeof(int) * (static_cast<size_t>(N) + 1), s) != cudaSuccess)
            return check_cuda(cudaGetLastError(), "csr2csc memset");
        return AS_OK;
    }
    if (M == 0) return fail(AS_ERR_INVALID_CSR, "csr2csc: nnz > 0 with zero rows");
    if (N == 0) return fail(AS_ERR_INVALID_CSR, "csr2csc: nnz > 0 with zero columns");
    // the payload: the values' bits, or (perm given) each entry's CSR position
    const bool wv = val != nullptr || perm != nullptr;
    unsigned *final_v = perm ? reinterpret_cast<unsigned *>(perm)
                             : reinterpret_cast<unsigned *>(cscval);
    const int tiles = static_cast<int>(ceil_div(nnz, kTile));
    const long hist_n = static_cast<long>(tiles) * kBins;
    char *p = static_cast<char *>(work);
    auto take = [&](size_t bytes) { char *q = p; p += align256(bytes); return q; };
    int *rowidx = reinterpret_cast<int *>(take(sizeof(int) * static_cast<size_t>(nnz)));
    int *keysA = reinterpret_cast<int *>(take(sizeof(int) * static_cast<size_t>(nnz)));
    int *keysB = reinterpret_cast<int *>(take(sizeof(int) * static_cast<size_t>(nnz)));
    int *rowsT = reinterpret_cast<int *>(take(sizeof(int) * static_cast<size_t>(nnz)));
    unsigned *valsT = wv ? reinterpret_cast<unsigned *>(take(sizeof(unsigned) * static_cast<size_t>(nnz))) : nullptr;
    int *hist = reinterpret_cast<int *>(take(sizeof(int) * static_cast<size_t>(hist_n)));
    int *sums = reinterpret_cast<int *>(take(sizeof(int) * static_cast<size_t>(ceil_div(hist_n, kScanChunk) + 1)));

    const unsigned gw = static_cast<unsigned>(ceil_div(ceil_div(nnz, kExpand), kThreads));
    expand_rows<<<gw, kThreads, 0, s>>>(M, nnz, rowptr, rowidx, ctx->d_status);
    check_rowptr_ends<<<static_cast<unsigned>(ceil_div(nnz, kThreads) < 4096 ? ceil_div(nnz, kThreads) : 4096),
                        kThreads, 0, s>>>(M, nnz, rowptr, rowidx, ctx->d_status);
    ctx->launches += 2;

    // Keys alternate between keysA and keysB. Rows and values of a non-last pass go to
    // either the scratch buffer or the caller's output (free until the last pass), chosen
    // backwards from the last pass so that no pass reads and writes the same buffer and
    // the last pass reads scratch and writes rowind / cscval.
    const int passes = radix_passes(N);
    const int *src_k = colind;
    const int *src_r = rowidx;
    const unsigned *src_v = perm ? nullptr : reinterpret_cast<const unsigned *>(val);
    for (int pass = 0; pass < passes; ++pass) {
        const bool last = pass == passes - 1;
        const bool to_scratch = ((passes - 1 - pass) & 1) != 0;
        int *dk = (pass & 1) ? keysB : keysA;
        int *dr = (last || !to_scratch) ? rowind : rowsT;
        unsigned *dv = wv ? ((last || !to_scratch) ? final_v : valsT) : nullptr;
        const int shift = 8 * pass;
        radix_histogram<<<tiles, kThreads, 0, s>>>(src_k, nnz, shift, tiles, N, hist,
                                                   ctx->d_status, pass == 0);
        ctx->launches++;
        as_status st = exclusive_scan(ctx, hist, hist, hist_n, sums, s);
        if (st != AS_OK) return st;
        radix_scatter<<<tiles, kThreads, 0, s>>>(src_k, src_r, src_v, perm && pass == 0, nnz,
                                                 shift, tiles, hist, dk, dr, dv);
        ctx->launches++;
        src_k = dk;
        src_r = dr;
        src_v = dv;
    }
    colptr_from_keys<<<static_cast<unsigned>(ceil_div(static_cast<long>(nnz) + 1, kThreads)),
                       kThreads, 0, s>>>(src_k, nnz, N, colptr);
    ctx->launches++;
    return check_cuda(cudaGetLastError(), "csr2csc launch");
}

as_status csr_validate_launch(as_ctx *ctx, int n_rows, int n_cols, int nnz, const int *rowptr,
                              const int *colind, int require_sorted, unsigned *result,
                              cudaStream_t s) {
    zero_u32<<<1, 1, 0, s>>>(result);
    csr_validate<<<static_cast<unsigned>(ceil_div(static_cast<long>(n_rows) + 1, kThreads)),
                   kThreads, 0, s>>>(n_rows, n_cols, nnz, rowptr, colind, require_sorted, result);
    ctx->launches += 2;
    return check_cuda(cudaGetLastError(), "csr_validate launch");
}

// dst[i] = src[idx[i]] for i < n (idx in [0, n_src); others flag and give 0): values moved
// between orderings of the same entries, e.g. from CSC to CSR order through the inverse of
// as_csr2csc_perm's permutation. Four outputs per thread: one 16-byte index load, four
// independent gathers, one 16-byte store.
__global__ void __launch_bounds__(kThreads)
gather_f32(long n, long n_src, const float *__restrict__ src, const int *__restrict__ idx,
           float *__restrict__ dst, unsigned *status) {
    const long stride = static_cast<long>(gridDim.x) * kThreads * 4;
    for (long i = (static_cast<long>(blockIdx.x) * kThreads + threadIdx.x) * 4; i < n; i += stride) {
        if (i + 4 <= n) {
            const int4 k = __ldcs(reinterpret_cast<const int4 *>(idx + i));
            const int kk[4] = {k.x, k.y, k.z, k.w};
            float v[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const bool ok = static_cast<unsigned long>(static_cast<unsigned>(kk[q])) <
                                static_cast<unsigned long>(n_src);
                if (!ok) flag(status, kFlagBadPerm);
                v[q] = ok ? __ldg(src + kk[q]) : 0.0f;
            }
            __stcs(reinterpret_cast<float4 *>(dst + i), make_float4(v[0], v[1], v[2], v[3]));
        } else {
            for (long j = i; j < n; ++j) {
                const int k = idx[j];
                const bool ok = k >= 0 && static_cast<long>(k) < n_src;
                if (!ok) flag(status, kFlagBadPerm);
                dst[j] = ok ? src[k] : 0.0f;
            }
        }
    }
}

as_status gather_f32_launch(as_ctx *ctx, long n, long n_src, const float *src, const int *idx,
                            float *dst, cudaStream_t s) {
    if (n == 0) return AS_OK;
    if (reinterpret_cast<uintptr_t>(idx) % 16 || reinterpret_cast<uintptr_t>(dst) % 16)
        return fail(AS_ERR_UNSUPPORTED, "gather_f32: idx and dst must be 16-byte aligned");
    long blocks = ceil_div(ceil_div(n, 4), kThreads);
    if (blocks > static_cast<long>(ctx->sms) * 16) blocks = static_cast<long>(ctx->sms) * 16;
    gather_f32<<<static_cast<unsigned>(blocks), kThreads, 0, s>>>(n, n_src, src, idx, dst,
                                                                  ctx->d_status);
    ctx->launches++;
    return check_cuda(cudaGetLastError(), "gather_f32 launch");
}

as_status f32_to_bf16_launch(as_ctx *ctx, long n, const float *src, uint16_t *dst,
                             cudaStream_t s) {
    long blocks = ceil_div(n, kThreads);
    if (blocks > 152L * 16) blocks = 152L * 16;
    f32_to_bf16_kernel<<<static_cast<unsigned>(blocks), kThreads, 0, s>>>(n, src, dst);
    ctx->launches++;
    return check_cuda(cudaGetLastError(), "f32_to_bf16 launch");
}

}  // namespace as

// ---- no-allocation transpose -----------------------------------------------------------------
// as_csr2csc_static: the same transpose with its scratch in a file-scope device array, for
// callers that cannot allocate device memory. The array is sized for
// AS_CSR2CSC_STATIC_MAX_NNZ entries; every GPU that loads this library holds it until the
// process exits. Host code only knows the array through the address cudaGetSymbolAddress
// returns for the current device (the symbol itself is a host-side stand-in), fetched once
// per device by the first call on that device and kept for the life of the process.
#include <mutex>

namespace as {
namespace {

constexpr size_t align256c(size_t b) { return (b + 255) & ~size_t(255); }
constexpr long kStaticTiles = (AS_CSR2CSC_STATIC_MAX_NNZ + kTile - 1) / kTile;
constexpr long kStaticHist = kStaticTiles * kBins;
constexpr size_t kStaticScratchBytes =
    5 * align256c(sizeof(int) * static_cast<size_t>(AS_CSR2CSC_STATIC_MAX_NNZ)) +
    align256c(sizeof(int) * static_cast<size_t>(kStaticHist)) +
    align256c(sizeof(int) * static_cast<size_t>((kStaticHist + kScanChunk - 1) / kScanChunk + 1));
constexpr int kStaticMaxDevices = 64;

}  // namespace

static __device__ __align__(256) unsigned char g_csr2csc_static_scratch[kStaticScratchBytes];
static __device__ unsigned g_csr2csc_static_status;

namespace {

struct StaticSlot {
    bool ready = false;
    unsigned char *scratch = nullptr;
    unsigned *status = nullptr;
};
std::mutex g_static_mu;
StaticSlot g_static_slots[kStaticMaxDevices];

// Device addresses of the static scratch and status word on the current device.
cudaError_t static_slot(int dev, StaticSlot *out) {
    std::lock_guard<std::mutex> lock(g_static_mu);
    StaticSlot &s = g_static_slots[dev];
    if (!s.ready) {
        void *p = nullptr, *q = nullptr;
        cudaError_t e = cudaGetSymbolAddress(&p, g_csr2csc_static_scratch);
        if (e != cudaSuccess) return e;
        e = cudaGetSymbolAddress(&q, g_csr2csc_static_status);
        if (e != cudaSuccess) return e;
        s.scratch = static_cast<unsigned char *>(p);
        s.status = static_cast<unsigned *>(q);
        s.ready = true;
    }
    *out = s;
    return cudaSuccess;
}

// The launch sequence of csr2csc_launch, reporting through cudaError_t only.
cudaError_t csr2csc_static_run(int M, int N, int nnz, const int *rowptr, const int *colind,
                               const float *val, int *colptr, int *rowind, float *cscval,
                               unsigned char *work, unsigned *status, cudaStream_t s) {
    const bool wv = val != nullptr;
    const int tiles = static_cast<int>(ceil_div(nnz, kTile));
    const long hist_n = static_cast<long>(tiles) * kBins;
    const size_t cap = align256c(sizeof(int) * static_cast<size_t>(AS_CSR2CSC_STATIC_MAX_NNZ));
    int *rowidx = reinterpret_cast<int *>(work);
    int *keysA = reinterpret_cast<int *>(work + cap);
    int *keysB = reinterpret_cast<int *>(work + 2 * cap);
    int *rowsT = reinterpret_cast<int *>(work + 3 * cap);
    float *valsT = reinterpret_cast<float *>(work + 4 * cap);
    int *hist = reinterpret_cast<int *>(work + 5 * cap);
    int *sums = reinterpret_cast<int *>(work + 5 * cap + align256c(sizeof(int) * kStaticHist));

    const unsigned gw = static_cast<unsigned>(ceil_div(ceil_div(nnz, kExpand), kThreads));
    expand_rows<<<gw, kThreads, 0, s>>>(M, nnz, rowptr, rowidx, status);
    const long cb = ceil_div(nnz, kThreads);
    check_rowptr_ends<<<static_cast<unsigned>(cb < 4096 ? cb : 4096), kThreads, 0, s>>>(
        M, nnz, rowptr, rowidx, status);
    const int passes = radix_passes(N);
    const int *src_k = colind;
    const int *src_r = rowidx;
    const unsigned *src_v = reinterpret_cast<const unsigned *>(val);  // value bits, moved as is
    const long nb = ceil_div(hist_n, kScanChunk);
    for (int pass = 0; pass < passes; ++pass) {
        const bool last = pass == passes - 1;
        const bool to_scratch = ((passes - 1 - pass) & 1) != 0;
        int *dk = (pass & 1) ? keysB : keysA;
        int *dr = (last || !to_scratch) ? rowind : rowsT;
        unsigned *dv = wv ? reinterpret_cast<unsigned *>((last || !to_scratch) ? cscval : valsT)
                          : nullptr;
        const int shift = 8 * pass;
        radix_histogram<<<tiles, kThreads, 0, s>>>(src_k, nnz, shift, tiles, N, hist, status,
                                                   pass == 0);
        scan_reduce<<<static_cast<unsigned>(nb), kThreads, 0, s>>>(hist, hist_n, sums);
        scan_block_sums<<<1, kThreads, 0, s>>>(sums, static_cast<int>(nb));
        scan_downsweep<<<static_cast<unsigned>(nb), kThreads, 0, s>>>(hist, hist_n, sums, hist);
        radix_scatter<<<tiles, kThreads, 0, s>>>(src_k, src_r, src_v, false, nnz, shift, tiles,
                                                 hist, dk, dr, dv);
        src_k = dk;
        src_r = dr;
        src_v = dv;
    }
    colptr_from_keys<<<static_cast<unsigned>(ceil_div(static_cast<long>(nnz) + 1, kThreads)),
                       kThreads, 0, s>>>(src_k, nnz, N, colptr);
    return cudaGetLastError();
}

}  // namespace
}  // namespace as

extern "C" as_status as_csr2csc_static(int M, int N, int nnz, const int *rowptr,
                                       const int *colind, const float *val, int *colptr,
                                       int *rowind, float *cscval, void *stream) {
    using namespace as;
    if (M < 0 || N < 0 || nnz < 0) return AS_ERR_INVALID_VALUE;
    if (nnz > AS_CSR2CSC_STATIC_MAX_NNZ) return AS_ERR_UNSUPPORTED;
    if (!rowptr || !colptr || (nnz > 0 && (!colind || !rowind))) return AS_ERR_INVALID_VALUE;
    if ((val == nullptr) != (cscval == nullptr)) return AS_ERR_INVALID_VALUE;
    if (nnz > 0 && (M == 0 || N == 0)) return AS_ERR_INVALID_CSR;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return AS_ERR_CUDA;
    if (dev < 0 || dev >= kStaticMaxDevices) return AS_ERR_UNSUPPORTED;
    // a launch error left pending by earlier, unrelated work would otherwise be returned as this
    // call's: take it off first, so the status below belongs to this call's own launches
    (void)cudaGetLastError();
    StaticSlot slot;
    if (static_slot(dev, &slot) != cudaSuccess) return AS_ERR_CUDA;
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    // slot.status only gives the kernels a word to flag malformed input into; nothing reads it
    // (the entry point reports argument errors only), so it is not reset between calls
    if (nnz == 0) {
        return cudaMemsetAsync(colptr, 0, sizeof(int) * (static_cast<size_t>(N) + 1), s) ==
                       cudaSuccess
                   ? AS_OK
                   : AS_ERR_CUDA;
    }
    return csr2csc_static_run(M, N, nnz, rowptr, colind, val, colptr, rowind, cscval,
                              slot.scratch, slot.status, s) == cudaSuccess
               ? AS_OK
               : AS_ERR_CUDA;
}
