// Host-pointer shims with the reference drivers' signatures (include/armsparse_drivers.h).
// Each call: copy the host arrays to cached device buffers, run the kernel through the C
// ABI, copy the result back, wait. The process-wide state is guarded by one mutex.
#include <cuda_runtime.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <atomic>
#include <mutex>
#include <thread>
#include <vector>

#include "armsparse_drivers.h"

namespace {

constexpr int kColBlocks = 8;  // at most this many SpMM column blocks (B in, kernel, C out)
constexpr size_t kMinBlockBytes = size_t(16) << 20;  // each block's columns of B: >= 16 MB
                                                     // (4 blocks at 4096 x 4096: 0.74 ms a
                                                     // call, against 0.78 with 2 or 8)
constexpr int kColAlign = 32;  // block widths in columns (128-byte aligned fp32 starts)

struct State {
    std::mutex mu;
    as_ctx *ctx = nullptr;
    cudaStream_t stream = nullptr;
    cudaStream_t in_stream = nullptr;    // host -> device copies of column blocks
    cudaStream_t copy_stream = nullptr;  // device -> host copies of finished column blocks
    cudaEvent_t in_done[kColBlocks] = {};  // column block j's inputs are on the device
    cudaEvent_t done[kColBlocks] = {};     // column block j's kernels have finished
    void *buf = nullptr;
    size_t cap = 0;
    as_status last = AS_OK;
};

State &state() {
    static State s;
    return s;
}

as_status report(State &s, as_status st, const char *fn) {
    s.last = st;
    if (st != AS_OK) fprintf(stderr, "armsparse %s: %s: %s\n", fn, as_status_string(st), as_last_error());
    return st;
}

// Lazily creates the context/stream on the current device and grows the device arena.
as_status prepare(State &s, size_t bytes, char **base) {
    if (!s.ctx) {
        int dev = 0;
        cudaGetDevice(&dev);
        as_status st = as_ctx_create(&s.ctx, dev);
        if (st != AS_OK) return st;
        if (cudaStreamCreateWithFlags(&s.stream, cudaStreamNonBlocking) != cudaSuccess ||
            cudaStreamCreateWithFlags(&s.in_stream, cudaStreamNonBlocking) != cudaSuccess ||
            cudaStreamCreateWithFlags(&s.copy_stream, cudaStreamNonBlocking) != cudaSuccess)
            return AS_ERR_CUDA;
        for (int j = 0; j < kColBlocks; ++j)
            if (cudaEventCreateWithFlags(&s.in_done[j], cudaEventDisableTiming) != cudaSuccess ||
                cudaEventCreateWithFlags(&s.done[j], cudaEventDisableTiming) != cudaSuccess)
                return AS_ERR_CUDA;
    }
    if (bytes > s.cap) {
        if (s.buf) cudaFree(s.buf);
        s.buf = nullptr;
        s.cap = 0;
        if (cudaMalloc(&s.buf, bytes) != cudaSuccess) {
            cudaGetLastError();
            return AS_ERR_ALLOC;
        }
        s.cap = bytes;
    }
    *base = static_cast<char *>(s.buf);
    return AS_OK;
}

size_t al(size_t b) { return (b + 255) & ~size_t(255); }

struct Arena {
    char *p;
    template <typename T>
    T *take(size_t n) {
        T *q = reinterpret_cast<T *>(p);
        p += al(n * sizeof(T));
        return q;
    }
};

as_status h2d(State &s, void *d, const void *h, size_t bytes) {
    if (bytes == 0) return AS_OK;
    return cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, s.stream) == cudaSuccess ? AS_OK
                                                                                           : AS_ERR_CUDA;
}

as_status finish(State &s, void *h, const void *d, size_t bytes) {
    if (bytes && cudaMemcpyAsync(h, d, bytes, cudaMemcpyDeviceToHost, s.stream) != cudaSuccess)
        return AS_ERR_CUDA;
    if (cudaStreamSynchronize(s.stream) != cudaSuccess) return AS_ERR_CUDA;
    return as_ctx_sync_status(s.ctx, s.stream);
}

as_status spmm_host(const int *rowPtr, const int *colInd, const float *val, const float *B,
                    float *C, int M, int K, int N, float beta) {
    State &s = state();
    if (M < 0 || K < 0 || N < 0 || !rowPtr) return AS_ERR_INVALID_VALUE;
    const int nnz = rowPtr[M];
    if (nnz < 0) return AS_ERR_INVALID_CSR;
    const size_t bytes = al(sizeof(int) * (M + 1)) + 2 * al(sizeof(int) * nnz) +
                         al(sizeof(float) * size_t(K) * N) + al(sizeof(float) * size_t(M) * N);
    char *base = nullptr;
    as_status st = prepare(s, bytes, &base);
    if (st != AS_OK) return st;
    Arena a{base};
    int *drp = a.take<int>(M + 1);
    int *dci = a.take<int>(nnz);
    float *dv = a.take<float>(nnz);
    float *dB = a.take<float>(size_t(K) * N);
    float *dC = a.take<float>(size_t(M) * N);
    // Column blocks. Block j's columns of B (and of C, when accumulating) go in, its kernel
    // runs, and its columns of C come back; copies of pageable memory hold the calling thread
    // until they finish, so the copies back run on a helper thread while this one copies the
    // next blocks in: the link then carries both directions at once. Each block is the same
    // library call on a column slice (B and C offsets, ldb = ldc = N), so every output is the
    // same fused chain as in one call.
    const size_t b_bytes = sizeof(float) * size_t(K) * N;
    int blocks = int(std::max<size_t>(1, std::min<size_t>(kColBlocks, b_bytes / kMinBlockBytes)));
    const int width = std::max(kColAlign, (N + blocks - 1) / blocks + kColAlign - 1) / kColAlign * kColAlign;
    blocks = N > 0 ? (N + width - 1) / width : 1;
    auto copy2d = [&](float *dst, const float *src, int c0, int w, int rows, cudaMemcpyKind kind,
                      cudaStream_t str) {
        return cudaMemcpy2DAsync(dst + c0, sizeof(float) * size_t(N), src + c0,
                                 sizeof(float) * size_t(N), sizeof(float) * size_t(w), rows, kind,
                                 str) == cudaSuccess;
    };
    auto in = [&](void *d, const void *h, size_t bytes) {
        return bytes == 0 || cudaMemcpyAsync(d, h, bytes, cudaMemcpyHostToDevice, s.in_stream) ==
                                 cudaSuccess;
    };
    if (!in(drp, rowPtr, sizeof(int) * (M + 1)) || !in(dci, colInd, sizeof(int) * nnz) ||
        !in(dv, val, sizeof(float) * nnz)) {
        cudaStreamSynchronize(s.in_stream);
        return AS_ERR_CUDA;
    }
    // the helper: copies block j back once its kernel was enqueued (`enqueued` > j); stops
    // after `enqueued` blocks once `last` is set
    std::atomic<int> enqueued{0};
    std::atomic<bool> last{false};
    std::atomic<bool> out_ok{true};
    int dev = 0;
    cudaGetDevice(&dev);
    auto copy_back = [&]() {
        cudaSetDevice(dev);
        for (int j = 0;; ++j) {
            while (enqueued.load() <= j && !last.load()) std::this_thread::yield();
            if (enqueued.load() <= j) break;
            const int c0 = j * width, w = std::min(width, N - c0);
            if (cudaStreamWaitEvent(s.copy_stream, s.done[j], 0) != cudaSuccess ||
                (M > 0 && w > 0 && !copy2d(C, dC, c0, w, M, cudaMemcpyDeviceToHost, s.copy_stream)))
                out_ok = false;
        }
        if (cudaStreamSynchronize(s.copy_stream) != cudaSuccess) out_ok = false;
    };
    std::thread helper;
    if (blocks > 1) {
        try {
            helper = std::thread(copy_back);
        } catch (...) {  // no thread: the copies back run after the loop, on this thread
        }
    }
    for (int j = 0; j < blocks && st == AS_OK; ++j) {
        const int c0 = j * width, w = std::min(width, N - c0);
        if (K > 0 && w > 0 && !copy2d(dB, B, c0, w, K, cudaMemcpyHostToDevice, s.in_stream)) st = AS_ERR_CUDA;
        if (st == AS_OK && beta != 0.0f && M > 0 && w > 0 &&
            !copy2d(dC, C, c0, w, M, cudaMemcpyHostToDevice, s.in_stream))
            st = AS_ERR_CUDA;
        if (st == AS_OK && (cudaEventRecord(s.in_done[j], s.in_stream) != cudaSuccess ||
                            cudaStreamWaitEvent(s.stream, s.in_done[j], 0) != cudaSuccess))
            st = AS_ERR_CUDA;
        if (st == AS_OK)
            st = as_spmm_csr_f32(s.ctx, M, K, w, nnz, drp, dci, dv, dB + c0, N, dC + c0, N, beta,
                                 0, s.stream);
        if (st == AS_OK && cudaEventRecord(s.done[j], s.stream) != cudaSuccess) st = AS_ERR_CUDA;
        if (st == AS_OK) enqueued = j + 1;
    }
    last = true;
    if (helper.joinable()) {
        helper.join();
    } else {
        copy_back();  // one block: the copy back on this thread
    }
    // all three streams drain before the call returns, whatever happened
    const bool in_synced = cudaStreamSynchronize(s.in_stream) == cudaSuccess;
    if (st != AS_OK) {
        cudaStreamSynchronize(s.stream);
        return st;
    }
    if (!in_synced || !out_ok.load()) return AS_ERR_CUDA;
    return finish(s, nullptr, nullptr, 0);
}

as_status spgemm_host(const int *rp1, const int *ci1, const float *v1, const int *rp2,
                      const int *ci2, const float *v2, float *C, int M, int K, int N) {
    State &s = state();
    if (M < 0 || K < 0 || N < 0 || !rp1 || !rp2) return AS_ERR_INVALID_VALUE;
    const int nnz_a = rp1[M], nnz_b = rp2[K];
    if (nnz_a < 0 || nnz_b < 0) return AS_ERR_INVALID_CSR;
    const size_t bytes = al(sizeof(int) * (M + 1)) + 2 * al(sizeof(int) * nnz_a) +
                         al(sizeof(int) * (K + 1)) + 2 * al(sizeof(int) * nnz_b) +
                         al(sizeof(float) * size_t(M) * N);
    char *base = nullptr;
    as_status st = prepare(s, bytes, &base);
    if (st != AS_OK) return st;
    Arena a{base};
    int *drp1 = a.take<int>(M + 1);
    int *dci1 = a.take<int>(nnz_a);
    float *dv1 = a.take<float>(nnz_a);
    int *drp2 = a.take<int>(K + 1);
    int *dci2 = a.take<int>(nnz_b);
    float *dv2 = a.take<float>(nnz_b);
    float *dC = a.take<float>(size_t(M) * N);
    if ((st = h2d(s, drp1, rp1, sizeof(int) * (M + 1))) != AS_OK) return st;
    if ((st = h2d(s, dci1, ci1, sizeof(int) * nnz_a)) != AS_OK) return st;
    if ((st = h2d(s, dv1, v1, sizeof(float) * nnz_a)) != AS_OK) return st;
    if ((st = h2d(s, drp2, rp2, sizeof(int) * (K + 1))) != AS_OK) return st;
    if ((st = h2d(s, dci2, ci2, sizeof(int) * nnz_b)) != AS_OK) return st;
    if ((st = h2d(s, dv2, v2, sizeof(float) * nnz_b)) != AS_OK) return st;
    if ((st = h2d(s, dC, C, sizeof(float) * size_t(M) * N)) != AS_OK) return st;
    st = as_spgemm_csr_dense_f32(s.ctx, M, K, N, nnz_a, drp1, dci1, dv1, nnz_b, drp2, dci2, dv2,
                                 dC, N, 1.0f, s.stream);
    if (st != AS_OK) return st;
    return finish(s, C, dC, sizeof(float) * size_t(M) * N);
}

}  // namespace

void sparse_matrix_mul3(int rowPtr1[], int colInd1[], float val1[], int rowPtr2[],
                        int colInd2[], float val2[], float *matrixC, int M, int K, int N,
                        int threads) {
    (void)threads;
    State &s = state();
    std::lock_guard<std::mutex> g(s.mu);
    report(s, spgemm_host(rowPtr1, colInd1, val1, rowPtr2, colInd2, val2, matrixC, M, K, N),
           "sparse_matrix_mul3");
}

void rowBaseSpmm3(int rowPtr[], int colInd[], float val[], float B[], float C[], int M, int K,
                  int N, int threads) {
    (void)threads;
    State &s = state();
    std::lock_guard<std::mutex> g(s.mu);
    report(s, spmm_host(rowPtr, colInd, val, B, C, M, K, N, 1.0f), "rowBaseSpmm3");
}

void rowBaseSpmm2(int rowPtr[], int colInd[], float val[], float B[], float C[], int M, int K,
                  int N, int threads) {
    (void)threads;
    State &s = state();
    std::lock_guard<std::mutex> g(s.mu);
    report(s, spmm_host(rowPtr, colInd, val, B, C, M, K, N, 1.0f), "rowBaseSpmm2");
}

void origin(int rowPtr[], int colInd[], float val[], float B[], float C[], int M, int K, int N,
            int threads) {
    (void)threads;
    State &s = state();
    std::lock_guard<std::mutex> g(s.mu);
    report(s, spmm_host(rowPtr, colInd, val, B, C, M, K, N, 0.0f), "origin");
}

void csr_spmm_kernel(int A_nrows, int B_ncols, int *A_csrRowPtr, int *A_csrColInd,
                     float *A_csrVal, float *B_dnVal, float *C_dnVal) {
    State &s = state();
    std::lock_guard<std::mutex> g(s.mu);
    int K = 0;
    if (A_csrRowPtr && A_nrows > 0) {
        const int nnz = A_csrRowPtr[A_nrows];
        for (int e = 0; e < nnz; ++e) K = std::max(K, A_csrColInd[e] + 1);
    }
    report(s, spmm_host(A_csrRowPtr, A_csrColInd, A_csrVal, B_dnVal, C_dnVal, A_nrows, K, B_ncols,
                        1.0f),
           "csr_spmm_kernel");
}

void sparse_dense_vector(float *B, float *C, int rowPtr[], int colInd[], float val[], int M,
                         int threads) {
    (void)threads;
    State &s = state();
    std::lock_guard<std::mutex> g(s.mu);
    auto run = [&]() -> as_status {
        if (M < 0 || !rowPtr) return AS_ERR_INVALID_VALUE;
        const int ns = rowPtr[M];
        int K = 0;
        for (int e = 0; e < ns; e += 4) K = std::max(K, colInd[e] + 4);
        const size_t bytes = al(sizeof(int) * (M + 1)) + 2 * al(sizeof(int) * ns) +
                             al(sizeof(float) * K) + al(sizeof(float) * M);
        char *base = nullptr;
        as_status st = prepare(s, bytes, &base);
        if (st != AS_OK) return st;
        Arena a{base};
        int *drp = a.take<int>(M + 1);
        int *dci = a.take<int>(ns);
        float *dv = a.take<float>(ns);
        float *dx = a.take<float>(K);
        float *dy = a.take<float>(M);
        if ((st = h2d(s, drp, rowPtr, sizeof(int) * (M + 1))) != AS_OK) return st;
        if ((st = h2d(s, dci, colInd, sizeof(int) * ns)) != AS_OK) return st;
        if ((st = h2d(s, dv, val, sizeof(float) * ns)) != AS_OK) return st;
        if ((st = h2d(s, dx, B, sizeof(float) * K)) != AS_OK) return st;
        if ((st = h2d(s, dy, C, sizeof(float) * M)) != AS_OK) return st;
        st = as_spmv_vcsr4_f32(s.ctx, M, K, ns, drp, dci, dv, dx, dy, 1.0f, s.stream);
        if (st != AS_OK) return st;
        return finish(s, C, dy, sizeof(float) * M);
    };
    report(s, run(), "sparse_dense_vector");
}

void DataReuseSpmm(int rowPtr[], int colInd[], float val[], float B[], float C[], int M, int K,
                   int N, int threads, bool *flag) {
    (void)threads;
    State &s = state();
    std::lock_guard<std::mutex> g(s.mu);
    auto run = [&]() -> as_status {
        if (M < 0 || K < 0 || N < 0 || !rowPtr) return AS_ERR_INVALID_VALUE;
        const int nnz = rowPtr[M];
        if (nnz < 0) return AS_ERR_INVALID_CSR;
        const size_t bytes = al(sizeof(int) * (M + 1)) + 2 * al(sizeof(int) * nnz) + al(nnz) +
                             al(sizeof(float) * size_t(K) * N) + al(sizeof(float) * size_t(M) * N);
        char *base = nullptr;
        as_status st = prepare(s, bytes, &base);
        if (st != AS_OK) return st;
        Arena a{base};
        int *drp = a.take<int>(M + 1);
        int *dci = a.take<int>(nnz);
        float *dv = a.take<float>(nnz);
        uint8_t *df = a.take<uint8_t>(nnz);
        float *dB = a.take<float>(size_t(K) * N);
        float *dC = a.take<float>(size_t(M) * N);
        static_assert(sizeof(bool) == 1, "the reference's flag array is one byte per entry");
        if ((st = h2d(s, drp, rowPtr, sizeof(int) * (M + 1))) != AS_OK) return st;
        if ((st = h2d(s, dci, colInd, sizeof(int) * nnz)) != AS_OK) return st;
        if ((st = h2d(s, dv, val, sizeof(float) * nnz)) != AS_OK) return st;
        if ((st = h2d(s, df, flag, size_t(nnz))) != AS_OK) return st;
        if ((st = h2d(s, dB, B, sizeof(float) * size_t(K) * N)) != AS_OK) return st;
        if ((st = h2d(s, dC, C, sizeof(float) * size_t(M) * N)) != AS_OK) return st;
        st = as_spmm_rowpair_f32(s.ctx, M, K, N, nnz, drp, dci, dv, df, dB, N, dC, N, 1.0f,
                                 s.stream);
        if (st != AS_OK) return st;
        return finish(s, C, dC, sizeof(float) * size_t(M) * N);
    };
    report(s, run(), "DataReuseSpmm");
}

void toDataReuseFormat(float *matrix, int rows, int cols, int *rowPtr, int *colInd, float *val,
                       bool *flag) {
    State &s = state();
    std::lock_guard<std::mutex> g(s.mu);
    auto run = [&]() -> as_status {
        if (rows < 0 || cols < 0 || !matrix || !rowPtr) return AS_ERR_INVALID_VALUE;
        const size_t dense = sizeof(float) * size_t(rows) * cols;
        // dense -> CSR (count, then fill once nnz is known) -> row-pair layout
        const size_t head = al(dense) + 2 * al(sizeof(int) * (size_t(rows) + 1));
        char *base = nullptr;
        as_status st = prepare(s, head, &base);
        if (st != AS_OK) return st;
        Arena a{base};
        float *dD = a.take<float>(size_t(rows) * cols);
        int *drp = a.take<int>(size_t(rows) + 1);
        int *drp2 = a.take<int>(size_t(rows) + 1);
        if ((st = h2d(s, dD, matrix, dense)) != AS_OK) return st;
        if ((st = as_dense_to_csr_count(s.ctx, rows, cols, dD, cols, drp, s.stream)) != AS_OK)
            return st;
        int nnz = 0;
        if (cudaMemcpyAsync(&nnz, drp + rows, sizeof(int), cudaMemcpyDeviceToHost, s.stream) !=
                cudaSuccess ||
            cudaStreamSynchronize(s.stream) != cudaSuccess)
            return AS_ERR_CUDA;
        // the arena may grow: keep the dense matrix and row pointers by recopying into it
        const size_t need = head + 4 * al(sizeof(int) * size_t(nnz)) + al(size_t(nnz));
        if (need > s.cap) {
            std::vector<int> hrp(size_t(rows) + 1);
            if (cudaMemcpy(hrp.data(), drp, sizeof(int) * hrp.size(), cudaMemcpyDeviceToHost) !=
                cudaSuccess)
                return AS_ERR_CUDA;
            if ((st = prepare(s, need, &base)) != AS_OK) return st;
            a = Arena{base};
            dD = a.take<float>(size_t(rows) * cols);
            drp = a.take<int>(size_t(rows) + 1);
            drp2 = a.take<int>(size_t(rows) + 1);
            if ((st = h2d(s, dD, matrix, dense)) != AS_OK) return st;
            if ((st = h2d(s, drp, hrp.data(), sizeof(int) * hrp.size())) != AS_OK) return st;
        }
        int *dci = a.take<int>(nnz);
        float *dv = a.take<float>(nnz);
        int *dci2 = a.take<int>(nnz);
        float *dv2 = a.take<float>(nnz);
        uint8_t *df = a.take<uint8_t>(nnz);
        if ((st = as_dense_to_csr_fill(s.ctx, rows, cols, dD, cols, drp, dci, dv, s.stream)) != AS_OK)
            return st;
        if ((st = as_csr_to_rowpair_count(s.ctx, rows, nnz, drp, dci, drp2, s.stream)) != AS_OK)
            return st;
        if ((st = as_csr_to_rowpair_fill(s.ctx, rows, nnz, drp, dci, dv, drp2, dci2, dv2, df,
                                         s.stream)) != AS_OK)
            return st;
        if (cudaMemcpyAsync(rowPtr, drp2, sizeof(int) * (size_t(rows) + 1), cudaMemcpyDeviceToHost,
                            s.stream) != cudaSuccess ||
            (nnz && (cudaMemcpyAsync(colInd, dci2, sizeof(int) * nnz, cudaMemcpyDeviceToHost,
                                     s.stream) != cudaSuccess ||
                     cudaMemcpyAsync(val, dv2, sizeof(float) * nnz, cudaMemcpyDeviceToHost,
                                     s.stream) != cudaSuccess ||
                     cudaMemcpyAsync(flag, df, size_t(nnz), cudaMemcpyDeviceToHost, s.stream) !=
                         cudaSuccess)))
            return AS_ERR_CUDA;
        if ((st = finish(s, nullptr, nullptr, 0)) != AS_OK) return st;
        // as the reference does, the entries moved into the previous row's segment are zeroed
        // in the dense matrix
        for (int r = 0; r + 1 < rows; r += 2)
            for (int e = rowPtr[r]; e < rowPtr[r + 1]; ++e)
                if (flag[e]) matrix[size_t(r + 1) * cols + colInd[e]] = 0.0f;
        return AS_OK;
    };
    report(s, run(), "toDataReuseFormat");
}

static as_status transpose_host(int *sm, int *res) {
    State &s = state();
    if (!sm || !res) return AS_ERR_INVALID_VALUE;
    const int M = sm[0], N = sm[1], nnz = sm[2];
    if (M < 0 || N < 0 || nnz < 0) return AS_ERR_INVALID_VALUE;
    std::vector<int> rowptr(M + 1, 0), colind(nnz);
    std::vector<float> val(nnz);
    int prev_r = -1, prev_c = -1;
    for (int e = 0; e < nnz; ++e) {
        const int r = sm[3 * (e + 1)], c = sm[3 * (e + 1) + 1];
        if (r < 0 || r >= M || c < 0 || c >= N) return AS_ERR_INVALID_CSR;
        if (r < prev_r || (r == prev_r && c <= prev_c)) return AS_ERR_INVALID_VALUE;  // not row-major
        prev_r = r;
        prev_c = c;
        rowptr[r + 1]++;
        colind[e] = c;
        memcpy(&val[e], &sm[3 * (e + 1) + 2], sizeof(float));  // int payload moves bit-exactly
    }
    for (int r = 0; r < M; ++r) rowptr[r + 1] += rowptr[r];
    const size_t bytes = al(sizeof(int) * (M + 1)) + al(sizeof(int) * nnz) + al(sizeof(float) * nnz) +
                         al(sizeof(int) * (N + 1)) + al(sizeof(int) * nnz) + al(sizeof(float) * nnz);
    char *base = nullptr;
    as_status st = prepare(s, bytes, &base);
    if (st != AS_OK) return st;
    Arena a{base};
    int *drp = a.take<int>(M + 1);
    int *dci = a.take<int>(nnz);
    float *dv = a.take<float>(nnz);
    int *dcp = a.take<int>(N + 1);
    int *dri = a.take<int>(nnz);
    float *dcv = a.take<float>(nnz);
    if ((st = h2d(s, drp, rowptr.data(), sizeof(int) * (M + 1))) != AS_OK) return st;
    if ((st = h2d(s, dci, colind.data(), sizeof(int) * nnz)) != AS_OK) return st;
    if ((st = h2d(s, dv, val.data(), sizeof(float) * nnz)) != AS_OK) return st;
    st = as_csr2csc(s.ctx, M, N, nnz, drp, dci, dv, dcp, dri, dcv, s.stream);
    if (st != AS_OK) return st;
    std::vector<int> colptr(N + 1), rowind(nnz);
    std::vector<float> cval(nnz);
    if (cudaMemcpyAsync(colptr.data(), dcp, sizeof(int) * (N + 1), cudaMemcpyDeviceToHost, s.stream) != cudaSuccess ||
        cudaMemcpyAsync(rowind.data(), dri, sizeof(int) * nnz, cudaMemcpyDeviceToHost, s.stream) != cudaSuccess)
        return AS_ERR_CUDA;
    if ((st = finish(s, cval.data(), dcv, sizeof(float) * nnz)) != AS_OK) return st;
    res[0] = N;
    res[1] = M;
    res[2] = nnz;
    for (int c = 0; c < N; ++c)
        for (int p = colptr[c]; p < colptr[c + 1]; ++p) {
            res[3 * (p + 1)] = c;
            res[3 * (p + 1) + 1] = rowind[p];
            memcpy(&res[3 * (p + 1) + 2], &cval[p], sizeof(int));
        }
    return AS_OK;
}

void fast_transpose(int *sm, int *res, std::mutex mtx[]) {
    (void)mtx;
    State &s = state();
    std::lock_guard<std::mutex> g(s.mu);
    report(s, transpose_host(sm, res), "fast_transpose");
}

extern "C" {
void as_drv_rowBaseSpmm3(int *rowPtr, int *colInd, float *val, float *B, float *C, int M, int K,
                         int N, int threads) {
    rowBaseSpmm3(rowPtr, colInd, val, B, C, M, K, N, threads);
}
void as_drv_rowBaseSpmm2(int *rowPtr, int *colInd, float *val, float *B, float *C, int M, int K,
                         int N, int threads) {
    rowBaseSpmm2(rowPtr, colInd, val, B, C, M, K, N, threads);
}
void as_drv_origin(int *rowPtr, int *colInd, float *val, float *B, float *C, int M, int K, int N,
                   int threads) {
    origin(rowPtr, colInd, val, B, C, M, K, N, threads);
}
void as_drv_sparse_matrix_mul3(int *rowPtr1, int *colInd1, float *val1, int *rowPtr2,
                               int *colInd2, float *val2, float *C, int M, int K, int N,
                               int threads) {
    sparse_matrix_mul3(rowPtr1, colInd1, val1, rowPtr2, colInd2, val2, C, M, K, N, threads);
}
void as_drv_sparse_dense_vector(float *B, float *C, int *rowPtr, int *colInd, float *val, int M,
                                int threads) {
    sparse_dense_vector(B, C, rowPtr, colInd, val, M, threads);
}
void as_drv_csr_spmm_kernel(int A_nrows, int B_ncols, int *rowptr, int *colind, float *val,
                            float *B, float *C) {
    csr_spmm_kernel(A_nrows, B_ncols, rowptr, colind, val, B, C);
}
void as_drv_fast_transpose(int *sm, int *res) { fast_transpose(sm, res, nullptr); }
void as_drv_DataReuseSpmm(int *rowPtr, int *colInd, float *val, float *B, float *C, int M, int K,
                          int N, int threads, unsigned char *flag) {
    DataReuseSpmm(rowPtr, colInd, val, B, C, M, K, N, threads, reinterpret_cast<bool *>(flag));
}
void as_drv_toDataReuseFormat(float *matrix, int rows, int cols, int *rowPtr, int *colInd,
                              float *val, unsigned char *flag) {
    toDataReuseFormat(matrix, rows, cols, rowPtr, colInd, val, reinterpret_cast<bool *>(flag));
}
as_status as_drv_last_status(void) { return state().last; }
}
