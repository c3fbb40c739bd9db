// C-ABI entry points (include/armsparse_gpu.h): argument checks, context, dispatch.
#include <stdio.h>

#include <string>

#include "common.cuh"
#include "internal.h"

namespace as {

static thread_local std::string g_last_error = "no error";

as_status fail(as_status s, const std::string &msg) {
    g_last_error = msg;
    return s;
}

as_status check_cuda(cudaError_t e, const char *what) {
    if (e == cudaSuccess) return AS_OK;
    return fail(AS_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

as_status scratch(as_ctx *ctx, size_t bytes, void **out) {
    bytes = (bytes + 255) & ~size_t(255);
    if (bytes == 0) bytes = 256;
    if (bytes > ctx->scratch_bytes) {
        size_t grow = bytes + bytes / 4;
        void *p = nullptr;
        if (cudaMalloc(&p, grow) != cudaSuccess) {
            cudaGetLastError();
            if (cudaMalloc(&p, bytes) != cudaSuccess) {
                cudaGetLastError();
                return fail(AS_ERR_ALLOC, "scratch allocation of " + std::to_string(bytes) +
                                              " bytes failed");
            }
            grow = bytes;
        }
        if (ctx->scratch) ctx->retired.push_back(ctx->scratch);
        ctx->scratch = p;
        ctx->scratch_bytes = grow;
    }
    *out = ctx->scratch;
    return AS_OK;
}

struct DeviceGuard {
    int prev = -1;
    explicit DeviceGuard(int dev) {
        cudaGetDevice(&prev);
        if (prev != dev) cudaSetDevice(dev);
    }
    ~DeviceGuard() {
        int cur = -1;
        cudaGetDevice(&cur);
        if (prev >= 0 && cur != prev) cudaSetDevice(prev);
    }
};

static bool aligned_to(const void *p, size_t a) {
    return (reinterpret_cast<uintptr_t>(p) % a) == 0;
}

static as_status check_csr_args(const char *fn, int M, int K, int nnz, const int *rowptr,
                                const int *colind, const void *val, bool need_val) {
    if (M < 0 || K < 0 || nnz < 0)
        return fail(AS_ERR_INVALID_VALUE, std::string(fn) + ": negative size");
    if (!rowptr) return fail(AS_ERR_INVALID_VALUE, std::string(fn) + ": rowptr is NULL");
    if (nnz > 0 && !colind)
        return fail(AS_ERR_INVALID_VALUE, std::string(fn) + ": colind is NULL");
    if (need_val && nnz > 0 && !val)
        return fail(AS_ERR_INVALID_VALUE, std::string(fn) + ": val is NULL");
    if (!aligned_to(rowptr, 4) || (colind && !aligned_to(colind, 4)))
        return fail(AS_ERR_INVALID_VALUE, std::string(fn) + ": index arrays must be 4-byte aligned");
    return AS_OK;
}

}  // namespace as

using namespace as;

extern "C" {

const char *as_last_error(void) { return g_last_error.c_str(); }

const char *as_status_string(as_status s) {
    switch (s) {
        case AS_OK: return "AS_OK";
        case AS_ERR_INVALID_VALUE: return "AS_ERR_INVALID_VALUE";
        case AS_ERR_INVALID_CSR: return "AS_ERR_INVALID_CSR";
        case AS_ERR_UNSUPPORTED: return "AS_ERR_UNSUPPORTED";
        case AS_ERR_CUDA: return "AS_ERR_CUDA";
        case AS_ERR_TIMEOUT: return "AS_ERR_TIMEOUT";
        case AS_ERR_ALLOC: return "AS_ERR_ALLOC";
    }
    return "AS_ERR_UNKNOWN";
}

as_status as_ctx_create(as_ctx **out, int device) {
    if (!out) return fail(AS_ERR_INVALID_VALUE, "as_ctx_create: out is NULL");
    int n = 0;
    cudaError_t e = cudaGetDeviceCount(&n);
    if (e != cudaSuccess) return check_cuda(e, "as_ctx_create: cudaGetDeviceCount");
    if (device < 0 || device >= n)
        return fail(AS_ERR_INVALID_VALUE, "as_ctx_create: no such device");
    DeviceGuard g(device);
    as_ctx *c = new as_ctx();
    c->device = device;
    e = cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, device);
    if (e != cudaSuccess) {
        delete c;
        return check_cuda(e, "as_ctx_create: multiprocessor count");
    }
    e = cudaMalloc(&c->d_status, 4 * sizeof(unsigned));
    if (e != cudaSuccess) {
        delete c;
        return check_cuda(e, "as_ctx_create: status word");
    }
    c->d_long = c->d_status + 1;
    e = cudaMemset(c->d_status, 0, 4 * sizeof(unsigned));
    if (e != cudaSuccess) {
        cudaFree(c->d_status);
        delete c;
        return check_cuda(e, "as_ctx_create: memset");
    }
    *out = c;
    return AS_OK;
}

as_status as_ctx_destroy(as_ctx *c) {
    if (!c) return AS_OK;
    DeviceGuard g(c->device);
    cudaDeviceSynchronize();
    if (c->scratch) cudaFree(c->scratch);
    for (void *p : c->retired) cudaFree(p);
    if (c->d_status) cudaFree(c->d_status);
    delete c;
    return AS_OK;
}

uint64_t as_ctx_launch_count(const as_ctx *c) { return c ? c->launches : 0; }

as_status as_ctx_set_spin_limit(as_ctx *c, unsigned polls) {
    if (!c) return fail(AS_ERR_INVALID_VALUE, "as_ctx_set_spin_limit: ctx is NULL");
    c->spin_limit = polls;
    return AS_OK;
}

as_status as_ctx_sync_status(as_ctx *c, void *stream) {
    if (!c) return fail(AS_ERR_INVALID_VALUE, "as_ctx_sync_status: ctx is NULL");
    DeviceGuard g(c->device);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    unsigned h = 0;
    cudaError_t e = cudaMemcpyAsync(&h, c->d_status, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->d_status, 0, sizeof(unsigned), s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return check_cuda(e, "as_ctx_sync_status");
    if (h & kFlagTimeout) return fail(AS_ERR_TIMEOUT, "a bounded device wait gave up");
    if (h & kFlagLongList)
        return fail(AS_ERR_CUDA, "SpMM long-row list found non-empty at the start of a call "
                                 "(an earlier call on this context failed part-way)");
    if (h & kFlagBadPerm)
        return fail(AS_ERR_INVALID_VALUE, "permutation entry out of range seen on the device");
    if (h & kFlagBadLabel)
        return fail(AS_ERR_INVALID_VALUE, "class label out of range seen on the device");
    if (h & (kFlagBadRowptr | kFlagBadColind))
        return fail(AS_ERR_INVALID_CSR,
                    (h & kFlagBadRowptr) ? "malformed rowptr seen on the device"
                                         : "column index out of range seen on the device");
    return AS_OK;
}

as_status as_csr_validate(as_ctx *c, int n_rows, int n_cols, int nnz, const int *rowptr,
                          const int *colind, int require_sorted, void *stream) {
    if (!c) return fail(AS_ERR_INVALID_VALUE, "as_csr_validate: ctx is NULL");
    as_status st = check_csr_args("as_csr_validate", n_rows, n_cols, nnz, rowptr, colind,
                                  nullptr, false);
    if (st != AS_OK) return st;
    DeviceGuard g(c->device);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    void *w = nullptr;
    if ((st = scratch(c, sizeof(unsigned), &w)) != AS_OK) return st;
    unsigned *res = static_cast<unsigned *>(w);
    st = csr_validate_launch(c, n_rows, n_cols, nnz, rowptr, colind, require_sorted, res, s);
    if (st != AS_OK) return st;
    unsigned h = 0;
    cudaError_t e = cudaMemcpyAsync(&h, res, sizeof(unsigned), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) return check_cuda(e, "as_csr_validate");
    if (h & 1u) return fail(AS_ERR_INVALID_CSR, "rowptr[0] != 0 or rowptr[n_rows] != nnz");
    if (h & 2u) return fail(AS_ERR_INVALID_CSR, "rowptr is not non-decreasing");
    if (h & 4u) return fail(AS_ERR_INVALID_CSR, "column index out of range");
    if (h & 8u) return fail(AS_ERR_INVALID_CSR, "columns not strictly ascending in a row");
    return AS_OK;
}

static as_status spmm_common(const char *fn, int dtype, as_ctx *c, int M, int K, int N, int nnz,
                             const int *rowptr, const int *colind, const void *val,
                             const void *B, long ldb, float *C, long ldc, float beta,
                             int variant, void *stream, uint16_t *C16 = nullptr,
                             bool relu = false) {
    if (!c) return fail(AS_ERR_INVALID_VALUE, std::string(fn) + ": ctx is NULL");
    as_status st = check_csr_args(fn, M, K, nnz, rowptr, colind, val, true);
    if (st != AS_OK) return st;
    if (N < 0) return fail(AS_ERR_INVALID_VALUE, std::string(fn) + ": negative N");
    if (M == 0 || N == 0) return AS_OK;
    if (nnz > 0 && K == 0)  // every entry's column would be out of range (B has no rows)
        return fail(AS_ERR_INVALID_CSR, std::string(fn) + ": entries in a matrix without columns");
    if (!C && !C16) return fail(AS_ERR_INVALID_VALUE, std::string(fn) + ": C is NULL");
    if (K > 0 && nnz > 0 && !B) return fail(AS_ERR_INVALID_VALUE, std::string(fn) + ": B is NULL");
    if (ldb < N || ldc < N)
        return fail(AS_ERR_INVALID_VALUE, std::string(fn) + ": leading dimension below N");
    if (variant < 0 || variant > spmm_variant_count(dtype))
        return fail(AS_ERR_INVALID_VALUE, std::string(fn) + ": unknown variant");
    DeviceGuard g(c->device);
    SpmmArgs a{M, K, N, nnz, rowptr, colind, val, B, ldb, C, ldc, beta, c->d_status, C16, relu};
    if (variant == 0)
        variant = spmm_default_variant(dtype, M, K, N, nnz, ldb, ldc, B,
                                       C16 ? static_cast<const void *>(C16) : C);
    return spmm_launch(c, dtype, variant, a, static_cast<cudaStream_t>(stream));
}

as_status as_spmm_csr_f32(as_ctx *c, int M, int K, int N, int nnz, const int *rowptr,
                          const int *colind, const float *val, const float *B, long ldb,
                          float *C, long ldc, float beta, int variant, void *stream) {
    return spmm_common("as_spmm_csr_f32", 0, c, M, K, N, nnz, rowptr, colind, val, B, ldb, C,
                       ldc, beta, variant, stream);
}

as_status as_spmm_csr_bf16(as_ctx *c, int M, int K, int N, int nnz, const int *rowptr,
                           const int *colind, const uint16_t *val, const uint16_t *B,
                           long ldb, float *C, long ldc, float beta, int variant,
                           void *stream) {
    return spmm_common("as_spmm_csr_bf16", 1, c, M, K, N, nnz, rowptr, colind, val, B, ldb, C,
                       ldc, beta, variant, stream);
}

static as_status spmm_sddmm_common(const char *fn, int dtype, as_ctx *c, int M, int K, int N,
                                   int nnz, const int *rowptr, const int *colind,
                                   const void *val, const void *B, long ldb, float *C, long ldc,
                                   float beta, const void *F, long ldf, const int *perm,
                                   float *dA, int variant, void *stream,
                                   uint16_t *C16 = nullptr) {
    if (!c) return fail(AS_ERR_INVALID_VALUE, std::string(fn) + ": ctx is NULL");
    as_status st = check_csr_args(fn, M, K, nnz, rowptr, colind, val, true);
    if (st != AS_OK) return st;
    if (N < 0) return fail(AS_ERR_INVALID_VALUE, std::string(fn) + ": negative N");
    if (M == 0) return AS_OK;
    if (N == 0) {  // empty dot products
        if (nnz > 0 && !dA) return fail(AS_ERR_INVALID_VALUE, std::string(fn) + ": dA is NULL");
        if (nnz == 0) return AS_OK;
        if (perm)
            return fail(AS_ERR_UNSUPPORTED, std::string(fn) + ": N = 0 with a permutation");
        DeviceGuard g(c->device);
        return check_cuda(cudaMemsetAsync(dA, 0, sizeof(float) * static_cast<size_t>(nnz),
                                          static_cast<cudaStream_t>(stream)),
                          fn);
    }
    if (nnz > 0 && K == 0)
        return fail(AS_ERR_INVALID_CSR, std::string(fn) + ": entries in a matrix without columns");
    if (!C && !C16) return fail(AS_ERR_INVALID_VALUE, std::string(fn) + ": C is NULL");
    if (nnz > 0 && (!B || !F || !dA))
        return fail(AS_ERR_INVALID_VALUE, std::string(fn) + ": B, F or dA is NULL");
    if (ldb < N || ldc < N || ldf < N)
        return fail(AS_ERR_INVALID_VALUE, std::string(fn) + ": leading dimension below N");
    if (variant < 0 || variant > spmm_variant_count(dtype))
        return fail(AS_ERR_INVALID_VALUE, std::string(fn) + ": unknown variant");
    DeviceGuard g(c->device);
    SpmmArgs a{M, K, N, nnz, rowptr, colind, val, B, ldb, C, ldc, beta, c->d_status, C16};
    SddmmFuse f{F, ldf, perm, dA};
    return spmm_sddmm_launch(c, dtype, variant, a, f, static_cast<cudaStream_t>(stream));
}

as_status as_spmm_csr_bf16_out16(as_ctx *c, int M, int K, int N, int nnz, const int *rowptr,
                                 const int *colind, const uint16_t *val, const uint16_t *B,
                                 long ldb, uint16_t *C, long ldc, int relu, int variant,
                                 void *stream) {
    return spmm_common("as_spmm_csr_bf16_out16", 1, c, M, K, N, nnz, rowptr, colind, val, B, ldb,
                       nullptr, ldc, 0.0f, variant, stream, C, relu != 0);
}

as_status as_spmm_sddmm_csr_bf16_out16(as_ctx *c, int M, int K, int N, int nnz,
                                       const int *rowptr, const int *colind,
                                       const uint16_t *val, const uint16_t *B, long ldb,
                                       uint16_t *C, long ldc, const uint16_t *F, long ldf,
                                       const int *perm, float *dA, int variant, void *stream) {
    return spmm_sddmm_common("as_spmm_sddmm_csr_bf16_out16", 1, c, M, K, N, nnz, rowptr, colind,
                             val, B, ldb, nullptr, ldc, 0.0f, F, ldf, perm, dA, variant, stream,
                             C);
}

as_status as_spmm_sddmm_csr_f32(as_ctx *c, int M, int K, int N, int nnz, const int *rowptr,
                                const int *colind, const float *val, const float *B, long ldb,
                                float *C, long ldc, float beta, const float *F, long ldf,
                                const int *perm, float *dA, int variant, void *stream) {
    return spmm_sddmm_common("as_spmm_sddmm_csr_f32", 0, c, M, K, N, nnz, rowptr, colind, val,
                             B, ldb, C, ldc, beta, F, ldf, perm, dA, variant, stream);
}

as_status as_spmm_sddmm_csr_bf16(as_ctx *c, int M, int K, int N, int nnz, const int *rowptr,
                                 const int *colind, const uint16_t *val, const uint16_t *B,
                                 long ldb, float *C, long ldc, float beta, const uint16_t *F,
                                 long ldf, const int *perm, float *dA, int variant,
                                 void *stream) {
    return spmm_sddmm_common("as_spmm_sddmm_csr_bf16", 1, c, M, K, N, nnz, rowptr, colind, val,
                             B, ldb, C, ldc, beta, F, ldf, perm, dA, variant, stream);
}

as_status as_softmax_xent_bf16(as_ctx *c, int n, int C, const uint16_t *S, long lds,
                               const int64_t *labels, float *lse, float *loss, void *stream) {
    if (!c) return fail(AS_ERR_INVALID_VALUE, "as_softmax_xent_bf16: ctx is NULL");
    if (n < 0 || lds < C || !loss || (n > 0 && (!S || !labels || !lse)))
        return fail(AS_ERR_INVALID_VALUE, "as_softmax_xent_bf16: bad arguments");
    DeviceGuard g(c->device);
    return xent_fwd_launch(c, n, C, S, lds, labels, lse, loss, static_cast<cudaStream_t>(stream));
}

as_status as_softmax_xent_bwd_bf16(as_ctx *c, int n, int C, const uint16_t *S, long lds,
                                   const int64_t *labels, const float *lse, const float *gscale,
                                   uint16_t *G, long ldg, int width, void *stream) {
    if (!c) return fail(AS_ERR_INVALID_VALUE, "as_softmax_xent_bwd_bf16: ctx is NULL");
    if (n < 0 || lds < C || ldg < width || !gscale || (n > 0 && (!S || !labels || !lse || !G)))
        return fail(AS_ERR_INVALID_VALUE, "as_softmax_xent_bwd_bf16: bad arguments");
    DeviceGuard g(c->device);
    return xent_bwd_launch(c, n, C, S, lds, labels, lse, gscale, G, ldg, width,
                           static_cast<cudaStream_t>(stream));
}

as_status as_spmm_csr_reduce_f32(as_ctx *c, int M, int K, int N, int nnz, const int *rowptr,
                                 const int *colind, const float *val, const float *B, long ldb,
                                 float *C, long ldc, int op, void *stream) {
    if (!c) return fail(AS_ERR_INVALID_VALUE, "as_spmm_csr_reduce_f32: ctx is NULL");
    as_status st = check_csr_args("as_spmm_csr_reduce_f32", M, K, nnz, rowptr, colind, nullptr, false);
    if (st != AS_OK) return st;
    if (op != AS_REDUCE_SUM && op != AS_REDUCE_MAX && op != AS_REDUCE_MAX_DGL)
        return fail(AS_ERR_INVALID_VALUE, "as_spmm_csr_reduce_f32: unknown reduction");
    if (N < 0) return fail(AS_ERR_INVALID_VALUE, "as_spmm_csr_reduce_f32: negative N");
    if (M == 0 || N == 0) return AS_OK;
    if (!C || (nnz > 0 && K > 0 && !B) || ldb < N || ldc < N)
        return fail(AS_ERR_INVALID_VALUE, "as_spmm_csr_reduce_f32: bad dense operand");
    DeviceGuard g(c->device);
    SpmmArgs a{M, K, N, nnz, rowptr, colind, val, B, ldb, C, ldc, 0.0f, c->d_status};
    return spmm_reduce_launch(c, op, a, static_cast<cudaStream_t>(stream));
}

as_status as_spgemm_csr_dense_f32(as_ctx *c, int M, int K, int N, int nnz_a,
                                  const int *a_rowptr, const int *a_colind, const float *a_val,
                                  int nnz_b, const int *b_rowptr, const int *b_colind,
                                  const float *b_val, float *C, long ldc, float beta,
                                  void *stream) {
    if (!c) return fail(AS_ERR_INVALID_VALUE, "as_spgemm_csr_dense_f32: ctx is NULL");
    as_status st = check_csr_args("as_spgemm_csr_dense_f32 (A)", M, K, nnz_a, a_rowptr, a_colind,
                                  a_val, true);
    if (st != AS_OK) return st;
    st = check_csr_args("as_spgemm_csr_dense_f32 (B)", K, N, nnz_b, b_rowptr, b_colind, b_val,
                        true);
    if (st != AS_OK) return st;
    if (N < 0) return fail(AS_ERR_INVALID_VALUE, "as_spgemm_csr_dense_f32: negative N");
    if (M == 0 || N == 0) return AS_OK;
    if (!C || ldc < N) return fail(AS_ERR_INVALID_VALUE, "as_spgemm_csr_dense_f32: bad C");
    DeviceGuard g(c->device);
    return spgemm_dense_launch(c, M, K, N, nnz_a, a_rowptr, a_colind, a_val, nnz_b, b_rowptr,
                               b_colind, b_val, C, ldc, beta, static_cast<cudaStream_t>(stream));
}

int as_spmm_variant_count(int dtype) { return spmm_variant_count(dtype); }
int as_spmm_variant_supported(int dtype, int variant, int N, long ldb, long ldc, const void *B,
                              const void *C) {
    return spmm_variant_supported(dtype, variant, N, ldb, ldc, B, C) ? 1 : 0;
}
const char *as_spmm_variant_name(int dtype, int variant) {
    return spmm_variant_name(dtype, variant);
}
int as_spmm_default_variant(int dtype, int M, int K, int N, int nnz, long ldb, long ldc,
                            const void *B, const void *C) {
    return spmm_default_variant(dtype, M, K, N, nnz, ldb, ldc, B, C);
}

as_status as_spmv_csr_f32(as_ctx *c, int M, int K, int nnz, const int *rowptr,
                          const int *colind, const float *val, const float *x, float *y,
                          float beta, void *stream) {
    if (!c) return fail(AS_ERR_INVALID_VALUE, "as_spmv_csr_f32: ctx is NULL");
    as_status st = check_csr_args("as_spmv_csr_f32", M, K, nnz, rowptr, colind, val, true);
    if (st != AS_OK) return st;
    if (M == 0) return AS_OK;
    if (!y || (nnz > 0 && !x)) return fail(AS_ERR_INVALID_VALUE, "as_spmv_csr_f32: x or y is NULL");
    DeviceGuard g(c->device);
    return spmv_csr_launch(c, M, K, nnz, rowptr, colind, val, x, y, beta,
                           static_cast<cudaStream_t>(stream));
}

as_status as_spmv_vcsr4_f32(as_ctx *c, int M, int K, int nslots, const int *rowptr,
                            const int *colind, const float *val, const float *x, float *y,
                            float beta, void *stream) {
    if (!c) return fail(AS_ERR_INVALID_VALUE, "as_spmv_vcsr4_f32: ctx is NULL");
    as_status st = check_csr_args("as_spmv_vcsr4_f32", M, K, nslots, rowptr, colind, val, true);
    if (st != AS_OK) return st;
    if (nslots % 4 != 0)
        return fail(AS_ERR_INVALID_VALUE, "as_spmv_vcsr4_f32: slot count is not a multiple of 4");
    if (M == 0) return AS_OK;
    if (!y || (nslots > 0 && !x))
        return fail(AS_ERR_INVALID_VALUE, "as_spmv_vcsr4_f32: x or y is NULL");
    DeviceGuard g(c->device);
    return spmv_vcsr4_launch(c, M, K, nslots, rowptr, colind, val, x, y, beta,
                             static_cast<cudaStream_t>(stream));
}

static as_status sddmm_common(const char *fn, bool tc, as_ctx *c, int M, int N, int K, int nnz,
                              const int *rowptr, const int *colind, const float *aval,
                              const float *X, long ldx, const float *Y, long ldy, float *out,
                              void *stream, int variant = 0) {
    if (!c) return fail(AS_ERR_INVALID_VALUE, std::string(fn) + ": ctx is NULL");
    as_status st = check_csr_args(fn, M, N, nnz, rowptr, colind, nullptr, false);
    if (st != AS_OK) return st;
    if (K < 0) return fail(AS_ERR_INVALID_VALUE, std::string(fn) + ": negative K");
    if (nnz == 0) return AS_OK;
    if (!out) return fail(AS_ERR_INVALID_VALUE, std::string(fn) + ": out is NULL");
    if (K > 0 && (!X || !Y)) return fail(AS_ERR_INVALID_VALUE, std::string(fn) + ": X or Y is NULL");
    if (ldx < K || ldy < K)
        return fail(AS_ERR_INVALID_VALUE, std::string(fn) + ": leading dimension below K");
    DeviceGuard g(c->device);
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    if (tc) {
        if (variant < 0 || variant > sddmm_tc_variant_count())
            return fail(AS_ERR_INVALID_VALUE, std::string(fn) + ": unknown variant");
        return sddmm_bf16x3_launch(c, M, N, K, nnz, rowptr, colind, aval, X, ldx, Y, ldy, out,
                                   variant, s);
    }
    return sddmm_f32_launch(c, M, N, K, nnz, rowptr, colind, aval, X, ldx, Y, ldy, out, s);
}

as_status as_sddmm_csr_f32(as_ctx *c, int M, int N, int K, int nnz, const int *rowptr,
                           const int *colind, const float *aval, const float *X, long ldx,
                           const float *Y, long ldy, float *out, void *stream) {
    return sddmm_common("as_sddmm_csr_f32", false, c, M, N, K, nnz, rowptr, colind, aval, X,
                        ldx, Y, ldy, out, stream);
}

as_status as_sddmm_csr_bf16(as_ctx *c, int M, int N, int K, int nnz, const int *rowptr,
                            const int *colind, const float *aval, const uint16_t *X, long ldx,
                            const uint16_t *Y, long ldy, float *out, void *stream) {
    const char *fn = "as_sddmm_csr_bf16";
    if (!c) return fail(AS_ERR_INVALID_VALUE, std::string(fn) + ": ctx is NULL");
    as_status st = check_csr_args(fn, M, N, nnz, rowptr, colind, nullptr, false);
    if (st != AS_OK) return st;
    if (K < 0) return fail(AS_ERR_INVALID_VALUE, std::string(fn) + ": negative K");
    if (nnz == 0) return AS_OK;
    if (!out) return fail(AS_ERR_INVALID_VALUE, std::string(fn) + ": out is NULL");
    if (K > 0 && (!X || !Y)) return fail(AS_ERR_INVALID_VALUE, std::string(fn) + ": X or Y is NULL");
    if (ldx < K || ldy < K)
        return fail(AS_ERR_INVALID_VALUE, std::string(fn) + ": leading dimension below K");
    if (!aligned_to(X, 2) || !aligned_to(Y, 2))
        return fail(AS_ERR_INVALID_VALUE, std::string(fn) + ": X and Y must be 2-byte aligned");
    DeviceGuard g(c->device);
    return sddmm_bf16_launch(c, M, N, K, nnz, rowptr, colind, aval, X, ldx, Y, ldy, out,
                             static_cast<cudaStream_t>(stream));
}

as_status as_sddmm_csr_bf16x3(as_ctx *c, int M, int N, int K, int nnz, const int *rowptr,
                              const int *colind, const float *aval, const float *X, long ldx,
                              const float *Y, long ldy, float *out, void *stream) {
    return sddmm_common("as_sddmm_csr_bf16x3", true, c, M, N, K, nnz, rowptr, colind, aval, X,
                        ldx, Y, ldy, out, stream);
}

as_status as_sddmm_csr_bf16x3_v(as_ctx *c, int M, int N, int K, int nnz, const int *rowptr,
                                const int *colind, const float *aval, const float *X, long ldx,
                                const float *Y, long ldy, float *out, int variant, void *stream) {
    return sddmm_common("as_sddmm_csr_bf16x3_v", true, c, M, N, K, nnz, rowptr, colind, aval, X,
                        ldx, Y, ldy, out, stream, variant);
}

int as_sddmm_bf16x3_variant_count(void) { return sddmm_tc_variant_count(); }

as_status as_sddmm_coo_f32(as_ctx *c, int M, int N, int K, int nnz, const int *rowind,
                           const int *colind, const float *aval, const float *X, long ldx,
                           const float *Y, long ldy, float *out, void *stream) {
    if (!c) return fail(AS_ERR_INVALID_VALUE, "as_sddmm_coo_f32: ctx is NULL");
    if (M < 0 || N < 0 || K < 0 || nnz < 0)
        return fail(AS_ERR_INVALID_VALUE, "as_sddmm_coo_f32: negative size");
    if (nnz == 0) return AS_OK;
    if (!rowind || !colind || !out)
        return fail(AS_ERR_INVALID_VALUE, "as_sddmm_coo_f32: NULL index or output array");
    if (K > 0 && (!X || !Y)) return fail(AS_ERR_INVALID_VALUE, "as_sddmm_coo_f32: X or Y is NULL");
    if (ldx < K || ldy < K)
        return fail(AS_ERR_INVALID_VALUE, "as_sddmm_coo_f32: leading dimension below K");
    DeviceGuard g(c->device);
    return sddmm_coo_f32_launch(c, M, N, K, nnz, rowind, colind, aval, X, ldx, Y, ldy, out,
                                static_cast<cudaStream_t>(stream));
}

as_status as_csr2csc(as_ctx *c, int M, int N, int nnz, const int *rowptr, const int *colind,
                     const float *val, int *colptr, int *rowind, float *cscval, void *stream) {
    if (!c) return fail(AS_ERR_INVALID_VALUE, "as_csr2csc: ctx is NULL");
    as_status st = check_csr_args("as_csr2csc", M, N, nnz, rowptr, colind, nullptr, false);
    if (st != AS_OK) return st;
    if (!colptr) return fail(AS_ERR_INVALID_VALUE, "as_csr2csc: colptr is NULL");
    if (nnz > 0 && !rowind) return fail(AS_ERR_INVALID_VALUE, "as_csr2csc: rowind is NULL");
    if ((val == nullptr) != (cscval == nullptr))
        return fail(AS_ERR_INVALID_VALUE, "as_csr2csc: val and cscval must both be given or both NULL");
    DeviceGuard g(c->device);
    void *w = nullptr;
    st = scratch(c, csr2csc_scratch_bytes(nnz, N, val != nullptr), &w);
    if (st != AS_OK) return st;
    return csr2csc_launch(c, M, N, nnz, rowptr, colind, val, colptr, rowind, cscval, w,
                          static_cast<cudaStream_t>(stream));
}

as_status as_csr2csc_perm(as_ctx *c, int M, int N, int nnz, const int *rowptr,
                          const int *colind, int *colptr, int *rowind, int *perm, void *stream) {
    if (!c) return fail(AS_ERR_INVALID_VALUE, "as_csr2csc_perm: ctx is NULL");
    as_status st = check_csr_args("as_csr2csc_perm", M, N, nnz, rowptr, colind, nullptr, false);
    if (st != AS_OK) return st;
    if (!colptr) return fail(AS_ERR_INVALID_VALUE, "as_csr2csc_perm: colptr is NULL");
    if (nnz > 0 && (!rowind || !perm))
        return fail(AS_ERR_INVALID_VALUE, "as_csr2csc_perm: rowind or perm is NULL");
    DeviceGuard g(c->device);
    void *w = nullptr;
    st = scratch(c, csr2csc_scratch_bytes(nnz, N, true), &w);
    if (st != AS_OK) return st;
    return csr2csc_launch(c, M, N, nnz, rowptr, colind, nullptr, colptr, rowind, nullptr, w,
                          static_cast<cudaStream_t>(stream), perm);
}

as_status as_spmm_csr_f64(as_ctx *c, int M, int K, int N, int nnz, const int *rowptr,
                          const int *colind, const double *val, const double *B, long ldb,
                          double *C, long ldc, double beta, void *stream) {
    if (!c) return fail(AS_ERR_INVALID_VALUE, "as_spmm_csr_f64: ctx is NULL");
    as_status st = check_csr_args("as_spmm_csr_f64", M, K, nnz, rowptr, colind, val, true);
    if (st != AS_OK) return st;
    if (N < 0) return fail(AS_ERR_INVALID_VALUE, "as_spmm_csr_f64: negative N");
    if (M == 0 || N == 0) return AS_OK;
    if (!C || (nnz > 0 && K > 0 && !B))
        return fail(AS_ERR_INVALID_VALUE, "as_spmm_csr_f64: B or C is NULL");
    if (ldb < N || ldc < N)
        return fail(AS_ERR_INVALID_VALUE, "as_spmm_csr_f64: leading dimension below N");
    DeviceGuard g(c->device);
    return spmm_f64_launch(c, M, K, N, nnz, rowptr, colind, val, B, ldb, C, ldc, beta,
                           static_cast<cudaStream_t>(stream));
}

as_status as_sddmm_csr_f64(as_ctx *c, int M, int N, int K, int nnz, const int *rowptr,
                           const int *colind, const double *aval, const double *X, long ldx,
                           const double *Y, long ldy, double *out, void *stream) {
    if (!c) return fail(AS_ERR_INVALID_VALUE, "as_sddmm_csr_f64: ctx is NULL");
    as_status st = check_csr_args("as_sddmm_csr_f64", M, N, nnz, rowptr, colind, nullptr, false);
    if (st != AS_OK) return st;
    if (K < 0) return fail(AS_ERR_INVALID_VALUE, "as_sddmm_csr_f64: negative K");
    if (nnz == 0) return AS_OK;
    if (!out || (K > 0 && (!X || !Y)))
        return fail(AS_ERR_INVALID_VALUE, "as_sddmm_csr_f64: NULL operand");
    if (ldx < K || ldy < K)
        return fail(AS_ERR_INVALID_VALUE, "as_sddmm_csr_f64: leading dimension below K");
    DeviceGuard g(c->device);
    return sddmm_f64_launch(c, M, N, K, nnz, rowptr, colind, aval, X, ldx, Y, ldy, out,
                            static_cast<cudaStream_t>(stream));
}

as_status as_dense_to_csr_count(as_ctx *c, int M, int K, const float *D, long ld, int *rowptr,
                                void *stream) {
    if (!c) return fail(AS_ERR_INVALID_VALUE, "as_dense_to_csr_count: ctx is NULL");
    if (M < 0 || K < 0 || ld < K || !rowptr || (static_cast<long>(M) * K > 0 && !D))
        return fail(AS_ERR_INVALID_VALUE, "as_dense_to_csr_count: bad arguments");
    DeviceGuard g(c->device);
    return dense_to_csr_count_launch(c, M, K, D, ld, rowptr, static_cast<cudaStream_t>(stream));
}

as_status as_dense_to_csr_fill(as_ctx *c, int M, int K, const float *D, long ld,
                               const int *rowptr, int *colind, float *val, void *stream) {
    if (!c) return fail(AS_ERR_INVALID_VALUE, "as_dense_to_csr_fill: ctx is NULL");
    if (M < 0 || K < 0 || ld < K || !rowptr || (static_cast<long>(M) * K > 0 && (!D || !colind || !val)))
        return fail(AS_ERR_INVALID_VALUE, "as_dense_to_csr_fill: bad arguments");
    if (M == 0) return AS_OK;
    DeviceGuard g(c->device);
    return dense_to_csr_fill_launch(c, M, K, D, ld, rowptr, colind, val,
                                    static_cast<cudaStream_t>(stream));
}

as_status as_csr_to_vcsr4_count(as_ctx *c, int M, int nnz, const int *rowptr, const int *colind,
                                int *vrowptr, void *stream) {
    if (!c) return fail(AS_ERR_INVALID_VALUE, "as_csr_to_vcsr4_count: ctx is NULL");
    as_status st = check_csr_args("as_csr_to_vcsr4_count", M, 0, nnz, rowptr, colind, nullptr, false);
    if (st != AS_OK) return st;
    if (!vrowptr) return fail(AS_ERR_INVALID_VALUE, "as_csr_to_vcsr4_count: vrowptr is NULL");
    DeviceGuard g(c->device);
    return csr_to_vcsr4_count_launch(c, M, nnz, rowptr, colind, vrowptr,
                                     static_cast<cudaStream_t>(stream));
}

as_status as_csr_to_vcsr4_fill(as_ctx *c, int M, int nnz, const int *rowptr, const int *colind,
                               const float *val, const int *vrowptr, int *vcolind, float *vval,
                               void *stream) {
    if (!c) return fail(AS_ERR_INVALID_VALUE, "as_csr_to_vcsr4_fill: ctx is NULL");
    as_status st = check_csr_args("as_csr_to_vcsr4_fill", M, 0, nnz, rowptr, colind, val, true);
    if (st != AS_OK) return st;
    if (!vrowptr || (nnz > 0 && (!vcolind || !vval)))
        return fail(AS_ERR_INVALID_VALUE, "as_csr_to_vcsr4_fill: NULL output");
    if (M == 0) return AS_OK;
    DeviceGuard g(c->device);
    return csr_to_vcsr4_fill_launch(c, M, nnz, rowptr, colind, val, vrowptr, vcolind, vval,
                                    static_cast<cudaStream_t>(stream));
}

as_status as_csr_to_rowpair_count(as_ctx *c, int M, int nnz, const int *rowptr,
                                  const int *colind, int *rowptr2, void *stream) {
    if (!c) return fail(AS_ERR_INVALID_VALUE, "as_csr_to_rowpair_count: ctx is NULL");
    as_status st = check_csr_args("as_csr_to_rowpair_count", M, 0, nnz, rowptr, colind, nullptr,
                                  false);
    if (st != AS_OK) return st;
    if (!rowptr2) return fail(AS_ERR_INVALID_VALUE, "as_csr_to_rowpair_count: rowptr2 is NULL");
    DeviceGuard g(c->device);
    return csr_to_rowpair_count_launch(c, M, nnz, rowptr, colind, rowptr2,
                                       static_cast<cudaStream_t>(stream));
}

as_status as_csr_to_rowpair_fill(as_ctx *c, int M, int nnz, const int *rowptr, const int *colind,
                                 const float *val, const int *rowptr2, int *colind2, float *val2,
                                 uint8_t *flag2, void *stream) {
    if (!c) return fail(AS_ERR_INVALID_VALUE, "as_csr_to_rowpair_fill: ctx is NULL");
    as_status st = check_csr_args("as_csr_to_rowpair_fill", M, 0, nnz, rowptr, colind, val, true);
    if (st != AS_OK) return st;
    if (!rowptr2 || (nnz > 0 && (!colind2 || !val2 || !flag2)))
        return fail(AS_ERR_INVALID_VALUE, "as_csr_to_rowpair_fill: NULL output");
    if (M == 0) return AS_OK;
    DeviceGuard g(c->device);
    return csr_to_rowpair_fill_launch(c, M, nnz, rowptr, colind, val, rowptr2, colind2, val2,
                                      flag2, static_cast<cudaStream_t>(stream));
}

as_status as_spmm_rowpair_f32(as_ctx *c, int M, int K, int N, int nnz, const int *rowptr2,
                              const int *colind2, const float *val2, const uint8_t *flag2,
                              const float *B, long ldb, float *C, long ldc, float beta,
                              void *stream) {
    if (!c) return fail(AS_ERR_INVALID_VALUE, "as_spmm_rowpair_f32: ctx is NULL");
    as_status st = check_csr_args("as_spmm_rowpair_f32", M, K, nnz, rowptr2, colind2, val2, true);
    if (st != AS_OK) return st;
    if (N < 0) return fail(AS_ERR_INVALID_VALUE, "as_spmm_rowpair_f32: negative N");
    if (M == 0 || N == 0) return AS_OK;
    if (!C || (nnz > 0 && (!B || !flag2)) || ldb < N || ldc < N)
        return fail(AS_ERR_INVALID_VALUE, "as_spmm_rowpair_f32: bad dense operand");
    DeviceGuard g(c->device);
    SpmmArgs a{M, K, N, nnz, rowptr2, colind2, val2, B, ldb, C, ldc, beta, c->d_status};
    return spmm_rowpair_launch(c, a, flag2, static_cast<cudaStream_t>(stream));
}

as_status as_spmm_vcsr4_f32(as_ctx *c, int M, int K, int N, int nslots, const int *vrowptr,
                            const int *vcolind, const float *vval, const float *B, long ldb,
                            float *C, long ldc, float beta, void *stream) {
    if (!c) return fail(AS_ERR_INVALID_VALUE, "as_spmm_vcsr4_f32: ctx is NULL");
    as_status st = check_csr_args("as_spmm_vcsr4_f32", M, K, nslots, vrowptr, vcolind, vval, true);
    if (st != AS_OK) return st;
    if (N < 0) return fail(AS_ERR_INVALID_VALUE, "as_spmm_vcsr4_f32: negative N");
    if (M == 0 || N == 0) return AS_OK;
    if (!C || (nslots > 0 && K > 0 && !B) || ldb < N || ldc < N)
        return fail(AS_ERR_INVALID_VALUE, "as_spmm_vcsr4_f32: bad dense operand");
    DeviceGuard g(c->device);
    return spmm_vcsr4_launch(c, M, K, N, nslots, vrowptr, vcolind, vval, B, ldb, C, ldc, beta,
                             static_cast<cudaStream_t>(stream));
}

as_status as_gather_f32(as_ctx *c, long n, long n_src, const float *src, const int *idx,
                        float *dst, void *stream) {
    if (!c) return fail(AS_ERR_INVALID_VALUE, "as_gather_f32: ctx is NULL");
    if (n < 0 || n_src < 0 || (n > 0 && (!src || !idx || !dst)))
        return fail(AS_ERR_INVALID_VALUE, "as_gather_f32: bad arguments");
    DeviceGuard g(c->device);
    return gather_f32_launch(c, n, n_src, src, idx, dst, static_cast<cudaStream_t>(stream));
}

as_status as_f32_to_bf16(as_ctx *c, long n, const float *src, uint16_t *dst, void *stream) {
    if (!c) return fail(AS_ERR_INVALID_VALUE, "as_f32_to_bf16: ctx is NULL");
    if (n < 0) return fail(AS_ERR_INVALID_VALUE, "as_f32_to_bf16: negative size");
    if (n == 0) return AS_OK;
    if (!src || !dst) return fail(AS_ERR_INVALID_VALUE, "as_f32_to_bf16: NULL pointer");
    DeviceGuard g(c->device);
    return f32_to_bf16_launch(c, n, src, dst, static_cast<cudaStream_t>(stream));
}

}  // extern "C"
