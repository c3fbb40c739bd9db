// Host-side declarations shared between the C-ABI layer (api.cu) and the kernel files.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include <string>
#include <vector>

#include "armsparse_gpu.h"

struct as_ctx {
    int device = 0;
    unsigned *d_status = nullptr;  // device words: [0] status (bit flags from common.cuh),
                                   // [1..3] long-row list: rows listed from the front, CTA-done
                                   // count, huge rows listed from the end
    unsigned *d_long = nullptr;    // = d_status + 1
    int sms = 1;                   // multiprocessors of the device
    void *scratch = nullptr;       // scratch arena
    size_t scratch_bytes = 0;
    std::vector<void *> retired;   // outgrown arenas: kept until the context is destroyed, since
                                   // kernels in flight or recorded in a CUDA graph may use them
    uint64_t launches = 0;         // kernels this library launched through the context
    unsigned spin_limit = 1u << 22;  // polls of a coordination wait before it gives up
                                     // (as_ctx_set_spin_limit); copy-drain waits keep 1 << 22
};

namespace as {

// Records the message for as_last_error() and returns s.
as_status fail(as_status s, const std::string &msg);
// Maps a CUDA error (from the last launch or a runtime call) to AS_ERR_CUDA with its text.
as_status check_cuda(cudaError_t e, const char *what);
// Scratch arena of at least `bytes` (256-byte aligned). Growing allocates a larger arena and
// retires the old one (freed by as_ctx_destroy), so no call synchronises or invalidates a
// pointer that earlier work still holds.
as_status scratch(as_ctx *ctx, size_t bytes, void **out);

// ---- launchers (return AS_OK or an error; count launches in ctx) ----
struct SpmmArgs {
    int M, K, N, nnz;
    const int *rowptr, *colind;
    const void *val, *B;
    long ldb;
    float *C;
    long ldc;
    float beta;
    unsigned *status;
    uint16_t *C16 = nullptr;  // given: the output goes here in bf16 (ldc elements per row) and C
                              // is unused; beta must be 0
    bool relu = false;        // with C16: negative outputs are stored as 0
};
// The SDDMM fused into an nnz-split SpMM pass: dA[perm ? perm[e] : e] = <B[k, :], F[r, :]> for
// each entry e (row r, column k) of A; F is M x N (leading dimension ldf, A's value type).
struct SddmmFuse {
    const void *F;
    long ldf;
    const int *perm;
    float *dA;
};
as_status spmm_launch(as_ctx *ctx, int dtype, int variant, const SpmmArgs &a, cudaStream_t s);
// C = A*B + beta*C with the fused SDDMM; variant 0 picks an nnz-split variant whose column tile
// covers N. AS_ERR_UNSUPPORTED when the variant is not nnz-split or its tile is narrower than N.
as_status spmm_sddmm_launch(as_ctx *ctx, int dtype, int variant, const SpmmArgs &a,
                            const SddmmFuse &f, cudaStream_t s);
as_status spmm_reduce_launch(as_ctx *ctx, int op, const SpmmArgs &a, cudaStream_t s);
// dst[i] = src[idx[i]] (transpose.cu); idx and dst 16-byte aligned.
as_status gather_f32_launch(as_ctx *ctx, long n, long n_src, const float *src, const int *idx,
                            float *dst, cudaStream_t s);
// Softmax cross-entropy of bf16 class scores (xent.cu).
as_status xent_fwd_launch(as_ctx *ctx, int n, int C, const uint16_t *S, long lds,
                          const int64_t *labels, float *lse, float *loss, cudaStream_t s);
as_status xent_bwd_launch(as_ctx *ctx, int n, int C, const uint16_t *S, long lds,
                          const int64_t *labels, const float *lse, const float *gscale,
                          uint16_t *G, long ldg, int width, cudaStream_t s);
as_status spmm_nnz_launch(as_ctx *ctx, int dtype, int vb, int group, int cpl, int chunk,
                          int unroll, const SpmmArgs &a, cudaStream_t s,
                          const SddmmFuse *fuse = nullptr);
// Multi-entry nnz-split (narrow B rows): a warp per chunk, 32 / group sub-groups.
as_status spmm_nnzme_launch(as_ctx *ctx, int dtype, int vb, int group, int chunk,
                            const SpmmArgs &a, cudaStream_t s, const SddmmFuse *fuse = nullptr);
as_status spmm_bulk_launch(as_ctx *ctx, int dtype, int lane_bytes, int stages, const SpmmArgs &a,
                           cudaStream_t s);
// Long rows of the row-split kernels: the cp.async size (16 or 4 bytes) the layout allows,
// 0 when none does; the launch of the kernel that takes the listed rows.
int spmm_long_granule(int dtype, int N, long ldb, const void *B);
// `op` is the chain's step: 0 the SpMM's fused multiply-add, 1 the unweighted sum, 2 max from
// -inf, 3 the DGL max (spmm_reduce.cu's reductions), 4 the fused multiply-add skipping zero
// values (spmm_vcsr4.cu's empty slots), 5 the row-pair layout's two chains per listed pair
// (spmm_rowpair.cu; `pair_flag` is its flag array); the steps other than 0 take fp32.
as_status spmm_long_launch(as_ctx *ctx, int dtype, int granule, const SpmmArgs &a,
                           const int *list, cudaStream_t s, int op = 0,
                           const uint8_t *pair_flag = nullptr);
as_status spgemm_dense_launch(as_ctx *ctx, int M, int K, int N, int nnz_a, const int *rp1,
                              const int *ci1, const float *v1, int nnz_b, const int *rp2,
                              const int *ci2, const float *v2, float *C, long ldc, float beta,
                              cudaStream_t s);
int spmm_variant_count(int dtype);
bool spmm_variant_supported(int dtype, int variant, int N, long ldb, long ldc, const void *B,
                            const void *C);
const char *spmm_variant_name(int dtype, int variant);
int spmm_default_variant(int dtype, int M, int K, int N, int nnz, long ldb, long ldc,
                         const void *B, const void *C);

as_status spmv_csr_launch(as_ctx *ctx, int M, int K, int nnz, const int *rowptr,
                          const int *colind, const float *val, const float *x, float *y,
                          float beta, cudaStream_t s);
as_status spmv_vcsr4_launch(as_ctx *ctx, int M, int K, int nslots, const int *rowptr,
                            const int *colind, const float *val, const float *x, float *y,
                            float beta, cudaStream_t s);

as_status sddmm_f32_launch(as_ctx *ctx, int M, int N, int K, int nnz, const int *rowptr,
                           const int *colind, const float *aval, const float *X, long ldx,
                           const float *Y, long ldy, float *out, cudaStream_t s);
as_status sddmm_bf16_launch(as_ctx *ctx, int M, int N, int K, int nnz, const int *rowptr,
                            const int *colind, const float *aval, const uint16_t *X, long ldx,
                            const uint16_t *Y, long ldy, float *out, cudaStream_t s);
as_status sddmm_coo_f32_launch(as_ctx *ctx, int M, int N, int K, int nnz, const int *rowind,
                               const int *colind, const float *aval, const float *X, long ldx,
                               const float *Y, long ldy, float *out, cudaStream_t s);
as_status sddmm_bf16x3_launch(as_ctx *ctx, int M, int N, int K, int nnz, const int *rowptr,
                              const int *colind, const float *aval, const float *X, long ldx,
                              const float *Y, long ldy, float *out, int variant, cudaStream_t s);
int sddmm_tc_variant_count();

as_status spmm_f64_launch(as_ctx *ctx, int M, int K, int N, int nnz, const int *rowptr,
                          const int *colind, const double *val, const double *B, long ldb,
                          double *C, long ldc, double beta, cudaStream_t s);
as_status sddmm_f64_launch(as_ctx *ctx, int M, int N, int K, int nnz, const int *rowptr,
                           const int *colind, const double *aval, const double *X, long ldx,
                           const double *Y, long ldy, double *out, cudaStream_t s);

// Transpose; `work` is caller-provided scratch of csr2csc_scratch_bytes(nnz, N) bytes (with_val
// also when perm is given). perm (optional): the CSR position of each CSC entry, written in
// place of the values (val and cscval are then ignored).
size_t csr2csc_scratch_bytes(int nnz, int N, bool with_val);
as_status csr2csc_launch(as_ctx *ctx, int M, int N, int nnz, const int *rowptr,
                         const int *colind, const float *val, int *colptr, int *rowind,
                         float *cscval, void *work, cudaStream_t s, int *perm = nullptr);

as_status csr_validate_launch(as_ctx *ctx, int n_rows, int n_cols, int nnz, const int *rowptr,
                              const int *colind, int require_sorted, unsigned *result,
                              cudaStream_t s);
// Exclusive scan of n ints (in may equal out); block sums live in the context's scratch.
as_status exclusive_scan_i32(as_ctx *ctx, const int *in, int *out, long n, cudaStream_t s);
as_status dense_to_csr_count_launch(as_ctx *ctx, int M, int K, const float *D, long ld,
                                    int *rowptr, cudaStream_t s);
as_status dense_to_csr_fill_launch(as_ctx *ctx, int M, int K, const float *D, long ld,
                                   const int *rowptr, int *colind, float *val, cudaStream_t s);
as_status csr_to_rowpair_count_launch(as_ctx *ctx, int M, int nnz, const int *rowptr,
                                      const int *colind, int *rowptr2, cudaStream_t s);
as_status csr_to_rowpair_fill_launch(as_ctx *ctx, int M, int nnz, const int *rowptr,
                                     const int *colind, const float *val, const int *rowptr2,
                                     int *colind2, float *val2, uint8_t *flag2, cudaStream_t s);
as_status spmm_rowpair_launch(as_ctx *ctx, const SpmmArgs &a, const uint8_t *flag2,
                              cudaStream_t s);
as_status spmm_vcsr4_launch(as_ctx *ctx, int M, int K, int N, int nslots, const int *vrowptr,
                            const int *vcolind, const float *vval, const float *B, long ldb,
                            float *C, long ldc, float beta, cudaStream_t s);
as_status csr_to_vcsr4_count_launch(as_ctx *ctx, int M, int nnz, const int *rowptr,
                                    const int *colind, int *vrowptr, cudaStream_t s);
as_status csr_to_vcsr4_fill_launch(as_ctx *ctx, int M, int nnz, const int *rowptr,
                                   const int *colind, const float *val, const int *vrowptr,
                                   int *vcolind, float *vval, cudaStream_t s);
as_status f32_to_bf16_launch(as_ctx *ctx, long n, const float *src, uint16_t *dst,
                             cudaStream_t s);

}  // namespace as
