/*
 * armsparse_gpu.h -- C ABI of the GB300 (sm_103a) sparse kernels.
 *
 * Every entry point takes plain device pointers and sizes, is asynchronous on the given
 * stream (a cudaStream_t passed as void*, NULL = legacy default stream) and returns an
 * as_status. The caller owns every input and output buffer; the library allocates only
 * scratch memory, which lives in the as_ctx. Nothing here calls exit(), traps or asserts
 * on the device: malformed CSR arrays are detected on the device, recorded in the
 * context's status word, and reported by as_ctx_sync_status() (or synchronously by
 * as_csr_validate()).
 *
 * Index arrays are int32, CSR row pointers are zero-based, dense matrices are row-major
 * with a leading dimension in elements. bf16 data is passed as uint16_t bit patterns.
 */
#ifndef ARMSPARSE_GPU_H
#define ARMSPARSE_GPU_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef enum as_status {
    AS_OK = 0,
    AS_ERR_INVALID_VALUE = 1, /* a size, pointer, leading dimension or alignment is wrong  */
    AS_ERR_INVALID_CSR = 2,   /* rowptr not monotone / out of [0,nnz], colind out of range */
    AS_ERR_UNSUPPORTED = 3,   /* the requested variant cannot run these arguments          */
    AS_ERR_CUDA = 4,          /* a CUDA runtime call failed (as_last_error() has the text) */
    AS_ERR_TIMEOUT = 5,       /* a bounded device-side wait gave up                        */
    AS_ERR_ALLOC = 6          /* scratch allocation failed                                 */
} as_status;

typedef struct as_ctx as_ctx;

/* ---- context ---------------------------------------------------------------------------
 * One context per host thread and device. It owns the device status word and the scratch
 * arena. The arena grows on demand: a larger one is allocated and the outgrown one is kept
 * until as_ctx_destroy, so device work already issued keeps valid pointers. */
as_status as_ctx_create(as_ctx **ctx, int device);
as_status as_ctx_destroy(as_ctx *ctx);
/* Waits for `stream`, returns and clears the device status word (AS_OK if no kernel since
 * the last call found malformed input). */
as_status as_ctx_sync_status(as_ctx *ctx, void *stream);
/* Text of the last error raised on this host thread (never NULL). */
const char *as_last_error(void);
const char *as_status_string(as_status s);
/* Number of this library's kernels launched through `ctx` since creation. */
uint64_t as_ctx_launch_count(const as_ctx *ctx);
/* How many times a kernel polls a coordination wait (the bulk-copy SpMM variants' wait for a
 * gathered row to land in shared memory; the long-row SpMM kernel's wait for a pipeline
 * stage) before it gives up: it then sets AS_ERR_TIMEOUT in the status word, waits for the
 * copies it issued (that drain always completes, whatever this setting), and leaves its
 * outputs unwritten. Default 2^22 (a few
 * seconds). 0 makes every such wait give up at once: tests use it to take the timeout path
 * without a fault or a hang. Applies to launches issued after the call. No counterpart in the
 * reference, which has no device-side waits. */
as_status as_ctx_set_spin_limit(as_ctx *ctx, unsigned polls);

/* ---- CSR validation (synchronous) --------------------------------------------------------
 * rowptr[0] == 0, rowptr non-decreasing, rowptr[n_rows] == nnz, 0 <= colind < n_cols.
 * With require_sorted != 0 also checks strictly ascending columns within each row. */
as_status as_csr_validate(as_ctx *ctx, int n_rows, int n_cols, int nnz, const int *rowptr,
                          const int *colind, int require_sorted, void *stream);

/* ---- SpMM: C = A * B + beta * C ------------------------------------------------------------
 * A: M x K CSR (rowptr[M+1], colind[nnz], val[nnz]); B: K x N (ldb >= N); C: M x N (ldc >= N).
 * beta == 0 overwrites C without reading it; beta == 1 accumulates, which is the reference
 * driver's C += A*B.
 * variant: 0 = library choice; otherwise an id from as_spmm_variant_*().
 * Replaces: rowBaseSpmm3 / rowBaseSpmm2 / origin (SDMM.cpp:90, :65, :422), the GCN op's
 * csr_spmm_kernel (gcn/pytorch-custom/spmm.cpp:49-71) and spmm_cuda
 * (gcn/pytorch-custom/spmm_kernel.cu:425-458).
 * Row-split ("rowsplit_*") and shared-memory-staged ("bulk_*") variants are bit-identical to
 * rowBaseSpmm3: every output is one fused multiply-add chain over the row's entries in CSR
 * order. NNZ-split variants ("nnzsplit_*") balance skewed rows by cutting the entries into
 * fixed chunks; a row that crosses a chunk boundary gets its partial sums added in chunk
 * order (deterministic, not bit-identical for those rows; rows inside one chunk are). */
as_status as_spmm_csr_f32(as_ctx *ctx, int M, int K, int N, int nnz, const int *rowptr,
                          const int *colind, const float *val, const float *B, long ldb,
                          float *C, long ldc, float beta, int variant, void *stream);

/* Same with A's values and B stored as bf16, products accumulated in fp32, C fp32. */
as_status as_spmm_csr_bf16(as_ctx *ctx, int M, int K, int N, int nnz, const int *rowptr,
                           const int *colind, const uint16_t *val, const uint16_t *B,
                           long ldb, float *C, long ldc, float beta, int variant,
                           void *stream);

/* Other reductions: C[i,:] = reduce_{e in row i} w_e * B[col(e),:], reduce = sum or max,
 * w_e = val[e] (val may be NULL: every w_e = 1, the unweighted "copy" aggregation). Overwrites C.
 *  - AS_REDUCE_SUM: unweighted sum adds in CSR order exactly as the reference's
 *    topo*SPMMKernel family (gcn/pytorch-custom/spmm_kernel.cu:31-207); rows without entries
 *    give 0.
 *  - AS_REDUCE_MAX: max starting from -inf (fmaxf, NaN entries ignored); rows without entries
 *    give 0.
 *  - AS_REDUCE_MAX_DGL: the reference's copy-max aggregation as its DGL kernels compute it
 *    (gcn/dgl-custom/binary_reduce_max.cu:18-24, :41-54, :151-166): the accumulator starts at
 *    -10000 and each entry applies acc = (acc > x) ? acc : x in CSR order. So values below
 *    -10000 never show, a NaN entry sets the accumulator to NaN and the entry after it
 *    replaces that NaN (no comparison with NaN is true), and rows without entries give
 *    -10000. */
#define AS_REDUCE_SUM 0
#define AS_REDUCE_MAX 1
#define AS_REDUCE_MAX_DGL 2
as_status as_spmm_csr_reduce_f32(as_ctx *ctx, int M, int K, int N, int nnz, const int *rowptr,
                                 const int *colind, const float *val, const float *B, long ldb,
                                 float *C, long ldc, int op, void *stream);

/* Sparse x sparse -> dense: C = beta*C + A*B with A (M x K, nnz_a entries) and B (K x N,
 * nnz_b entries) in CSR and C dense row-major (ldc >= N). Replaces sparse_matrix_mul3
 * (SpMM.cpp:309-327; beta = 1 is its accumulate): every output element is the reference's
 * fused-FMA chain over A's row in CSR order, bit for bit. B's rows must hold distinct column
 * indices (as CSR does). */
as_status as_spgemm_csr_dense_f32(as_ctx *ctx, int M, int K, int N, int nnz_a,
                                  const int *a_rowptr, const int *a_colind, const float *a_val,
                                  int nnz_b, const int *b_rowptr, const int *b_colind,
                                  const float *b_val, float *C, long ldc, float beta,
                                  void *stream);

/* Variant table for tuning: ids are 1..count. dtype 0 = f32, 1 = bf16. */
int as_spmm_variant_count(int dtype);
const char *as_spmm_variant_name(int dtype, int variant);
/* 1 if `variant` can run this layout (N, leading dimensions, pointer alignment), else 0 -- the
 * launch would return AS_ERR_UNSUPPORTED. */
int as_spmm_variant_supported(int dtype, int variant, int N, long ldb, long ldc, const void *B,
                              const void *C);
/* The variant the library picks for these arguments (what variant 0 runs). */
int as_spmm_default_variant(int dtype, int M, int K, int N, int nnz, long ldb, long ldc,
                            const void *B, const void *C);

/* ---- SpMV: y = A * x + beta * y ------------------------------------------------------------
 * Plain CSR. Replaces sparse_dense_vector (SpMV.cpp:155-179) for callers holding CSR. */
as_status as_spmv_csr_f32(as_ctx *ctx, int M, int K, int nnz, const int *rowptr,
                          const int *colind, const float *val, const float *x, float *y,
                          float beta, void *stream);

/* The reference's 1x4-blocked layout unchanged (SpMV.cpp:15-38): each stored block is four
 * consecutive slots whose first colind is the block's first column; nslots = rowptr[M] is a
 * multiple of 4 and the block's columns must lie in [0, K). Each row's four lane sums are
 * combined as (s2 + s0) + (s3 + s1), as the reference does (SpMV.cpp:175-176).
 * Replaces sparse_dense_vector (SpMV.cpp:155). */
as_status as_spmv_vcsr4_f32(as_ctx *ctx, int M, int K, int nslots, const int *rowptr,
                            const int *colind, const float *val, const float *x, float *y,
                            float beta, void *stream);

/* ---- SDDMM: out[e] = s_e * <X[row(e), :], Y[col(e), :]> ---------------------------------------
 * Pattern: M x N CSR; X: M x K (ldx >= K); Y: N x K (ldy >= K); out: nnz values in CSR
 * order. s_e = aval[e], or 1 when aval is NULL (exactly the reference's sddmm_cuda_csr,
 * gcn/pytorch-custom/sddmm.cu:459-483, which never scales).
 * as_sddmm_csr_f32: FP32 CUDA-core dot products.
 * as_sddmm_csr_bf16x3: tensor cores (tcgen05), operands split as x = hi + lo in bf16 and
 * x.y ~ hi.hi + hi.lo + lo.hi accumulated in FP32 (relative error near FP32's). */
as_status as_sddmm_csr_f32(as_ctx *ctx, int M, int N, int K, int nnz, const int *rowptr,
                           const int *colind, const float *aval, const float *X, long ldx,
                           const float *Y, long ldy, float *out, void *stream);
as_status as_sddmm_csr_bf16x3(as_ctx *ctx, int M, int N, int K, int nnz, const int *rowptr,
                              const int *colind, const float *aval, const float *X, long ldx,
                              const float *Y, long ldy, float *out, void *stream);
/* X and Y stored as bf16 (uint16_t bit patterns), FP32 products and sums, FP32 out: the
 * dot products of as_sddmm_csr_f32 run on the bf16 values (bit for bit what
 * as_sddmm_csr_f32 gives for those values widened to FP32), with half the bytes gathered.
 * Used for the edge-value gradient of bf16 GCN layers. */
as_status as_sddmm_csr_bf16(as_ctx *ctx, int M, int N, int K, int nnz, const int *rowptr,
                            const int *colind, const float *aval, const uint16_t *X, long ldx,
                            const uint16_t *Y, long ldy, float *out, void *stream);

/* bf16 output: C = bf16(A*B) (round to nearest even from the FP32 sums; beta is 0), so a bf16
 * pipeline stores half the bytes and needs no conversion pass. The FP32 sums are those of
 * as_spmm_csr_bf16 with the same variant, so C is that call's result rounded, bit for bit.
 * relu != 0: negative sums are stored as 0 (a layer followed by a ReLU, in the same pass).
 * C (ldc elements per row) is aligned to the variant's vectors (min(2 x elements, 16) bytes);
 * the bulk-copy variants have no bf16 output (AS_ERR_UNSUPPORTED). */
as_status as_spmm_csr_bf16_out16(as_ctx *ctx, int M, int K, int N, int nnz, const int *rowptr,
                                 const int *colind, const uint16_t *val, const uint16_t *B,
                                 long ldb, uint16_t *C, long ldc, int relu, int variant,
                                 void *stream);

/* ---- Softmax cross-entropy of class scores (the GCN's loss) ----------------------------------
 * n rows of C class scores in bf16 (row stride lds >= C elements), int64 labels in [0, C).
 * as_softmax_xent_bf16: loss[0] = (1/n) sum_i (lse_i - S_i[label_i]) with lse_i =
 * logsumexp(S_i) (also written, n floats, for the backward) -- the mean negative
 * log-likelihood of log_softmax (gcn/pytorch-custom/gcn_custom.py:90, :122-126), FP32, summed
 * in a fixed order (deterministic). A label out of range counts 0 and is reported by
 * as_ctx_sync_status (AS_ERR_INVALID_VALUE).
 * as_softmax_xent_bwd_bf16: its gradient times the device scalar gscale[0] (the upstream
 * gradient, read on the device): G[i, j] = bf16((exp(S_ij - lse_i) - [j == label_i]) * gscale
 * / n) for j < C and 0 for C <= j < width (padding columns); ldg >= width.
 * 1 <= C <= width <= 64. */
as_status as_softmax_xent_bf16(as_ctx *ctx, int n, int C, const uint16_t *S, long lds,
                               const int64_t *labels, float *lse, float *loss, void *stream);
as_status as_softmax_xent_bwd_bf16(as_ctx *ctx, int n, int C, const uint16_t *S, long lds,
                                   const int64_t *labels, const float *lse, const float *gscale,
                                   uint16_t *G, long ldg, int width, void *stream);

/* ---- SpMM and SDDMM in one pass over A ---------------------------------------------------------
 * C = A*B + beta*C (A: M x K CSR, B: K x N, C: M x N, as as_spmm_csr_*) and, for every entry e
 * of A (row r, column k):  dA[perm ? perm[e] : e] = <B[k, :], F[r, :]>  (F: M x N, ldf >= N,
 * same storage type as B; FP32 products and sums). No reference counterpart: it is the
 * backward of out = A_fwd * X with trainable edge values (gcn/pytorch-custom/op.py:30 computes
 * only the first half and returns no gradient for the values, op.py:31). Called with A = the
 * CSC of A_fwd (colptr, rowind, values in CSC order), B = dOut, F = X and perm from
 * as_csr2csc_perm, it gives dX = A_fwd^T * dOut and the values' gradient in CSR order, gathering
 * dOut's rows once for both (separately, the SDDMM gathers a second time).
 * C follows the nnz-split SpMM variants (see as_spmm_csr_f32); each dA value is one FMA chain
 * per lane over the lane's columns, then a butterfly sum over the variant's lane group.
 * variant: 0 = library choice, else an nnz-split variant whose column tile (vector elements x
 * group x vectors per lane) covers N; others return AS_ERR_UNSUPPORTED. */
as_status as_spmm_sddmm_csr_f32(as_ctx *ctx, int M, int K, int N, int nnz, const int *rowptr,
                                const int *colind, const float *val, const float *B, long ldb,
                                float *C, long ldc, float beta, const float *F, long ldf,
                                const int *perm, float *dA, int variant, void *stream);
as_status as_spmm_sddmm_csr_bf16(as_ctx *ctx, int M, int K, int N, int nnz, const int *rowptr,
                                 const int *colind, const uint16_t *val, const uint16_t *B,
                                 long ldb, float *C, long ldc, float beta, const uint16_t *F,
                                 long ldf, const int *perm, float *dA, int variant,
                                 void *stream);
/* as_spmm_sddmm_csr_bf16 with C in bf16 (as as_spmm_csr_bf16_out16). */
as_status as_spmm_sddmm_csr_bf16_out16(as_ctx *ctx, int M, int K, int N, int nnz,
                                       const int *rowptr, const int *colind,
                                       const uint16_t *val, const uint16_t *B, long ldb,
                                       uint16_t *C, long ldc, const uint16_t *F, long ldf,
                                       const int *perm, float *dA, int variant, void *stream);

/* as_sddmm_csr_bf16x3 with an explicit kernel variant (tuning): 0 = library choice,
 * 1 = one 128 x 256 output tile per CTA, 2 = persistent CTAs with two tensor-memory
 * accumulators (epilogue of one tile under the MMAs of the next), 64-wide K stages,
 * 3 = persistent with 32-wide K stages (4-deep pipeline). Same results for every variant
 * up to FP32 accumulation order. */
as_status as_sddmm_csr_bf16x3_v(as_ctx *ctx, int M, int N, int K, int nnz, const int *rowptr,
                                const int *colind, const float *aval, const float *X, long ldx,
                                const float *Y, long ldy, float *out, int variant, void *stream);
int as_sddmm_bf16x3_variant_count(void);

/* COO form: entry e has row rowind[e] and column colind[e] (any order); X, Y, out as above.
 * Replaces sddmm_cuda_coo (gcn/pytorch-custom/sddmm.cu:427-457). */
as_status as_sddmm_coo_f32(as_ctx *ctx, int M, int N, int K, int nnz, const int *rowind,
                           const int *colind, const float *aval, const float *X, long ldx,
                           const float *Y, long ldy, float *out, void *stream);

/* ---- CSR -> CSC (transpose) ------------------------------------------------------------------
 * A: M x N CSR. Outputs colptr[N+1], rowind[nnz], cscval[nnz] (val / cscval may be NULL
 * for a pattern-only transpose). Rows are ascending within every column, so the result is
 * unique and bit-exact (a stable counting sort by column; deterministic run to run).
 * Replaces csr2csc_cuda (gcn/pytorch-custom/spmm_kernel.cu:460-476) and the CPU
 * fast_transpose (sparseTranspose.cpp:95-142). */
as_status as_csr2csc(as_ctx *ctx, int M, int N, int nnz, const int *rowptr, const int *colind,
                     const float *val, int *colptr, int *rowind, float *cscval, void *stream);

/* as_csr2csc giving, in place of the values, the permutation perm[nnz]: perm[j] is the CSR
 * position of CSC entry j (so cscval[j] = val[perm[j]] for any values). No reference
 * counterpart: it lets a caller whose edge values change every step (trainable edge weights)
 * gather them into CSC order, and lets as_spmm_sddmm_* write results at CSR positions while
 * walking the CSC. */
as_status as_csr2csc_perm(as_ctx *ctx, int M, int N, int nnz, const int *rowptr,
                          const int *colind, int *colptr, int *rowind, int *perm, void *stream);

/* dst[i] = src[idx[i]] for i < n: values moved between two orders of the same entries, e.g.
 * an SDDMM result from CSC to CSR order with the inverse of as_csr2csc_perm's permutation. An
 * index outside [0, n_src) gives 0 and is reported by as_ctx_sync_status. idx and dst are
 * 16-byte aligned. */
as_status as_gather_f32(as_ctx *ctx, long n, long n_src, const float *src, const int *idx,
                        float *dst, void *stream);

/* ---- CSR -> CSC without allocating ------------------------------------------------------------
 * No counterpart in the reference. Some callers of this library cannot allocate device
 * memory: a plugin inside a host framework that owns every device allocation through its own
 * pool, or a serving loop that forbids allocation after start-up because cudaMalloc/cudaFree
 * synchronise the device and fragment it. They cannot create an as_ctx (its status word and
 * scratch arena are allocated). as_csr2csc_static is as_csr2csc for them: the caller passes
 * the inputs and outputs, and the transpose's scratch is a fixed device array inside this
 * library (about 5 MB, reserved on every GPU that loads the library until the process exits).
 * It calls no cudaMalloc, cudaFree or other allocating routine.
 *  - Limit: nnz <= AS_CSR2CSC_STATIC_MAX_NNZ; larger calls return AS_ERR_UNSUPPORTED and launch
 *    nothing. Other argument errors return AS_ERR_INVALID_VALUE (AS_ERR_INVALID_CSR for entries
 *    without rows or columns); these statuses are the whole report (as_last_error() is not set).
 *  - The first call on a device looks up the array's device address (cudaGetSymbolAddress)
 *    with that device current; make that first call before any stream capture. The address is
 *    kept for the life of the process: after cudaDeviceReset (or anything else that tears down
 *    and recreates the device's primary context) this entry point must not be called again on
 *    that device.
 *  - A launch error that earlier, unrelated work left pending in the CUDA runtime is cleared
 *    at entry (cudaGetLastError), so that the status returned is this call's own.
 *  - All calls share the one array: calls whose work overlaps on the GPU (different streams or
 *    threads, no ordering between them) race and corrupt each other's results. Serialise them.
 *  - Malformed CSR is handled memory-safely but not reported (there is no context to hold the
 *    flag): every row index written is still in [0, M), but the result is meaningless.
 *    Validate with as_csr_validate beforehand where that matters.
 * Same output contract as as_csr2csc (rows ascending within columns, bit-exact). */
#define AS_CSR2CSC_STATIC_MAX_NNZ (1 << 18)
as_status as_csr2csc_static(int M, int N, int nnz, const int *rowptr, const int *colind,
                            const float *val, int *colptr, int *rowind, float *cscval,
                            void *stream);

/* ---- FP64 forms, for gradient checks only ---------------------------------------------------
 * Same contracts as as_spmm_csr_f32 (row-split order, one output per thread) and
 * as_sddmm_csr_f32, in double precision. Not tuned; they exist so that the autograd op can be
 * checked against finite differences in float64. */
as_status as_spmm_csr_f64(as_ctx *ctx, int M, int K, int N, int nnz, const int *rowptr,
                          const int *colind, const double *val, const double *B, long ldb,
                          double *C, long ldc, double beta, void *stream);
as_status as_sddmm_csr_f64(as_ctx *ctx, int M, int N, int K, int nnz, const int *rowptr,
                           const int *colind, const double *aval, const double *X, long ldx,
                           const double *Y, long ldy, double *out, void *stream);

/* ---- format builders (two passes: count, then fill) -----------------------------------------
 * Dense M x K (row-major, ld >= K) -> CSR, the reference's toCSR (SDMM.cpp:355-370): entries
 * where value != 0 in row-major order, columns ascending. _count writes rowptr[0..M]
 * (rowptr[M] = nnz, read it to size colind / val); _fill writes colind and val. */
as_status as_dense_to_csr_count(as_ctx *ctx, int M, int K, const float *D, long ld, int *rowptr,
                                void *stream);
as_status as_dense_to_csr_fill(as_ctx *ctx, int M, int K, const float *D, long ld,
                               const int *rowptr, int *colind, float *val, void *stream);
/* CSR (columns ascending in rows) -> the reference's 1x4-blocked layout, toVectorAwareCSR
 * (SpMV.cpp:15-38): one block of 4 slots per aligned 4-column group holding an entry, lane l
 * of a block has column 4*group + l and the entry's value or 0. _count writes vrowptr[0..M]
 * (vrowptr[M] = number of slots); _fill writes vcolind and vval. */
as_status as_csr_to_vcsr4_count(as_ctx *ctx, int M, int nnz, const int *rowptr, const int *colind,
                                int *vrowptr, void *stream);
as_status as_csr_to_vcsr4_fill(as_ctx *ctx, int M, int nnz, const int *rowptr, const int *colind,
                               const float *val, const int *vrowptr, int *vcolind, float *vval,
                               void *stream);

/* C = A*B + beta*C with A in the reference's 1x4-blocked layout (vrowptr[M+1], vcolind and vval
 * [nslots], as as_csr_to_vcsr4_* write it): the SpMM counterpart of sparse_dense_vector
 * (SpMV.cpp:155-179). Slots holding 0 are skipped (the layout does not tell a stored zero from
 * an empty slot), so each output is the fused chain over the row's nonzero entries in column
 * order -- bit for bit the CSR SpMM of the matrix without stored zeros. */
as_status as_spmm_vcsr4_f32(as_ctx *ctx, int M, int K, int N, int nslots, const int *vrowptr,
                            const int *vcolind, const float *vval, const float *B, long ldb,
                            float *C, long ldc, float beta, void *stream);

/* CSR (columns ascending in rows) -> the reference's row-pair reuse layout, toDataReuseFormat
 * (suitesparse_sdmm.cpp:150-179): rows are paired (2p, 2p+1); row 2p's segment lists its
 * entries in column order, each followed by row 2p+1's entry in the same column when there is
 * one (flag2 = 1: it belongs to the next row); row 2p+1's segment keeps its other entries; an
 * unpaired last row is copied. The total stays nnz. _count writes rowptr2[0..M]; _fill writes
 * colind2, val2 and flag2 (one byte per entry). Rows that are not sorted give a memory-safe
 * layout that is not the reference's. */
as_status as_csr_to_rowpair_count(as_ctx *ctx, int M, int nnz, const int *rowptr,
                                  const int *colind, int *rowptr2, void *stream);
as_status as_csr_to_rowpair_fill(as_ctx *ctx, int M, int nnz, const int *rowptr, const int *colind,
                                 const float *val, const int *rowptr2, int *colind2, float *val2,
                                 uint8_t *flag2, void *stream);
/* C = A*B + beta*C over the row-pair layout, bit-identical to DataReuseSpmm
 * (suitesparse_sdmm.cpp:25-44, its saxpy fused per element as OpenBLAS computes it): row 2p is
 * its CSR chain; row 2p+1 chains over the entries it shares with row 2p first (column order),
 * then over its own segment. A flagged entry reuses the B segment of the entry before it (the
 * same column) instead of gathering it again. beta = 1 is the reference's accumulate. Pairs
 * with more than 256 entries run on the long-row kernel, one unit per row of the pair, which
 * gathers each entry's own column (the same values in a well-formed layout; a malformed one,
 * e.g. a flagged first entry, can differ from the short-pair path). */
as_status as_spmm_rowpair_f32(as_ctx *ctx, int M, int K, int N, int nnz, const int *rowptr2,
                              const int *colind2, const float *val2, const uint8_t *flag2,
                              const float *B, long ldb, float *C, long ldc, float beta,
                              void *stream);

/* ---- small dense helpers used around the hot path ---------------------------------------- */
/* dst[i] = bf16(src[i]) (round to nearest even). */
as_status as_f32_to_bf16(as_ctx *ctx, long n, const float *src, uint16_t *dst, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* ARMSPARSE_GPU_H */
