/*
 * armsparse_drivers.h -- host-pointer shims with the reference drivers' exact signatures.
 *
 * Each shim takes the same host arrays the reference's CPU kernel takes, copies them to the
 * GPU, runs the sm_103a kernel through the C ABI (armsparse_gpu.h), copies the result back
 * and returns after the device finished. `threads` (an OpenMP thread count in the
 * reference) is accepted and ignored. Semantics follow the replaced function: the SpMM and
 * SpMV shims ACCUMULATE into C / y exactly like the reference (the caller zeroes them), and
 * their results are bit-identical to the reference kernels (fused-FMA chains in CSR order).
 * The reference functions have no error path; a failure here prints one line to stderr and
 * is readable through as_drv_last_status(); the output is left untouched, except that an
 * SpMM shim may already have written the column blocks finished before the failure.
 *
 * Calls are serialised by a process-wide lock; device buffers are cached between calls and
 * grown on demand. The SpMM shims run in column blocks and copy each block's C back from a
 * helper thread (started and joined within the call) while the next blocks' B goes in.
 */
#ifndef ARMSPARSE_DRIVERS_H
#define ARMSPARSE_DRIVERS_H

#include "armsparse_gpu.h"

#ifdef __cplusplus
#include <mutex>

/* SDMM.cpp:90 -- C[M x N] += A * B, A CSR (M x K), B (K x N) row-major. */
void rowBaseSpmm3(int rowPtr[], int colInd[], float val[], float B[], float C[], int M, int K,
                  int N, int threads);
/* SDMM.cpp:65 -- the cblas_saxpy variant: same contract and same result as rowBaseSpmm3. */
void rowBaseSpmm2(int rowPtr[], int colInd[], float val[], float B[], float C[], int M, int K,
                  int N, int threads);
/* SDMM.cpp:422 -- C = A * B (overwrite). */
void origin(int rowPtr[], int colInd[], float val[], float B[], float C[], int M, int K, int N,
            int threads);
/* SpMM.cpp:309 -- matrixC[M x N] += A * B with A (M x K) and B (K x N) both CSR. */
void sparse_matrix_mul3(int rowPtr1[], int colInd1[], float val1[], int rowPtr2[],
                        int colInd2[], float val2[], float *matrixC, int M, int K, int N,
                        int threads);
/* SpMV.cpp:155 -- y[M] += A * x over the 1x4-blocked layout (rowPtr[M] slots). The length of
 * x is not an argument in the reference; the shim takes max(colInd) + 4. */
void sparse_dense_vector(float *B, float *C, int rowPtr[], int colInd[], float val[], int M,
                         int threads);
/* gcn/pytorch-custom/spmm.cpp:49 -- C[A_nrows x B_ncols] += A * B; B has max(colind) + 1 rows. */
void csr_spmm_kernel(int A_nrows, int B_ncols, int *A_csrRowPtr, int *A_csrColInd,
                     float *A_csrVal, float *B_dnVal, float *C_dnVal);
/* sparseTranspose.cpp:95 -- transpose of an int triplet matrix (header row m, n, nnz, then
 * (row, col, value) rows). The input must be in row-major order (what convert() writes); the
 * output lists each column's entries with rows ascending. mtx is not used. */
void fast_transpose(int *sm, int *res, std::mutex mtx[]);
/* suitesparse_sdmm.cpp:25 -- C[M x N] += A * B over the row-pair reuse layout (rowPtr[M+1],
 * colInd/val/flag[rowPtr[M]]), bit-identical to the reference with its saxpy fused. */
void DataReuseSpmm(int rowPtr[], int colInd[], float val[], float B[], float C[], int M, int K,
                   int N, int threads, bool *flag);
/* suitesparse_sdmm.cpp:150 -- dense matrix (rows x cols, row-major) -> the row-pair reuse
 * layout; rowPtr needs rows + 1 ints, the other arrays one slot per nonzero. As in the
 * reference, the entries that move into the previous row's segment are zeroed in `matrix`. */
void toDataReuseFormat(float *matrix, int rows, int cols, int *rowPtr, int *colInd, float *val,
                       bool *flag);
#endif

#ifdef __cplusplus
extern "C" {
#endif
/* C-linkage aliases of the shims above, for FFI callers (ctypes, cgo, JNI). */
void as_drv_rowBaseSpmm3(int *rowPtr, int *colInd, float *val, float *B, float *C, int M, int K,
                         int N, int threads);
/* SDMM.cpp:65 -- rowBaseSpmm2, the cblas_saxpy variant; same contract and result as above. */
void as_drv_rowBaseSpmm2(int *rowPtr, int *colInd, float *val, float *B, float *C, int M, int K,
                         int N, int threads);
void as_drv_origin(int *rowPtr, int *colInd, float *val, float *B, float *C, int M, int K, int N,
                   int threads);
void as_drv_sparse_dense_vector(float *B, float *C, int *rowPtr, int *colInd, float *val, int M,
                                int threads);
void as_drv_sparse_matrix_mul3(int *rowPtr1, int *colInd1, float *val1, int *rowPtr2,
                               int *colInd2, float *val2, float *C, int M, int K, int N,
                               int threads);
void as_drv_csr_spmm_kernel(int A_nrows, int B_ncols, int *rowptr, int *colind, float *val,
                            float *B, float *C);
void as_drv_fast_transpose(int *sm, int *res);
void as_drv_DataReuseSpmm(int *rowPtr, int *colInd, float *val, float *B, float *C, int M, int K,
                          int N, int threads, unsigned char *flag);
void as_drv_toDataReuseFormat(float *matrix, int rows, int cols, int *rowPtr, int *colInd,
                              float *val, unsigned char *flag);
/* Status of the last shim call on any thread (AS_OK when it succeeded). */
as_status as_drv_last_status(void);
#ifdef __cplusplus
}
#endif

#endif /* ARMSPARSE_DRIVERS_H */
