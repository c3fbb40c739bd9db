// C-linkage wrapper around the GCN custom op's CPU kernel (gcn/pytorch-custom/spmm.cpp:49-71),
// called with a caller-zeroed output so that the op's uninitialised-output defect
// (spmm.cpp:41, torch::empty followed by +=) does not leak into golden vectors.
// Test infrastructure only.
void csr_spmm_kernel(int A_nrows, int B_ncols, int *A_csrRowPtr, int *A_csrColInd,
                     float *A_csrVal, float *B_dnVal, float *C_dnVal);

extern "C" void ref_csr_spmm_kernel(int A_nrows, int B_ncols, int *rowptr, int *colind,
                                    float *val, float *B, float *C) {
    csr_spmm_kernel(A_nrows, B_ncols, rowptr, colind, val, B, C);
}
