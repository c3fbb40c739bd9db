// C-linkage wrappers around the reference SpMV driver's kernels (SpMV.cpp:15, :155).
// Test infrastructure only.
void toVectorAwareCSR(float *matrix, int rows, int cols, int *rowPtr, int *colInd, float *val);
void sparse_dense_vector(float *B, float *C, int rowPtr[], int colInd[], float val[], int M,
                         int threads);

extern "C" {
void ref_toVectorAwareCSR(float *matrix, int rows, int cols, int *rowPtr, int *colInd,
                          float *val) {
    toVectorAwareCSR(matrix, rows, cols, rowPtr, colInd, val);
}
void ref_sparse_dense_vector(float *B, float *C, int *rowPtr, int *colInd, float *val, int M,
                             int threads) {
    sparse_dense_vector(B, C, rowPtr, colInd, val, M, threads);
}
}
