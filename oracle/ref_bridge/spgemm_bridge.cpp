// C-linkage wrapper around the reference's sparse x sparse -> dense kernel (SpMM.cpp), so
// that the oracle can call the reference's own code through ctypes. Test infrastructure only.
// Prototype as declared at SpMM.cpp:13-15 and defined at SpMM.cpp:309.
void sparse_matrix_mul3(int rowPtr1[], int colInd1[], float val1[], int rowPtr2[], int colInd2[],
                        float val2[], float *matrixC, int M, int K, int N, int threads);

extern "C" {
void ref_sparse_matrix_mul3(int *rowPtr1, int *colInd1, float *val1, int *rowPtr2, int *colInd2,
                            float *val2, float *C, int M, int K, int N, int threads) {
    sparse_matrix_mul3(rowPtr1, colInd1, val1, rowPtr2, colInd2, val2, C, M, K, N, threads);
}
}
