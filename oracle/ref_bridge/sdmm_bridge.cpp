// C-linkage wrappers around the reference SpMM driver's kernels (SDMM.cpp), so that the
// oracle can call the reference's own code through ctypes. Test infrastructure only.
// Prototypes as declared in SDMM.cpp:11-20 and defined at SDMM.cpp:65, :90, :355, :422.
void rowBaseSpmm2(int rowPtr[], int colInd[], float val[], float B[], float C[], int M, int K,
                  int N, int threads);
void rowBaseSpmm3(int rowPtr[], int colInd[], float val[], float B[], float C[], int M, int K,
                  int N, int threads);
void origin(int rowPtr[], int colInd[], float val[], float B[], float C[], int M, int K, int N,
            int threads);
void toCSR(float *matrix, int rows, int cols, int *rowPtr, int *colInd, float *val);

extern "C" {
void ref_rowBaseSpmm3(int *rowPtr, int *colInd, float *val, float *B, float *C, int M, int K,
                      int N, int threads) {
    rowBaseSpmm3(rowPtr, colInd, val, B, C, M, K, N, threads);
}
void ref_rowBaseSpmm2(int *rowPtr, int *colInd, float *val, float *B, float *C, int M, int K,
                      int N, int threads) {
    rowBaseSpmm2(rowPtr, colInd, val, B, C, M, K, N, threads);
}
void ref_origin(int *rowPtr, int *colInd, float *val, float *B, float *C, int M, int K, int N,
                int threads) {
    origin(rowPtr, colInd, val, B, C, M, K, N, threads);
}
void ref_toCSR(float *matrix, int rows, int cols, int *rowPtr, int *colInd, float *val) {
    toCSR(matrix, rows, cols, rowPtr, colInd, val);
}
}
