// C-linkage wrappers around the reference's row-pair reuse format and its SpMM
// (suitesparse_sdmm.cpp: toDataReuseFormat :150-179, DataReuseSpmm :25-44, toCSR), so that the
// oracle can call the reference's own code through ctypes. Prototypes as declared in
// suitesparse_sdmm.cpp:20-25. Test infrastructure only.
void toCSR(float *matrix, int rows, int cols, int *rowPtr, int *colInd, float *val);
void toDataReuseFormat(float *matrix, int rows, int cols, int *rowPtr, int *colInd, float *val,
                       bool *flag);
void DataReuseSpmm(int rowPtr[], int colInd[], float val[], float B[], float C[], int M, int K,
                   int N, int threads, bool *flag);

extern "C" {
void ref_toCSR_rp(float *matrix, int rows, int cols, int *rowPtr, int *colInd, float *val) {
    toCSR(matrix, rows, cols, rowPtr, colInd, val);
}
// The dense matrix is modified (entries moved into the previous row's segment are zeroed), as
// the reference does.
void ref_toDataReuseFormat(float *matrix, int rows, int cols, int *rowPtr, int *colInd,
                           float *val, unsigned char *flag) {
    toDataReuseFormat(matrix, rows, cols, rowPtr, colInd, val, reinterpret_cast<bool *>(flag));
}
void ref_DataReuseSpmm(int *rowPtr, int *colInd, float *val, float *B, float *C, int M, int K,
                       int N, int threads, unsigned char *flag) {
    DataReuseSpmm(rowPtr, colInd, val, B, C, M, K, N, threads, reinterpret_cast<bool *>(flag));
}
}
