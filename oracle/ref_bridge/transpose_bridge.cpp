// C-linkage wrappers around the reference's COO-triplet transpose (sparseTranspose.cpp:71,
// :95, :143). The triplet layout is int[(nnz+1)*3] with a header row (rows, cols, nnz).
// fast_transpose orders entries within a column by OpenMP scheduling; the wrapper takes the
// thread count so that a single-threaded call gives the stable (row-ascending) order.
// Test infrastructure only.
#include <mutex>
#include <omp.h>

void convert(int *A, int *sm_A, int m, int n);
void fast_transpose(int *sm, int *res, std::mutex mtx[]);
void simpleTranspose(int *sm, int *res);

extern "C" {
void ref_convert(int *A, int *sm_A, int m, int n) { convert(A, sm_A, m, n); }
void ref_fast_transpose(int *sm, int *res, int threads) {
    int ncols = sm[1];
    std::mutex *mtx = new std::mutex[ncols > 0 ? ncols : 1];
    int saved = omp_get_max_threads();
    omp_set_num_threads(threads);
    fast_transpose(sm, res, mtx);
    omp_set_num_threads(saved);
    delete[] mtx;
}
void ref_simpleTranspose(int *sm, int *res) { simpleTranspose(sm, res); }
}
