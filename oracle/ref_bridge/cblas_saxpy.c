/* Scalar y += alpha*x for the reference's rowBaseSpmm2 comparison variant (test
 * infrastructure; not OpenBLAS). */
#include "cblas.h"

void cblas_saxpy(const int n, const float alpha, const float *x, const int incx, float *y,
                 const int incy) {
    for (int i = 0; i < n; ++i) y[i * incy] += alpha * x[i * incx];
}
