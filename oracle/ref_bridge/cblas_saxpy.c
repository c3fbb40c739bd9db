/* y += alpha*x for the reference's rowBaseSpmm2 comparison variant (test infrastructure; not
 * OpenBLAS). OpenBLAS 0.3.17, vendored with the reference, computes saxpy on ARMv8 with fused
 * multiply-adds (KERNEL.ARMV8:48 selects kernel/arm64/axpy.S: fmla on four lanes, fmadd on
 * the tail, axpy.S:64, :74, :91), and on x86_64 Haswell with vfmadd231ps
 * (kernel/x86_64/saxpy_microk_haswell-2.c:48): each y[i] is one fused step, restated here
 * with fmaf. */
#include <math.h>

#include "cblas.h"

void cblas_saxpy(const int n, const float alpha, const float *x, const int incx, float *y,
                 const int incy) {
    for (int i = 0; i < n; ++i) y[i * incy] = fmaf(alpha, x[i * incx], y[i * incy]);
}
