/*
 * Minimal declaration of the one CBLAS routine the reference's SpMM driver calls
 * (cblas_saxpy, used only by its comparison variant rowBaseSpmm2, SDMM.cpp:84).
 * Test infrastructure: the definition in ref_bridge/cblas_saxpy.c is a plain scalar loop,
 * not OpenBLAS 0.3.17.dev, so parity of that variant with OpenBLAS is unpinned.
 */
#ifndef ARMSPARSE_ORACLE_CBLAS_STUB_H
#define ARMSPARSE_ORACLE_CBLAS_STUB_H
#ifdef __cplusplus
extern "C" {
#endif
void cblas_saxpy(const int n, const float alpha, const float *x, const int incx, float *y,
                 const int incy);
#ifdef __cplusplus
}
#endif
#endif
