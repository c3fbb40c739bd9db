// Tensor-core SDDMM (tcgen05, split-bf16) -- entry point.
#include "common.cuh"
#include "internal.h"

namespace as {

as_status sddmm_bf16x3_launch(as_ctx *ctx, int M, int N, int K, int nnz, const int *rowptr,
                              const int *colind, const float *aval, const float *X, long ldx,
                              const float *Y, long ldy, float *out, cudaStream_t s) {
    (void)ctx; (void)M; (void)N; (void)K; (void)nnz; (void)rowptr; (void)colind; (void)aval;
    (void)X; (void)ldx; (void)Y; (void)ldy; (void)out; (void)s;
    return fail(AS_ERR_UNSUPPORTED, "as_sddmm_csr_bf16x3: not built yet");
}

}  // namespace as
