"""armsparse_gb300 -- GB300-native (sm_103a) sparse hot path of ARMSparse.

CSR SpMM (fp32 bit-identical to the reference's rowBaseSpmm3; bf16 storage with fp32
accumulation, optionally a bf16 output with a ReLU in the same store), CSR SpMV (plain and the
reference's 1x4-blocked layout), SDDMM (FP32 CUDA cores and tcgen05 split-bf16), the SpMM with
the SDDMM fused into its pass (the backward of a layer with trainable edge values), a
deterministic CSR->CSC transpose (optionally with the CSR position of each entry), the
sum/max aggregations, the sparse x sparse -> dense product and the GCN's softmax cross-entropy,
behind the C ABI in include/armsparse_gpu.h. The ops need the CUDA library built in-tree and a
GPU; there is no CPU fallback.
"""
from .sparse import (csr2csc, csr2csc_perm, csr_to_rowpair, csr_to_vcsr4, dense_to_csr,
                     gather, sddmm, spmm_rowpair, spmm_vcsr4,
                     sddmm_coo, softmax_xent, softmax_xent_grad, spgemm_dense, spmm,
                     spmm_default_variant, spmm_reduce, spmm_sddmm, spmm_variant_supported,
                     spmm_variants, spmv, spmv_vcsr4, sync_status, to_bf16, validate_csr)
from ._native import NativeError, Context, context

__all__ = ["spmm", "spmm_reduce", "spmm_sddmm", "spgemm_dense", "spmv", "spmv_vcsr4", "sddmm",
           "sddmm_coo", "csr2csc", "csr2csc_perm", "gather", "softmax_xent", "softmax_xent_grad",
           "csr_to_vcsr4", "csr_to_rowpair", "spmm_rowpair", "spmm_vcsr4", "dense_to_csr",
           "validate_csr", "sync_status", "to_bf16",
           "spmm_variants", "spmm_default_variant", "spmm_variant_supported", "NativeError",
           "Context", "context"]
