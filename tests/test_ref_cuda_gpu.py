"""The reference's own CUDA kernels (gcn/pytorch-custom/spmm_kernel.cu, sddmm.cu, compiled
here for sm_103a by oracle/Makefile's ref-cuda target) on the same GPU as this library's:
their outputs against ours and against FP64, on the full-size workloads. Skipped where the
cubins were not built (no reference sources)."""
import numpy as np
import pytest
import torch

import armsparse_gb300 as A
from armsparse_gb300 import synthetic as S
from gpu_util import bits, dev, to_dev

pytestmark = pytest.mark.gpu

ref_gpu = pytest.importorskip("oracle.ref_gpu")
if not ref_gpu.available():
    pytest.skip("reference cubins not built", allow_module_level=True)


@pytest.mark.parametrize("N", [4096, 48, 16])
def test_reference_spmm_cuda_matches_ours(N):
    """spmm_cuda's kernels accumulate acc += val * B in CSR order, which nvcc contracts to one
    fused multiply-add per entry: the same chain as rowBaseSpmm3 and this library's row-split
    kernels, so the outputs agree bit for bit (spmm_test2 at N = 4096, spmm_test1 at 48,
    spmm_test0 at 16)."""
    a = S.spmm_4096_d001(0)
    B = S.dense_uniform((4096, N), 1)
    rp, ci, v, Bd = to_dev(a.rowptr), to_dev(a.colind), to_dev(a.val), to_dev(B)
    ref = ref_gpu.spmm_cuda(rp, ci, v, Bd)
    ours = A.spmm(rp, ci, v, Bd)
    torch.cuda.synchronize()
    assert np.array_equal(bits(ref), bits(ours))


def test_reference_sddmm_cuda_csr_close_to_fp64(oracle):
    """sddmm_cuda_csr (sddmmCSR2Scale) on the 4096^3 density-0.1 pattern cut to a multiple of
    16 entries (its tail blocks read past row ends otherwise): within 1e-5 of FP64 like ours
    (its sums run in a different order, so not bit for bit)."""
    a = S.sddmm_4096_d01(0)
    nnz = a.nnz - a.nnz % 16
    rowptr = np.minimum(a.rowptr, nnz).astype(np.int32)
    X = S.dense_normal((4096, 4096), 1)
    Y = S.dense_normal((4096, 4096), 2)
    rp, ci = to_dev(rowptr), to_dev(a.colind[:nnz])
    Xd, Yd = to_dev(X), to_dev(Y)
    ref = ref_gpu.sddmm_cuda_csr(rp, ci, Xd, Yd)
    ours = A.sddmm(rp, ci, Xd, Yd)
    X64, Y64 = Xd.double(), Yd.double()
    r64 = A.sddmm(rp, ci, X64, Y64)
    s64 = A.sddmm(rp, ci, X64.abs(), Y64.abs())
    for got in (ref, ours):
        err = ((got.double() - r64).abs() / torch.maximum(r64.abs(), s64)).max().item()
        assert err < 1e-5, err
    with pytest.raises(ValueError):
        ref_gpu.sddmm_cuda_csr(to_dev(a.rowptr), to_dev(a.colind), Xd, Yd)  # nnz % 16 != 0
