"""SDDMM on the GPU: FP32 CUDA-core path bit-exact against the oracle's 8-lane
restatement and within 1e-5 (scaled) of FP64; reference semantics (unscaled) and scaled."""
import numpy as np
import pytest
import torch

import armsparse_gb300 as A
from armsparse_gb300 import _native as N
from armsparse_gb300 import synthetic as S
from gpu_util import bits, csr_dev, dev, to_dev

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("M,Ncol,K,nnz", [(64, 48, 1, 500), (100, 90, 3, 2000), (300, 200, 8, 6000),
                                          (500, 400, 64, 20000), (200, 300, 100, 5000),
                                          (256, 256, 4096, 6500), (1, 1, 16, 1)])
def test_f32_against_oracle(oracle, M, Ncol, K, nnz):
    a = S.uniform_csr(M, Ncol, nnz, seed=K, values="u0515")
    X = S.dense_normal((M, K), 1)
    Y = S.dense_normal((Ncol, K), 2)
    rp, ci, av = csr_dev(a)
    for aval in (None, a.val):
        out = A.sddmm(rp, ci, to_dev(X), to_dev(Y), aval=None if aval is None else av)
        lanes = oracle.sddmm_f32_lanes(a.rowptr, a.colind, X, Y, aval=aval)
        assert np.array_equal(bits(out), bits(lanes))
        r64, ab = oracle.sddmm_f64(a.rowptr, a.colind, X, Y, aval=aval)
        assert oracle.scaled_err(out.cpu().numpy(), r64, ab).max() < 1e-5
    A.sync_status()


def test_powerlaw_and_empty_rows(oracle):
    a = S.powerlaw_csr(5000, 2.0, 10.0, seed=5)
    X = S.dense_normal((5000, 32), 3)
    Y = S.dense_normal((5000, 32), 4)
    rp, ci, av = csr_dev(a)
    out = A.sddmm(rp, ci, to_dev(X), to_dev(Y), aval=av)
    lanes = oracle.sddmm_f32_lanes(a.rowptr, a.colind, X, Y, aval=a.val)
    assert np.array_equal(bits(out), bits(lanes))
    empty = A.sddmm(to_dev(np.zeros(5, np.int32)), to_dev(np.zeros(0, np.int32)),
                    torch.randn(4, 8, device=dev()), torch.randn(3, 8, device=dev()))
    assert empty.numel() == 0
    A.sync_status()


def test_malformed_pattern_is_flagged():
    a = S.uniform_csr(40, 30, 200, seed=1)
    bad = a.colind.copy()
    bad[3] = -1
    A.sddmm(to_dev(a.rowptr), to_dev(bad), torch.randn(40, 16, device=dev()),
            torch.randn(30, 16, device=dev()))
    with pytest.raises(N.NativeError) as ei:
        A.sync_status()
    assert ei.value.status == 2
