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
        lanes = oracle.sddmm_f32_group(a.rowptr, a.colind, X, Y, aval=aval)
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
    lanes = oracle.sddmm_f32_group(a.rowptr, a.colind, X, Y, aval=a.val)
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


# ---- tensor-core split-bf16 path -----------------------------------------------------------
# Error budget per product: x = hi + lo + r with |lo| <= 2^-9 |x|, |r| <= 2^-18 |x|; the dropped
# lo*lo and r terms are <= ~4 * 2^-18 |x y|, plus FP32 accumulation. Bar: scaled error
# (relative to sum |x_k y_k|) below 3e-5 per output.
TC_TOL = 3e-5
TC_VARIANTS = (1, 2, 3)  # one tile per CTA; persistent with 64-wide / 32-wide K stages


@pytest.mark.parametrize("M,Ncol,K,nnz", [(128, 256, 64, 3000), (300, 500, 100, 15000),
                                          (1000, 700, 4096, 35000), (129, 257, 8, 4000),
                                          (64, 32, 1, 300)])
def test_tc_against_fp64(oracle, M, Ncol, K, nnz):
    a = S.uniform_csr(M, Ncol, nnz, seed=K + 1, values="u0515")
    X = S.dense_normal((M, K), 11)
    Y = S.dense_normal((Ncol, K), 12)
    rp, ci, av = csr_dev(a)
    for variant in TC_VARIANTS:
        for aval in (None, a.val):
            out = A.sddmm(rp, ci, to_dev(X), to_dev(Y), aval=None if aval is None else av,
                          tensor_cores=True, variant=variant)
            r64, ab = oracle.sddmm_f64(a.rowptr, a.colind, X, Y, aval=aval)
            err = oracle.scaled_err(out.cpu().numpy(), r64, ab)
            assert err.max() < TC_TOL, (variant, err.max())
    A.sync_status()


def test_tc_sparse_tiles_and_determinism(oracle):
    a = S.banded_csr(3000, 16, seed=2, values="u0515")  # most 128x256 tiles are empty
    X = S.dense_normal((3000, 256), 13)
    Y = S.dense_normal((3000, 256), 14)
    rp, ci, av = csr_dev(a)
    r64, ab = oracle.sddmm_f64(a.rowptr, a.colind, X, Y, aval=a.val)
    for variant in TC_VARIANTS:
        o1 = A.sddmm(rp, ci, to_dev(X), to_dev(Y), aval=av, tensor_cores=True, variant=variant)
        o2 = A.sddmm(rp, ci, to_dev(X), to_dev(Y), aval=av, tensor_cores=True, variant=variant)
        assert torch.equal(o1, o2)
        assert oracle.scaled_err(o1.cpu().numpy(), r64, ab).max() < TC_TOL, variant
    A.sync_status()


def test_tc_full_size_4096_density_01(oracle):
    """The SDDMM workload at full size: 4096 x 4096 pattern, density 0.1, K = 4096."""
    a = S.sddmm_4096_d01(seed=0)
    X = S.dense_normal((4096, 4096), 1)
    Y = S.dense_normal((4096, 4096), 2)
    rp, ci, av = csr_dev(a)
    out32 = A.sddmm(rp, ci, to_dev(X), to_dev(Y), aval=av)
    r64, ab = oracle.sddmm_f64(a.rowptr, a.colind, X, Y, aval=a.val)
    e_32 = oracle.scaled_err(out32.cpu().numpy(), r64, ab)
    assert e_32.max() < 1e-5
    for variant in TC_VARIANTS:
        out = A.sddmm(rp, ci, to_dev(X), to_dev(Y), aval=av, tensor_cores=True, variant=variant)
        e_tc = oracle.scaled_err(out.cpu().numpy(), r64, ab)
        assert e_tc.max() < TC_TOL, variant
    A.sync_status()


def test_tc_unsorted_rows_flagged():
    a = S.uniform_csr(200, 300, 3000, seed=3)
    bad = a.colind.copy()
    lo = a.rowptr[10]
    bad[lo], bad[lo + 1] = bad[lo + 1], bad[lo]
    A.sddmm(to_dev(a.rowptr), to_dev(bad), torch.randn(200, 64, device=dev()),
            torch.randn(300, 64, device=dev()), tensor_cores=True)
    with pytest.raises(N.NativeError) as ei:
        A.sync_status()
    assert ei.value.status == 2


def test_coo_any_order(oracle):
    a = S.uniform_csr(300, 200, 5000, seed=21, values="u0515")
    X = S.dense_normal((300, 40), 22)
    Y = S.dense_normal((200, 40), 23)
    rows = np.repeat(np.arange(300, dtype=np.int32), np.diff(a.rowptr))
    perm = np.random.default_rng(24).permutation(a.nnz)
    out = A.sddmm_coo(to_dev(rows[perm]), to_dev(a.colind[perm]), to_dev(X), to_dev(Y),
                      aval=to_dev(a.val[perm]))
    lanes = oracle.sddmm_f32_group(a.rowptr, a.colind, X, Y, aval=a.val)
    assert np.array_equal(bits(out), bits(lanes[perm]))
    A.sync_status()


@pytest.mark.parametrize("K", [64, 47, 256])
def test_bf16_inputs_bit_exact(oracle, K):
    """bf16 X and Y, fp32 products and sums: bit for bit the eight-lane fp32 restatement run
    on the bf16 values widened to fp32 (vector path for K % 8 == 0, scalar otherwise)."""
    a = S.uniform_csr(500, 400, 20000, seed=K, values="u0515")
    X = S.dense_normal((500, K), K + 1)
    Y = S.dense_normal((400, K), K + 2)
    Xb, Yb = oracle.bf16_round(X), oracle.bf16_round(Y)
    rp, ci, v = to_dev(a.rowptr), to_dev(a.colind), to_dev(a.val)
    Xd, Yd = to_dev(X).to(torch.bfloat16), to_dev(Y).to(torch.bfloat16)
    for aval, av in ((None, None), (v, a.val)):
        out = A.sddmm(rp, ci, Xd, Yd, aval=aval)
        ref = oracle.sddmm_f32_group(a.rowptr, a.colind, Xb, Yb, aval=av)
        assert np.array_equal(bits(out), bits(ref)), (K, aval is None)
    A.sync_status()
