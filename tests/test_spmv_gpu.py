"""SpMV on the GPU: the reference's 1x4-blocked layout bit-exact against its golden
vectors, plain CSR against FP64."""
import numpy as np
import pytest
import torch

import armsparse_gb300 as A
from armsparse_gb300 import _native as N
from armsparse_gb300 import synthetic as S
from gpu_util import bits, csr_dev, dev, to_dev

pytestmark = pytest.mark.gpu


def test_vcsr4_golden(golden):
    g = golden["spmv_vcsr4"]
    for i in range(int(g["n_cases"])):
        y = A.spmv_vcsr4(to_dev(g[f"c{i}_vrowptr"]), to_dev(g[f"c{i}_vcolind"]),
                         to_dev(g[f"c{i}_vval"]), to_dev(g[f"c{i}_x"]))
        assert np.array_equal(bits(y), bits(g[f"c{i}_y"])), i
    A.sync_status()


def test_vcsr4_full_size_and_accumulate(oracle):
    a = S.spmm_4096_d001(seed=3)
    vr, vc, vv = oracle.csr_to_vcsr4(a.rowptr, a.colind, a.val)
    x = S.dense_uniform(4096, 4)
    y0 = S.dense_uniform(4096, 5)
    ref = oracle.spmv_vcsr4_f32(vr, vc, vv, x, y=y0, fused=True)
    y = to_dev(y0)
    A.spmv_vcsr4(to_dev(vr), to_dev(vc), to_dev(vv), to_dev(x), y=y, beta=1.0)
    assert np.array_equal(bits(y), bits(ref))
    A.sync_status()


def test_vcsr4_long_rows(oracle):
    """Rows past 4,096 slots (the longest 93,719 entries) get a CTA each: batches of blocks
    staged in shared memory, the four chains run in block order by four threads and combined
    as (s2 + s0) + (s3 + s1): bit for bit the reference's sums, with and without accumulate."""
    a = S.powerlaw_csr(200_000, 2.2, 10.0, seed=3)
    vr, vc, vv = oracle.csr_to_vcsr4(a.rowptr, a.colind, a.val)
    assert np.diff(vr).max() > 4096
    x = S.dense_uniform(a.n_cols, 7)
    y0 = S.dense_uniform(a.n_rows, 8)
    vrd, vcd, vvd, xd = to_dev(vr), to_dev(vc), to_dev(vv), to_dev(x)
    ref = oracle.spmv_vcsr4_f32(vr, vc, vv, x, fused=True)
    y = A.spmv_vcsr4(vrd, vcd, vvd, xd)
    assert np.array_equal(bits(y), bits(ref))
    ref = oracle.spmv_vcsr4_f32(vr, vc, vv, x, y=y0, fused=True)
    y = to_dev(y0)
    A.spmv_vcsr4(vrd, vcd, vvd, xd, y=y, beta=1.0)
    assert np.array_equal(bits(y), bits(ref))
    A.sync_status()


@pytest.mark.parametrize("M,K,nnz,kind", [(4096, 4096, 167772, "u"), (1, 10, 5, "u"),
                                           (100000, 100000, 0, "p"), (300000, 300000, 0, "h"),
                                           (3000, 3000, 0, "b"),
                                           (50, 50, 0, "e")])
def test_csr_against_fp64(oracle, M, K, nnz, kind):
    if kind == "u":
        a = S.uniform_csr(M, K, nnz, seed=1)
    elif kind == "p":
        a = S.powerlaw_csr(M, 2.1, 8.0, seed=2)
    elif kind == "h":  # a 300,000-entry hub row and many past 4,096 (a CTA each)
        a = S.powerlaw_csr(M, 2.0, 20.0, seed=0)
    elif kind == "b":
        a = S.banded_csr(M, 9, seed=3)
    else:
        a = S.CSR(np.zeros(M + 1, np.int32), np.zeros(0, np.int32), np.zeros(0, np.float32), M, K)
    x = S.dense_uniform(a.n_cols, 6)
    ref, ab = oracle.spmv_f64(a.rowptr, a.colind, a.val, x)
    rp, ci, v = csr_dev(a)
    y = A.spmv(rp, ci, v, to_dev(x))
    assert oracle.scaled_err(y.cpu().numpy(), ref, ab).max() < 1e-5
    y2 = A.spmv(rp, ci, v, to_dev(x))
    assert torch.equal(y, y2)
    yb = torch.ones(a.n_rows, device=dev())
    A.spmv(rp, ci, v, to_dev(x), y=yb, beta=2.0)
    assert oracle.scaled_err(yb.cpu().numpy(), ref + 2.0, ab + 2.0).max() < 1e-5
    A.sync_status()


def test_format_builders_match_reference_golden(golden):
    """dense -> CSR equals the reference's toCSR output; CSR -> 1x4 blocks equals the
    reference's toVectorAwareCSR output (both from its compiled code)."""
    g = golden["spmm_rowbasespmm3"]
    for i in range(int(g["n_cases"])):
        M, K, _ = (int(x) for x in g[f"c{i}_shape"])
        rp, ci, v = g[f"c{i}_rowptr"], g[f"c{i}_colind"], g[f"c{i}_val"]
        dense = np.zeros((M, K), np.float32)
        dense[np.repeat(np.arange(M), np.diff(rp)), ci] = v
        r, c, vv = A.dense_to_csr(to_dev(dense))
        assert np.array_equal(r.cpu().numpy(), rp) and np.array_equal(c.cpu().numpy(), ci)
        assert np.array_equal(bits(vv), bits(v))
    g = golden["spmv_vcsr4"]
    for i in range(int(g["n_cases"])):
        vr, vc, vv = A.csr_to_vcsr4(to_dev(g[f"c{i}_rowptr"]), to_dev(g[f"c{i}_colind"]),
                                    to_dev(g[f"c{i}_val"]))
        assert np.array_equal(vr.cpu().numpy(), g[f"c{i}_vrowptr"])
        assert np.array_equal(vc.cpu().numpy(), g[f"c{i}_vcolind"])
        assert np.array_equal(bits(vv), bits(g[f"c{i}_vval"]))


def test_format_builders_large(oracle):
    a = S.powerlaw_csr(20000, 2.0, 30.0, seed=9, n_cols=4096)  # rows longer than 32 entries
    vr, vc, vv = A.csr_to_vcsr4(to_dev(a.rowptr), to_dev(a.colind), to_dev(a.val))
    ovr, ovc, ovv = oracle.csr_to_vcsr4(a.rowptr, a.colind, a.val)
    assert np.array_equal(vr.cpu().numpy(), ovr) and np.array_equal(vc.cpu().numpy(), ovc)
    assert np.array_equal(bits(vv), bits(ovv))
    d = S.to_dense(S.uniform_csr(500, 3000, 40000, seed=3))
    d[7, 11] = -0.0
    r, c, v = A.dense_to_csr(to_dev(d))
    rows, cols = np.nonzero(d != 0)
    assert np.array_equal(c.cpu().numpy(), cols) and int(r[-1]) == rows.size
