"""The row-pair reuse layout of the reference's suitesparse_sdmm.cpp on the GPU: the converter
(toDataReuseFormat, :150-179) and the SpMM over it (DataReuseSpmm, :25-44) against the golden
vectors the reference's own code produced and against the oracle's restatement, bit for bit;
the reference-signature host shims likewise."""
import ctypes

import numpy as np
import pytest
import torch

import armsparse_gb300 as A
from armsparse_gb300 import synthetic as S
from gpu_util import bits, dev, to_dev

pytestmark = pytest.mark.gpu


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def test_rowpair_matches_reference_golden(golden):
    g = golden["rowpair_reuse"]
    for i in range(int(g["n_cases"])):
        M, K, N = (int(x) for x in g[f"c{i}_shape"])
        rp, ci, v = (to_dev(g[f"c{i}_{k}"]) for k in ("rowptr", "colind", "val"))
        rp2, ci2, v2, f2 = A.csr_to_rowpair(rp, ci, v)
        assert np.array_equal(rp2.cpu().numpy(), g[f"c{i}_rowptr2"]), i
        assert np.array_equal(ci2.cpu().numpy(), g[f"c{i}_colind2"]), i
        assert np.array_equal(bits(v2), g[f"c{i}_val2"].view(np.uint32)), i
        assert np.array_equal(f2.cpu().numpy(), g[f"c{i}_flag2"]), i
        C = A.spmm_rowpair(rp2, ci2, v2, f2, to_dev(g[f"c{i}_B"]))
        assert np.array_equal(bits(C), g[f"c{i}_C"].view(np.uint32)), i
    A.sync_status()


@pytest.mark.parametrize("N", [1, 7, 64, 256, 1000])
def test_rowpair_against_oracle_banded_and_skewed(oracle, N):
    """Banded rows (pairs share most columns) and power-law rows, with accumulate."""
    for a in (S.banded_csr(3001, 9, seed=91), S.powerlaw_csr(4000, 2.0, 12.0, seed=92)):
        rp, ci, v = to_dev(a.rowptr), to_dev(a.colind), to_dev(a.val)
        rp2, ci2, v2, f2 = A.csr_to_rowpair(rp, ci, v)
        orp, oci, ov, of = oracle.csr_to_rowpair(a.rowptr, a.colind, a.val)
        assert np.array_equal(rp2.cpu().numpy(), orp) and np.array_equal(ci2.cpu().numpy(), oci)
        assert np.array_equal(f2.cpu().numpy(), of)
        B = S.dense_uniform((a.n_cols, N), 93)
        C0 = S.dense_uniform((a.n_rows, N), 94)
        C = to_dev(C0)
        A.spmm_rowpair(rp2, ci2, v2, f2, to_dev(B), C=C, beta=1.0)
        ref = oracle.spmm_rowpair_f32(orp, oci, ov, of, B, C=C0)
        assert np.array_equal(bits(C), bits(ref)), N
    A.sync_status()


def test_rowpair_host_shims(golden):
    from armsparse_gb300 import build
    drv = ctypes.CDLL(build.build_drivers())
    g = golden["rowpair_reuse"]
    for i in range(int(g["n_cases"])):
        M, K, N = (int(x) for x in g[f"c{i}_shape"])
        dense = np.zeros((M, K), np.float32)
        rows = np.repeat(np.arange(M), np.diff(g[f"c{i}_rowptr"]))
        dense[rows, g[f"c{i}_colind"]] = g[f"c{i}_val"]
        nnz = int(g[f"c{i}_rowptr"][-1])
        rp2 = np.zeros(M + 1, np.int32)
        ci2 = np.zeros(nnz, np.int32)
        v2 = np.zeros(nnz, np.float32)
        f2 = np.zeros(nnz, np.uint8)
        work = dense.copy()
        drv.as_drv_toDataReuseFormat(_p(work), M, K, _p(rp2), _p(ci2), _p(v2), _p(f2))
        assert drv.as_drv_last_status() == 0
        assert np.array_equal(rp2, g[f"c{i}_rowptr2"]) and np.array_equal(ci2, g[f"c{i}_colind2"])
        assert np.array_equal(v2.view(np.uint32), g[f"c{i}_val2"].view(np.uint32))
        assert np.array_equal(f2, g[f"c{i}_flag2"])
        moved = np.zeros_like(dense, bool)
        for r in range(0, M - 1, 2):
            for e in range(rp2[r], rp2[r + 1]):
                if f2[e]:
                    moved[r + 1, ci2[e]] = True
        assert moved.any() and (work[moved] == 0).all() and (work[~moved] == dense[~moved]).all()
        B = np.ascontiguousarray(g[f"c{i}_B"])
        C = np.zeros((M, N), np.float32)
        drv.as_drv_DataReuseSpmm(_p(rp2), _p(ci2), _p(v2), _p(B), _p(C), M, K, N, 8, _p(f2))
        assert drv.as_drv_last_status() == 0
        assert np.array_equal(C.view(np.uint32), g[f"c{i}_C"].view(np.uint32))


@pytest.mark.parametrize("N", [3, 8, 64, 300])
def test_vcsr4_spmm_is_the_csr_chain(oracle, N):
    """The SpMM over the reference's 1x4-blocked layout, built on the GPU from CSR, gives the
    CSR chain bit for bit (empty slots skipped), with accumulate; and the format tuner times
    all three layouts and reports one of them."""
    from armsparse_gb300 import tuner
    for a in (S.banded_csr(5000, 11, seed=95), S.powerlaw_csr(3000, 2.0, 9.0, seed=96)):
        rp, ci, v = to_dev(a.rowptr), to_dev(a.colind), to_dev(a.val)
        vr, vc, vv = A.csr_to_vcsr4(rp, ci, v)
        B = S.dense_uniform((a.n_cols, N), 97)
        C0 = S.dense_uniform((a.n_rows, N), 98)
        C = to_dev(C0)
        A.spmm_vcsr4(vr, vc, vv, to_dev(B), C=C, beta=1.0)
        ref = oracle.spmm_fma_chain_f32(a.rowptr, a.colind, a.val, B, C=C0)
        assert np.array_equal(bits(C), bits(ref)), N
        res = tuner.autotune_formats(rp, ci, v, to_dev(B), reps=2, exact=False)
        assert res["pick"] in ("csr", "vcsr4", "rowpair")
        assert all(t["ms"] > 0 for t in res["times"].values())
    A.sync_status()


def test_vcsr4_spmm_long_rows(oracle):
    """Rows past 256 slots (one past 16,384) go to the long-row kernel with its zero-skipping
    step: still the CSR chain bit for bit, with and without accumulate, for 16-byte (N = 64)
    and 4-byte (N = 47) copies."""
    rng = np.random.default_rng(99)
    n_rows, n_cols = 2000, 40000
    lens = rng.integers(0, 40, n_rows)
    lens[[5, 700, 1500]] = [30000, 3000, 300]
    rp_h = np.zeros(n_rows + 1, np.int32)
    np.cumsum(lens, out=rp_h[1:])
    ci_h = np.concatenate([np.sort(rng.choice(n_cols, l, replace=False)) for l in lens]).astype(np.int32)
    a = S.CSR(rp_h, ci_h, rng.uniform(-1, 1, ci_h.size).astype(np.float32), n_rows, n_cols)
    rp, ci, v = to_dev(a.rowptr), to_dev(a.colind), to_dev(a.val)
    vr, vc, vv = A.csr_to_vcsr4(rp, ci, v)
    assert int(torch.diff(vr).max()) > 16384
    for N in (47, 64):
        B = S.dense_uniform((n_cols, N), 100 + N)
        C = A.spmm_vcsr4(vr, vc, vv, to_dev(B))
        ref = oracle.spmm_fma_chain_f32(a.rowptr, a.colind, a.val, B)
        assert np.array_equal(bits(C), bits(ref)), N
        C0 = S.dense_uniform((n_rows, N), 200 + N)
        C = to_dev(C0)
        A.spmm_vcsr4(vr, vc, vv, to_dev(B), C=C, beta=1.0)
        ref = oracle.spmm_fma_chain_f32(a.rowptr, a.colind, a.val, B, C=C0)
        assert np.array_equal(bits(C), bits(ref)), N
    A.sync_status()


def test_rowpair_long_pairs(oracle):
    """Pairs past 256 entries (one past 16,384, whose rows share most columns, and one with no
    partner at the end) go to the long-row kernel's row-pair step: a unit per row of the pair,
    the odd row chaining over the shared columns first. Bit for bit the oracle's restatement of
    DataReuseSpmm, with and without accumulate, for 16-byte (N = 64) and 4-byte (N = 47)
    copies."""
    rng = np.random.default_rng(101)
    n_rows, n_cols = 1001, 50000
    lens = rng.integers(0, 30, n_rows)
    lens[[10, 11, 400, 1000]] = [20000, 18000, 2000, 700]
    cols = [np.sort(rng.choice(n_cols, l, replace=False)) for l in lens]
    # rows 10 and 11 share most of their columns (many flagged entries)
    shared = np.sort(rng.choice(cols[10], 15000, replace=False))
    rest = np.setdiff1d(np.arange(n_cols), cols[10])
    cols[11] = np.sort(np.concatenate([shared, rng.choice(rest, 3000, replace=False)]))
    lens[11] = cols[11].size
    rp_h = np.zeros(n_rows + 1, np.int32)
    np.cumsum(lens, out=rp_h[1:])
    ci_h = np.concatenate(cols).astype(np.int32)
    a = S.CSR(rp_h, ci_h, rng.uniform(-1, 1, ci_h.size).astype(np.float32), n_rows, n_cols)
    rp, ci, v = to_dev(a.rowptr), to_dev(a.colind), to_dev(a.val)
    rp2, ci2, v2, f2 = A.csr_to_rowpair(rp, ci, v)
    orp, oci, ov, of = oracle.csr_to_rowpair(a.rowptr, a.colind, a.val)
    assert of.sum() > 10000
    for N in (47, 64):
        B = S.dense_uniform((n_cols, N), 102 + N)
        C = A.spmm_rowpair(rp2, ci2, v2, f2, to_dev(B))
        ref = oracle.spmm_rowpair_f32(orp, oci, ov, of, B)
        assert np.array_equal(bits(C), bits(ref)), N
        C0 = S.dense_uniform((n_rows, N), 202 + N)
        C = to_dev(C0)
        A.spmm_rowpair(rp2, ci2, v2, f2, to_dev(B), C=C, beta=1.0)
        ref = oracle.spmm_rowpair_f32(orp, oci, ov, of, B, C=C0)
        assert np.array_equal(bits(C), bits(ref)), N
    A.sync_status()
