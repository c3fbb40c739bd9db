"""The reference-signature host shims (libarmsparse_drivers.so) on the GPU, against the
golden vectors made from the reference's own kernels: same arguments, same results."""
import ctypes
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


@pytest.fixture(scope="module")
def drv():
    from armsparse_gb300 import build
    return ctypes.CDLL(build.build_drivers())


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def test_spmm_shims(drv, golden):
    g = golden["spmm_rowbasespmm3"]
    for i in range(int(g["n_cases"])):
        M, K, N = (int(x) for x in g[f"c{i}_shape"])
        rp, ci, v, B = (np.ascontiguousarray(g[f"c{i}_{k}"]) for k in ("rowptr", "colind", "val", "B"))
        C = np.zeros((M, N), np.float32)
        drv.as_drv_rowBaseSpmm3(_p(rp), _p(ci), _p(v), _p(B), _p(C), M, K, N, 32)
        assert drv.as_drv_last_status() == 0
        assert np.array_equal(C.view(np.uint32), g[f"c{i}_C"].view(np.uint32))
        drv.as_drv_rowBaseSpmm3(_p(rp), _p(ci), _p(v), _p(B), _p(C), M, K, N, 32)
        assert np.array_equal(C.view(np.uint32), g[f"c{i}_C_twice"].view(np.uint32))
        Cs = np.zeros((M, N), np.float32)
        drv.as_drv_rowBaseSpmm2(_p(rp), _p(ci), _p(v), _p(B), _p(Cs), M, K, N, 32)
        assert drv.as_drv_last_status() == 0
        # SDMM.cpp:65-89 (cblas_saxpy per entry) compiled from the reference, golden C_saxpy
        assert np.array_equal(Cs.view(np.uint32), g[f"c{i}_C_saxpy"].view(np.uint32))
        Co = np.full((M, N), 7.0, np.float32)
        drv.as_drv_origin(_p(rp), _p(ci), _p(v), _p(B), _p(Co), M, K, N, 32)
        assert np.array_equal(Co.view(np.uint32), g[f"c{i}_C"].view(np.uint32))
        Cg = np.zeros((M, N), np.float32)
        drv.as_drv_csr_spmm_kernel(M, N, _p(rp), _p(ci), _p(v), _p(B), _p(Cg))
        # csr_spmm_kernel infers K = max(colind) + 1; B's leading rows are what it reads
        assert np.array_equal(Cg.view(np.uint32), g[f"c{i}_C"].view(np.uint32))


def test_spmm_shims_column_blocks(drv, oracle):
    """B of 49 MB: the shim runs the SpMM in column blocks (B in, kernel, C out, the copies
    back on a second host thread), here 1024 + 1024 + 952 columns; origin (C = A*B) and
    rowBaseSpmm3 (C += A*B) stay bit-identical to the reference's chain, call after call."""
    from armsparse_gb300 import synthetic as S
    M, K, N = 1500, 4096, 3000
    a = S.uniform_csr(M, K, 30000, seed=91)
    B = S.dense_uniform((K, N), 92)
    ref = oracle.spmm_fma_chain_f32(a.rowptr, a.colind, a.val, B)
    ref2 = oracle.spmm_fma_chain_f32(a.rowptr, a.colind, a.val, B, C=ref)
    rp, ci, v = (np.ascontiguousarray(x) for x in (a.rowptr, a.colind, a.val))
    for _ in range(2):
        C = np.full((M, N), 5.0, np.float32)
        drv.as_drv_origin(_p(rp), _p(ci), _p(v), _p(B), _p(C), M, K, N, 16)
        assert drv.as_drv_last_status() == 0
        assert np.array_equal(C.view(np.uint32), ref.view(np.uint32))
        drv.as_drv_rowBaseSpmm3(_p(rp), _p(ci), _p(v), _p(B), _p(C), M, K, N, 16)
        assert drv.as_drv_last_status() == 0
        assert np.array_equal(C.view(np.uint32), ref2.view(np.uint32))


def test_spmv_shim(drv, golden):
    g = golden["spmv_vcsr4"]
    for i in range(int(g["n_cases"])):
        M = int(g[f"c{i}_shape"][0])
        vr, vc, vv, x = (np.ascontiguousarray(g[f"c{i}_{k}"]) for k in ("vrowptr", "vcolind", "vval", "x"))
        y = np.zeros(M, np.float32)
        drv.as_drv_sparse_dense_vector(_p(x), _p(y), _p(vr), _p(vc), _p(vv), M, 32)
        assert drv.as_drv_last_status() == 0
        assert np.array_equal(y.view(np.uint32), g[f"c{i}_y"].view(np.uint32))


def test_transpose_shim(drv, golden):
    g = golden["transpose_triplets"]
    for i in range(int(g["n_cases"])):
        sm = np.ascontiguousarray(g[f"c{i}_triplets"])
        res = np.zeros_like(sm)
        drv.as_drv_fast_transpose(_p(sm), _p(res))
        assert drv.as_drv_last_status() == 0
        assert np.array_equal(res, g[f"c{i}_transposed"])
