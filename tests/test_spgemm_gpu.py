"""Sparse x sparse -> dense on the GPU through the C ABI, against golden vectors made by the
reference's own sparse_matrix_mul3 (SpMM.cpp:309-327) and against the oracle at the SpMM
driver's shape: bit-identical, including the driver's accumulate pattern."""
import ctypes

import numpy as np
import pytest
import torch

import armsparse_gb300 as A
from armsparse_gb300 import _native as N
from armsparse_gb300 import synthetic as S
from gpu_util import bits, csr_dev, dev, to_dev

pytestmark = pytest.mark.gpu


def _golden_args(g, i):
    return [g[f"c{i}_{x}"] for x in ("a_rowptr", "a_colind", "a_val", "b_rowptr", "b_colind",
                                     "b_val")]


def test_golden_sparse_matrix_mul3(golden):
    g = golden["spgemm_dense"]
    for i in range(int(g["n_cases"])):
        M, K, Nn = (int(x) for x in g[f"c{i}_shape"])
        args = [to_dev(x) for x in _golden_args(g, i)]
        C = A.spgemm_dense(*args, Nn)
        assert np.array_equal(bits(C), bits(g[f"c{i}_C"])), i
        A.spgemm_dense(*args, Nn, C=C, beta=1.0)
        assert np.array_equal(bits(C), bits(g[f"c{i}_C_twice"])), i
    A.sync_status()


@pytest.mark.parametrize("M,K,Nn,da,db,seed", [(4096, 4096, 4096, 0.01, 0.01, 0),
                                                 (3000, 500, 47, 0.02, 0.05, 1),
                                                 (1, 300, 2500, 0.5, 0.01, 2),
                                                 (700, 900, 1, 0.01, 0.3, 3)])
def test_against_oracle(oracle, M, K, Nn, da, db, seed):
    """The driver's shape (4096^3 at density 0.01 for both operands, four column tiles of
    1024) and ragged ones, with C inside a wider buffer."""
    a = S.uniform_csr(M, K, max(1, int(da * M * K)), seed=seed)
    b = S.uniform_csr(K, Nn, max(1, int(db * K * Nn)), seed=seed + 100)
    C0 = S.dense_uniform((M, Nn), seed + 200)
    ref = oracle.spgemm_dense_f32(a.rowptr, a.colind, a.val, b.rowptr, b.colind, b.val, Nn,
                                  C=C0)
    Cw = torch.zeros((M, Nn + 5), device=dev())
    C = Cw[:, 2:Nn + 2]
    C.copy_(to_dev(C0))
    A.spgemm_dense(*csr_dev(a), *csr_dev(b), Nn, C=C, beta=1.0)
    assert np.array_equal(bits(C.contiguous()), bits(ref))
    assert torch.count_nonzero(Cw[:, :2]) == 0 and torch.count_nonzero(Cw[:, Nn + 2:]) == 0
    # overwrite, run to run identical
    C1 = A.spgemm_dense(*csr_dev(a), *csr_dev(b), Nn)
    assert torch.equal(C1, A.spgemm_dense(*csr_dev(a), *csr_dev(b), Nn))
    ref0 = oracle.spgemm_dense_f32(a.rowptr, a.colind, a.val, b.rowptr, b.colind, b.val, Nn)
    assert np.array_equal(bits(C1), bits(ref0))
    A.sync_status()


def test_long_b_rows_and_empty_operands(oracle):
    """B rows longer than one warp's 32 entries (several rounds per A entry), empty rows in
    both operands, no entries at all."""
    rng = np.random.default_rng(9)
    b = S.uniform_csr(50, 3000, 50 * 400, seed=10)  # 400 entries per B row
    a = S.uniform_csr(200, 50, 2000, seed=11)
    ref = oracle.spgemm_dense_f32(a.rowptr, a.colind, a.val, b.rowptr, b.colind, b.val, 3000)
    C = A.spgemm_dense(*csr_dev(a), *csr_dev(b), 3000)
    assert np.array_equal(bits(C), bits(ref))
    z = torch.zeros(201, dtype=torch.int32, device=dev())
    e = torch.zeros(0, dtype=torch.int32, device=dev())
    ev = torch.zeros(0, device=dev())
    C = A.spgemm_dense(z, e, ev, *csr_dev(b), 3000)
    assert torch.count_nonzero(C) == 0
    C2 = torch.full((200, 3000), 3.0, device=dev())
    A.spgemm_dense(z, e, ev, *csr_dev(b), 3000, C=C2, beta=0.5)
    assert torch.all(C2 == 1.5)
    del rng
    A.sync_status()


def test_malformed_is_flagged_not_faulted():
    a = S.uniform_csr(100, 60, 600, seed=4)
    b = S.uniform_csr(60, 80, 500, seed=5)
    bad_b = b.colind.copy()
    bad_b[3] = 80  # column out of range in B
    A.spgemm_dense(*csr_dev(a), to_dev(b.rowptr), to_dev(bad_b), to_dev(b.val), 80)
    with pytest.raises(N.NativeError) as ei:
        A.sync_status()
    assert ei.value.status == 2
    bad_a = a.colind.copy()
    bad_a[7] = 60  # row of B out of range
    A.spgemm_dense(to_dev(a.rowptr), to_dev(bad_a), to_dev(a.val), *csr_dev(b), 80)
    with pytest.raises(N.NativeError):
        A.sync_status()
    A.sync_status()


def test_drivers_shim(golden):
    from armsparse_gb300 import build
    drv = ctypes.CDLL(build.build_drivers())
    p = lambda x: x.ctypes.data_as(ctypes.c_void_p)
    g = golden["spgemm_dense"]
    for i in range(int(g["n_cases"])):
        M, K, Nn = (int(x) for x in g[f"c{i}_shape"])
        arrs = [np.ascontiguousarray(x) for x in _golden_args(g, i)]
        C = np.zeros((M, Nn), np.float32)
        drv.as_drv_sparse_matrix_mul3(*[p(x) for x in arrs], p(C), M, K, Nn, 16)
        assert drv.as_drv_last_status() == 0
        assert np.array_equal(C.view(np.uint32), g[f"c{i}_C"].view(np.uint32)), i
        drv.as_drv_sparse_matrix_mul3(*[p(x) for x in arrs], p(C), M, K, Nn, 16)
        assert np.array_equal(C.view(np.uint32), g[f"c{i}_C_twice"].view(np.uint32)), i
