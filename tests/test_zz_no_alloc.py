"""as_csr2csc_static -- the transpose for callers that cannot allocate device memory (a plugin
whose host framework owns all device memory, a serving loop that forbids allocation after
start-up). The caller allocates inputs and outputs; the entry point uses a fixed device array
inside the library as scratch and allocates nothing. Checked through the C ABI against
as_csr2csc on matrices called back to back (each call reuses the array the previous one left
behind), against the oracle with and without values, on an empty matrix, for its size limit,
and for allocating no device memory. This file runs last (its name sorts
last) and passes both alone and after the other tests."""
import numpy as np
import pytest
import torch

import armsparse_gb300 as A
from armsparse_gb300 import _native as N
from armsparse_gb300 import synthetic as S

pytestmark = pytest.mark.gpu

MAX_NNZ = 1 << 18  # AS_CSR2CSC_STATIC_MAX_NNZ in include/armsparse_gpu.h


def _static_transpose(a, dev, values=True):
    t = lambda x: torch.from_numpy(x).to(dev)
    rp, ci, v = t(a.rowptr), t(a.colind), t(a.val)
    colptr = torch.full((a.n_cols + 1,), -7, dtype=torch.int32, device=dev)
    rowind = torch.full((max(a.nnz, 1),), -7, dtype=torch.int32, device=dev)
    cscval = torch.full((max(a.nnz, 1),), float("nan"), device=dev)
    st = N.load().as_csr2csc_static(a.n_rows, a.n_cols, a.nnz, rp.data_ptr(), ci.data_ptr(),
                                    v.data_ptr() if values else None, colptr.data_ptr(),
                                    rowind.data_ptr(), cscval.data_ptr() if values else None,
                                    torch.cuda.current_stream(dev).cuda_stream)
    return st, (colptr, rowind, cscval), (rp, ci, v)


def test_static_transpose_matches_as_csr2csc_two_calls_in_a_row():
    dev = torch.device("cuda", 0)
    first = S.powerlaw_csr(60000, 2.0, 4.0, seed=31)       # 60,000 columns: 2 radix passes
    second = S.spmm_4096_d001(seed=32)                     # 167,772 entries, 4096 columns
    third = S.uniform_csr(900, 70000, 50000, seed=33)      # 70,000 columns: 3 radix passes
    for a in (first, second, third):
        assert a.nnz <= MAX_NNZ
        st, (cp, ri, cv), (rp, ci, v) = _static_transpose(a, dev)
        assert st == 0
        ecp, eri, ecv = A.csr2csc(rp, ci, v, a.n_cols)
        torch.cuda.synchronize()
        assert torch.equal(cp, ecp)
        assert torch.equal(ri, eri)
        assert torch.equal(cv.view(torch.int32), ecv.view(torch.int32))


def test_static_transpose_rejects_more_entries_than_its_array():
    dev = torch.device("cuda", 0)
    a = S.uniform_csr(1024, 1024, MAX_NNZ + 1, seed=34)
    st, (cp, ri, cv), _ = _static_transpose(a, dev)
    torch.cuda.synchronize()
    assert st == 3  # AS_ERR_UNSUPPORTED, nothing launched
    assert bool((cp == -7).all()) and bool((ri == -7).all())


def test_static_transpose_pattern_only_empty_and_oracle(oracle):
    """The pattern-only form (val = NULL: colptr and rowind only), an empty matrix, and the
    result against the oracle's stable counting transpose directly."""
    dev = torch.device("cuda", 0)
    a = S.powerlaw_csr(20000, 2.1, 6.0, seed=35, n_cols=30000)
    st, (cp, ri, cv), _ = _static_transpose(a, dev, values=False)
    torch.cuda.synchronize()
    assert st == 0
    ocp, ori, ocv = oracle.csr2csc(a.rowptr, a.colind, a.val, a.n_cols)
    assert np.array_equal(cp.cpu().numpy(), ocp) and np.array_equal(ri.cpu().numpy(), ori)
    assert bool(torch.isnan(cv).all())  # no values asked for, none written
    st, (cp, ri, cv), _ = _static_transpose(a, dev)
    torch.cuda.synchronize()
    assert st == 0 and np.array_equal(cv.cpu().numpy().view(np.uint32), ocv.view(np.uint32))
    empty = S.CSR(np.zeros(11, np.int32), np.zeros(0, np.int32), np.zeros(0, np.float32), 10, 7)
    st, (cp, ri, cv), _ = _static_transpose(empty, dev, values=False)  # empty: NULL pointers
    torch.cuda.synchronize()
    assert st == 0 and bool((cp == 0).all())


def test_static_transpose_allocates_no_device_memory():
    """After a first call, further calls leave the device's free memory unchanged: a call that
    fell back to cudaMalloc for its ~3 MB of scratch would show (above the driver's 2 MB
    allocation granularity)."""
    dev = torch.device("cuda", 0)
    a = S.spmm_4096_d001(seed=36)
    t = lambda x: torch.from_numpy(x).to(dev)
    rp, ci, v = t(a.rowptr), t(a.colind), t(a.val)
    cp = torch.empty(a.n_cols + 1, dtype=torch.int32, device=dev)
    ri = torch.empty(a.nnz, dtype=torch.int32, device=dev)
    cv = torch.empty(a.nnz, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    call = lambda: N.load().as_csr2csc_static(a.n_rows, a.n_cols, a.nnz, rp.data_ptr(),
                                              ci.data_ptr(), v.data_ptr(), cp.data_ptr(),
                                              ri.data_ptr(), cv.data_ptr(), stream)
    assert call() == 0
    torch.cuda.synchronize()
    free0 = torch.cuda.mem_get_info(dev)[0]
    for _ in range(5):
        assert call() == 0
    torch.cuda.synchronize()
    assert torch.cuda.mem_get_info(dev)[0] >= free0
