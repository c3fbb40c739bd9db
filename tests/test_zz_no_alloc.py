"""as_csr2csc_static -- the transpose for callers that cannot allocate device memory (a plugin
whose host framework owns all device memory, a serving loop that forbids allocation after
start-up). The caller allocates inputs and outputs; the entry point uses a fixed device array
inside the library as scratch and allocates nothing. Checked through the C ABI against
as_csr2csc on two different matrices called back to back (the second call reuses the array
the first one left behind), and for its size limit. This file runs last (its name sorts
last) and passes both alone and after the other tests."""
import numpy as np
import pytest
import torch

import armsparse_gb300 as A
from armsparse_gb300 import _native as N
from armsparse_gb300 import synthetic as S

pytestmark = pytest.mark.gpu

MAX_NNZ = 1 << 18  # AS_CSR2CSC_STATIC_MAX_NNZ in include/armsparse_gpu.h


def _static_transpose(a, dev):
    t = lambda x: torch.from_numpy(x).to(dev)
    rp, ci, v = t(a.rowptr), t(a.colind), t(a.val)
    colptr = torch.full((a.n_cols + 1,), -7, dtype=torch.int32, device=dev)
    rowind = torch.full((a.nnz,), -7, dtype=torch.int32, device=dev)
    cscval = torch.full((a.nnz,), float("nan"), device=dev)
    st = N.load().as_csr2csc_static(a.n_rows, a.n_cols, a.nnz, rp.data_ptr(), ci.data_ptr(),
                                    v.data_ptr(), colptr.data_ptr(), rowind.data_ptr(),
                                    cscval.data_ptr(), torch.cuda.current_stream(dev).cuda_stream)
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
