"""CSR -> CSC on the GPU: bit-exact against the oracle's stable transpose (scipy's tocsc
order, the reference's fast_transpose run in order), deterministic, an involution."""
import numpy as np
import pytest
import torch

import armsparse_gb300 as A
from armsparse_gb300 import _native as N
from armsparse_gb300 import synthetic as S
from gpu_util import bits, csr_dev, dev, to_dev

pytestmark = pytest.mark.gpu


def _check(oracle, a):
    rp, ci, v = csr_dev(a)
    cp, ri, cv = A.csr2csc(rp, ci, v, a.n_cols)
    ocp, ori, ocv = oracle.csr2csc(a.rowptr, a.colind, a.val, a.n_cols)
    assert np.array_equal(cp.cpu().numpy(), ocp)
    assert np.array_equal(ri.cpu().numpy(), ori)
    assert np.array_equal(bits(cv), bits(ocv))
    return cp, ri, cv


@pytest.mark.parametrize("case", ["u4096", "tiny", "n1", "n256", "n257", "wide70000",
                                  "powerlaw", "banded", "empty_rows_cols", "graph"])
def test_against_oracle(oracle, case):
    a = {
        "u4096": lambda: S.spmm_4096_d001(seed=2),
        "tiny": lambda: S.uniform_csr(3, 4, 5, seed=1),
        "n1": lambda: S.uniform_csr(1000, 1, 300, seed=2),
        "n256": lambda: S.uniform_csr(2000, 256, 30000, seed=3),
        "n257": lambda: S.uniform_csr(2000, 257, 30000, seed=4),
        "wide70000": lambda: S.uniform_csr(3000, 70000, 90000, seed=5),
        "powerlaw": lambda: S.powerlaw_csr(100000, 2.0, 12.0, seed=6),
        "banded": lambda: S.banded_csr(20000, 64, seed=7),
        "empty_rows_cols": lambda: S.uniform_csr(5000, 5000, 2000, seed=8),
        "graph": lambda: S.powerlaw_graph(19717, 88648, seed=9),
    }[case]()
    cp, ri, cv = _check(oracle, a)
    # transposing back gives the original (involution)
    rp2, ci2, v2 = A.csr2csc(cp, ri, cv, a.n_rows)
    assert np.array_equal(rp2.cpu().numpy(), a.rowptr)
    assert np.array_equal(ci2.cpu().numpy(), a.colind)
    assert np.array_equal(bits(v2), bits(a.val))
    A.sync_status()


def test_deterministic_and_pattern_only(oracle):
    a = S.powerlaw_csr(50000, 1.9, 30.0, seed=11)
    rp, ci, v = csr_dev(a)
    r1 = A.csr2csc(rp, ci, v, a.n_cols)
    r2 = A.csr2csc(rp, ci, v, a.n_cols)
    assert all(torch.equal(x, y) for x, y in zip(r1, r2))
    cp, ri, cv = A.csr2csc(rp, ci, None, a.n_cols)
    assert cv is None and torch.equal(cp, r1[0]) and torch.equal(ri, r1[1])


def test_no_entries():
    rp = torch.zeros(8, dtype=torch.int32, device=dev())
    ci = torch.zeros(0, dtype=torch.int32, device=dev())
    cp, ri, cv = A.csr2csc(rp, ci, torch.zeros(0, device=dev()), 5)
    assert cp.tolist() == [0] * 6 and ri.numel() == 0


def test_malformed_colind_flagged():
    a = S.uniform_csr(100, 64, 600, seed=1)
    bad = a.colind.copy()
    bad[5] = 64
    A.csr2csc(to_dev(a.rowptr), to_dev(bad), to_dev(a.val), 64)
    with pytest.raises(N.NativeError) as ei:
        A.sync_status()
    assert ei.value.status == 2
