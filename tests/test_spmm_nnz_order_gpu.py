"""Entry-balanced SpMM kernels against the oracle's statement of their order, bit for bit."""
import numpy as np
import pytest
import torch

import armsparse_gb300 as A
from armsparse_gb300 import synthetic as S
from gpu_util import csr_dev, to_dev

pytestmark = pytest.mark.gpu


def _graph(seed):
    rng = np.random.default_rng(seed)
    lens = rng.integers(0, 12, 900)
    lens[:3] = 0
    lens[10], lens[400], lens[401] = 5000, 700, 129
    rp = np.zeros(901, np.int32)
    np.cumsum(lens, out=rp[1:])
    ci = np.concatenate([np.sort(rng.choice(6000, l, replace=False)) for l in lens]).astype(np.int32)
    return S.CSR(rp, ci, rng.uniform(-1, 1, ci.size).astype(np.float32), 900, 6000)


def _params(name):
    parts = name.split("_")
    f = {p[0]: p[1:] for p in parts[1:] if p[:1] in "vgc" and p[1:].isdigit()}
    ch = int(next(p[2:] for p in parts if p.startswith("ch")))
    sub = 32 // int(f["g"]) if parts[0] == "nnzme" else 1
    return ch, sub


@pytest.mark.parametrize("dtype", [torch.float32, torch.bfloat16])
@pytest.mark.parametrize("N_", [8, 40, 64])
def test_entry_balanced_bit_exact(oracle, dtype, N_):
    a = _graph(N_)
    B = S.dense_uniform((6000, N_), N_ + 1)
    C0 = S.dense_uniform((900, N_), N_ + 2)
    if dtype == torch.bfloat16:
        v, Bh = oracle.bf16_round(a.val), oracle.bf16_round(B)
    else:
        v, Bh = a.val, B
    rp, ci, _ = csr_dev(a)
    vd, Bd = to_dev(v).to(dtype), to_dev(Bh).to(dtype)
    ran = 0
    for i, name in enumerate(A.spmm_variants(dtype)):
        if not name.startswith(("nnzsplit", "nnzme")) or not A.spmm_variant_supported(i + 1, N_, dtype):
            continue
        ch, sub = _params(name)
        want = oracle.spmm_nnz_order_f32(a.rowptr, a.colind, v, Bh, ch, sub)
        got = A.spmm(rp, ci, vd, Bd, variant=i + 1).cpu().numpy()
        assert np.array_equal(got.view(np.uint32), want.view(np.uint32)), name
        if dtype == torch.float32:
            Cd = to_dev(C0.copy())
            A.spmm(rp, ci, vd, Bd, C=Cd, beta=0.5, variant=i + 1)
            want_b = oracle.spmm_nnz_order_f32(a.rowptr, a.colind, v, Bh, ch, sub, C=C0, beta=0.5)
            assert np.array_equal(Cd.cpu().numpy().view(np.uint32), want_b.view(np.uint32)), name
        ran += 1
    assert ran >= 6
    A.sync_status()
