"""The SpMM with the SDDMM fused into its pass (as_spmm_sddmm_csr_*) and the transpose that
gives each CSC entry's CSR position (as_csr2csc_perm): the SpMM half bit-identical to the
unfused nnz-split kernel of the same variant, the dot products bit-identical to the oracle's
statement of the kernel's order, and placed through the permutation."""
import numpy as np
import pytest
import torch

import armsparse_gb300 as A
from armsparse_gb300 import _native as N
from armsparse_gb300 import synthetic as S
from gpu_util import bits, csr_dev, dev, to_dev

pytestmark = pytest.mark.gpu


def _skewed(seed, n_rows=1500, n_cols=3000, long_lens=(2500, 700)):
    rng = np.random.default_rng(seed)
    lens = rng.integers(0, 9, n_rows)
    lens[:5] = 0
    for i, l in enumerate(long_lens):
        lens[100 + 37 * i] = l
    rp = np.zeros(n_rows + 1, np.int32)
    np.cumsum(lens, out=rp[1:])
    ci = np.concatenate([np.sort(rng.choice(n_cols, l, replace=False)) for l in lens]).astype(np.int32)
    return S.CSR(rp, ci, rng.uniform(-1, 1, ci.size).astype(np.float32), n_rows, n_cols)


def _shape(name):
    """(vector bytes, group, vectors per lane) of an nnz-split or multi-entry variant name."""
    f = dict((p[0], p[1:]) for p in name.split("_")[1:] if p[0] in "vgc" and p[1:].isdigit())
    return int(f["v"]), int(f["g"]), int(f.get("c", 1))


def _fusable(dtype, N_):
    esz = 4 if dtype == torch.float32 else 2
    out = []
    for i, name in enumerate(A.spmm_variants(dtype)):
        if not name.startswith(("nnzsplit", "nnzme")) or not A.spmm_variant_supported(i + 1, N_, dtype):
            continue
        vb, g, c = _shape(name)
        if (vb // esz) * g * c >= N_:
            out.append((i + 1, name, g, vb // esz, c))
    return out


@pytest.mark.parametrize("dtype", [torch.float32, torch.bfloat16])
@pytest.mark.parametrize("N_", [48, 64, 256])
def test_fused_matches_spmm_and_slices_oracle(oracle, dtype, N_):
    a = _skewed(N_ + (dtype == torch.bfloat16))
    rp, ci, v = csr_dev(a)
    B = S.dense_uniform((a.n_cols, N_), 3 + N_)
    F = S.dense_uniform((a.n_rows, N_), 4 + N_)
    if dtype == torch.bfloat16:
        B, F, vh = oracle.bf16_round(B), oracle.bf16_round(F), oracle.bf16_round(a.val)
    else:
        vh = a.val
    vd, Bd, Fd = to_dev(vh).to(dtype), to_dev(B).to(dtype), to_dev(F).to(dtype)
    perm = np.random.default_rng(N_).permutation(a.colind.size).astype(np.int32)
    cases = _fusable(dtype, N_)
    assert len(cases) >= 2
    for var, name, g, e, c in cases:
        C, dA = A.spmm_sddmm(rp, ci, vd, Bd, Fd, variant=var)
        assert torch.equal(C, A.spmm(rp, ci, vd, Bd, variant=var)), name
        want = oracle.sddmm_f32_slices(a.rowptr, a.colind, F, B, g, e, c)
        assert np.array_equal(bits(dA), want.view(np.uint32)), name
        C2, dA2 = A.spmm_sddmm(rp, ci, vd, Bd, Fd, perm=to_dev(perm), variant=var)
        assert torch.equal(C2, C), name
        placed = np.empty_like(want)
        placed[perm] = want
        assert np.array_equal(bits(dA2), placed.view(np.uint32)), name
    # library choice: one of the fusable variants, same SpMM bits as that variant
    C0, dA0 = A.spmm_sddmm(rp, ci, vd, Bd, Fd)
    ref, ab = oracle.sddmm_f64(a.rowptr, a.colind, F, B)
    assert oracle.scaled_err(dA0.cpu().numpy(), ref, ab).max() < 1e-5
    A.sync_status()


def test_fused_beta_and_unsupported_tile(oracle):
    a = _skewed(7)
    rp, ci, v = csr_dev(a)
    B = to_dev(S.dense_uniform((a.n_cols, 256), 8))
    F = to_dev(S.dense_uniform((a.n_rows, 256), 9))
    narrow = [var for var, *_ in _fusable(torch.float32, 32)
              if var not in [w for w, *_ in _fusable(torch.float32, 256)]]
    assert narrow
    with pytest.raises(N.NativeError) as e:
        A.spmm_sddmm(rp, ci, v, B, F, variant=narrow[0])
    assert e.value.status == 3  # AS_ERR_UNSUPPORTED: the tile does not cover N
    row_split = 1
    with pytest.raises(N.NativeError) as e:
        A.spmm_sddmm(rp, ci, v, B, F, variant=row_split)
    assert e.value.status == 3
    var = _fusable(torch.float32, 256)[0][0]
    C = torch.full((a.n_rows, 256), 2.0, device=dev())
    C, dA = A.spmm_sddmm(rp, ci, v, B, F, C=C, beta=0.5, variant=var)
    C64, A64 = oracle.spmm_f64(a.rowptr, a.colind, a.val, B.cpu().numpy())
    assert oracle.scaled_err(C.cpu().numpy(), C64 + 1.0, A64 + 1.0).max() < 1e-5
    A.sync_status()


def test_fused_bad_column_is_flagged():
    rp = to_dev(np.array([0, 2, 3], np.int32))
    ci = to_dev(np.array([0, 7, 1], np.int32))  # 7 is out of range for K = 4
    v = to_dev(np.ones(3, np.float32))
    B = torch.ones(4, 64, device=dev())
    F = torch.ones(2, 64, device=dev())
    A.spmm_sddmm(rp, ci, v, B, F)
    with pytest.raises(N.NativeError) as e:
        A.sync_status()
    assert e.value.status == 2  # AS_ERR_INVALID_CSR


@pytest.mark.parametrize("M,Ncols,nnz,kind", [(1, 1, 1, "u"), (300, 500, 6000, "u"),
                                              (20000, 20000, 0, "p"), (70000, 300, 400000, "u")])
def test_csr2csc_perm(oracle, M, Ncols, nnz, kind):
    a = (S.uniform_csr(M, Ncols, nnz, seed=M) if kind == "u"
         else S.powerlaw_csr(M, 2.0, 12.0, seed=3, n_cols=Ncols))
    rp, ci, v = csr_dev(a)
    cp, ri, perm = A.csr2csc_perm(rp, ci, a.n_cols)
    cp0, ri0, cv0 = oracle.csr2csc(a.rowptr, a.colind, a.val, a.n_cols)
    assert np.array_equal(cp.cpu().numpy(), cp0)
    assert np.array_equal(ri.cpu().numpy(), ri0)
    assert np.array_equal(a.val[perm.cpu().numpy()].view(np.uint32), cv0.view(np.uint32))
    assert np.array_equal(np.sort(perm.cpu().numpy()), np.arange(a.colind.size))
    A.sync_status()


def test_fused_bad_permutation_is_flagged_and_skipped():
    rp = to_dev(np.array([0, 2, 3], np.int32))
    ci = to_dev(np.array([0, 3, 1], np.int32))
    v = to_dev(np.ones(3, np.float32))
    B = torch.ones(4, 64, device=dev())
    F = torch.ones(2, 64, device=dev())
    dA = torch.full((3,), -1.0, device=dev())
    perm = to_dev(np.array([2, 9, 0], np.int32))  # 9 is outside [0, 3): that write is skipped
    A.spmm_sddmm(rp, ci, v, B, F, perm=perm, dA=dA)
    with pytest.raises(N.NativeError) as e:
        A.sync_status()
    assert e.value.status == 1  # AS_ERR_INVALID_VALUE
    assert dA.cpu().tolist() == [64.0, -1.0, 64.0]


@pytest.mark.parametrize("N_", [48, 256])
def test_fused_bf16_output(oracle, N_):
    a = _skewed(20 + N_)
    rp, ci, v = csr_dev(a)
    vd = v.to(torch.bfloat16)
    Bd = to_dev(S.dense_uniform((a.n_cols, N_), 21)).to(torch.bfloat16)
    Fd = to_dev(S.dense_uniform((a.n_rows, N_), 22)).to(torch.bfloat16)
    perm = to_dev(np.random.default_rng(N_).permutation(a.colind.size).astype(np.int32))
    for var, name, *_ in _fusable(torch.bfloat16, N_):
        C, dA = A.spmm_sddmm(rp, ci, vd, Bd, Fd, perm=perm, variant=var)
        C16, dA16 = A.spmm_sddmm(rp, ci, vd, Bd, Fd, perm=perm, variant=var,
                                 out_dtype=torch.bfloat16)
        assert torch.equal(C16.view(torch.int16), C.to(torch.bfloat16).view(torch.int16)), name
        assert torch.equal(dA16, dA), name
    A.sync_status()


@pytest.mark.parametrize("n", [0, 3, 4, 1001, 100000])
def test_gather(n):
    gen = torch.Generator(device=dev()).manual_seed(n)
    src = torch.randn(max(n, 1) * 2, generator=gen, device=dev())
    idx = torch.randint(0, src.numel(), (n,), generator=gen, device=dev(), dtype=torch.int32)
    assert torch.equal(A.gather(src, idx), src[idx.long()])
    A.sync_status()
    if n >= 4:
        bad = idx.clone()
        bad[n // 2] = src.numel()  # out of range: that output is 0 and the call is flagged
        out = A.gather(src, bad)
        assert out[n // 2].item() == 0.0
        with pytest.raises(N.NativeError) as e:
            A.sync_status()
        assert e.value.status == 1
