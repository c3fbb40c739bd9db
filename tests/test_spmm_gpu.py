"""SpMM on the GPU through the C ABI against the oracle (bit-exact for row-split variants,
the reference's rowBaseSpmm3 per-output FMA chain) and against FP64 (bf16 path)."""
import numpy as np
import pytest
import torch

import armsparse_gb300 as A
from armsparse_gb300 import _native as N
from armsparse_gb300 import synthetic as S
from gpu_util import bits, csr_dev, dev, to_dev

pytestmark = pytest.mark.gpu


def _variants(dtype):
    return list(range(1, N.load().as_spmm_variant_count(0 if dtype == torch.float32 else 1) + 1))


def _run_all_supported(rp, ci, v, B):
    outs = {}
    for var in _variants(B.dtype):
        try:
            outs[var] = A.spmm(rp, ci, v, B, variant=var)
        except N.NativeError as e:
            assert e.status == 3, e  # AS_ERR_UNSUPPORTED for layouts a vector width cannot serve
    torch.cuda.synchronize()
    return outs


def test_golden_rowbasespmm3_every_variant(golden, oracle):
    g = golden["spmm_rowbasespmm3"]
    for i in range(int(g["n_cases"])):
        rp, ci, v, B = (to_dev(g[f"c{i}_rowptr"]), to_dev(g[f"c{i}_colind"]),
                        to_dev(g[f"c{i}_val"]), to_dev(g[f"c{i}_B"]))
        outs = _run_all_supported(rp, ci, v, B)
        assert len(outs) >= 18
        names = A.spmm_variants()
        C64, A64 = oracle.spmm_f64(g[f"c{i}_rowptr"], g[f"c{i}_colind"], g[f"c{i}_val"], g[f"c{i}_B"])
        for var, C in outs.items():
            if names[var - 1].startswith(("nnzsplit", "nnzme")):
                # rows that cross a chunk boundary are summed in chunk order (the multi-entry
                # kernels sum every row in sub-group order)
                assert oracle.scaled_err(C.cpu().numpy(), C64, A64).max() < 1e-5, names[var - 1]
            else:
                assert np.array_equal(bits(C), bits(g[f"c{i}_C"])), (i, names[var - 1])
        # the driver's accumulate pattern: a second call with beta = 1
        C = A.spmm(rp, ci, v, B)
        A.spmm(rp, ci, v, B, C=C, beta=1.0)
        assert np.array_equal(bits(C), bits(g[f"c{i}_C_twice"])), i
    A.sync_status()


@pytest.mark.parametrize("M,K,N,nnz,kind", [
    (1, 1, 1, 1, "u"), (5, 3, 1, 7, "u"), (257, 300, 3, 2000, "u"), (1000, 800, 64, 20000, "u"),
    (300, 500, 130, 6000, "u"), (64, 4096, 4096, 2600, "u"), (2000, 2000, 47, 0, "p"),
    (3000, 3000, 256, 0, "p"), (500, 500, 16, 0, "b")])
def test_bit_exact_against_oracle(oracle, M, K, N, nnz, kind):
    if kind == "u":
        a = S.uniform_csr(M, K, nnz, seed=M + N)
    elif kind == "p":
        a = S.powerlaw_csr(M, 2.0, 20.0, seed=N, n_cols=K)
    else:
        a = S.banded_csr(M, 33, seed=3)
    B = S.dense_uniform((a.n_cols, N), seed=7)
    ref = oracle.spmm_fma_chain_f32(a.rowptr, a.colind, a.val, B)
    rp, ci, v = csr_dev(a)
    C = A.spmm(rp, ci, v, to_dev(B))
    assert np.array_equal(bits(C), bits(ref))
    A.sync_status()


def test_full_size_4096_density_001(oracle):
    """The SpMM driver's shape at full size: 4096^3, 167,772 entries: bit-exact."""
    a = S.spmm_4096_d001(seed=0)
    B = S.dense_uniform((4096, 4096), seed=1)
    ref = oracle.spmm_fma_chain_f32(a.rowptr, a.colind, a.val, B)
    rp, ci, v = csr_dev(a)
    Bd = to_dev(B)
    C = A.spmm(rp, ci, v, Bd)
    assert np.array_equal(bits(C), bits(ref))
    # run to run identical, and accumulate == reference accumulate
    C2 = A.spmm(rp, ci, v, Bd)
    assert torch.equal(C, C2)
    A.spmm(rp, ci, v, Bd, C=C2, beta=1.0)
    ref2 = oracle.spmm_fma_chain_f32(a.rowptr, a.colind, a.val, B, C=ref)
    assert np.array_equal(bits(C2), bits(ref2))
    A.sync_status()


def test_strided_b_and_c(oracle):
    a = S.uniform_csr(300, 200, 3000, seed=4)
    Bw = S.dense_uniform((200, 96), seed=5)
    ref = oracle.spmm_fma_chain_f32(a.rowptr, a.colind, a.val, np.ascontiguousarray(Bw[:, :64]))
    rp, ci, v = csr_dev(a)
    Bd = to_dev(Bw)[:, :64]
    Cw = torch.zeros((300, 80), device=dev())
    C = Cw[:, 8:72]
    A.spmm(rp, ci, v, Bd, C=C, beta=0.0)
    assert np.array_equal(bits(C.contiguous()), bits(ref))
    assert torch.count_nonzero(Cw[:, :8]) == 0


def test_edge_cases(oracle):
    # no entries: C = beta * C
    rp = torch.zeros(11, dtype=torch.int32, device=dev())
    ci = torch.zeros(0, dtype=torch.int32, device=dev())
    v = torch.zeros(0, device=dev())
    B = torch.randn(6, 8, device=dev())
    C = A.spmm(rp, ci, v, B)
    assert torch.count_nonzero(C) == 0
    C0 = torch.randn(10, 8, device=dev())
    C1 = C0.clone()
    A.spmm(rp, ci, v, B, C=C1, beta=0.5)
    assert torch.equal(C1, C0 * 0.5)
    # zero rows / zero columns: nothing to do
    A.spmm(torch.zeros(1, dtype=torch.int32, device=dev()), ci, v, B)
    A.spmm(rp, ci, v, torch.zeros(6, 0, device=dev()))
    A.sync_status()


def test_malformed_csr_is_flagged_not_faulted():
    a = S.uniform_csr(100, 50, 500, seed=1)
    bad = a.colind.copy()
    bad[17] = 50  # out of range
    rp, v = to_dev(a.rowptr), to_dev(a.val)
    B = torch.randn(50, 32, device=dev())
    A.spmm(rp, to_dev(bad), v, B)
    with pytest.raises(N.NativeError) as ei:
        A.sync_status()
    assert ei.value.status == 2
    badrp = a.rowptr.copy()
    badrp[40] = badrp[41] + 5  # not monotone
    A.spmm(to_dev(badrp), to_dev(a.colind), v, B)
    with pytest.raises(N.NativeError):
        A.sync_status()
    A.sync_status()  # cleared
    with pytest.raises(N.NativeError):
        A.validate_csr(to_dev(badrp), to_dev(a.colind), 50)
    A.validate_csr(rp, to_dev(a.colind), 50, require_sorted=True)


@pytest.mark.parametrize("N_", [3, 64, 256, 4096])
def test_bf16_storage_fp32_accumulate(oracle, N_):
    M = K = 4096 if N_ == 4096 else 2000
    a = S.uniform_csr(M, K, int(0.01 * M * K), seed=N_)
    B = S.dense_uniform((K, N_), seed=2)
    vb, Bb = oracle.bf16_round(a.val), oracle.bf16_round(B)
    rp, ci, _ = csr_dev(a)
    C = A.spmm(rp, ci, to_dev(a.val).to(torch.bfloat16), to_dev(B).to(torch.bfloat16))
    got = C.cpu().numpy()
    # against FP64 of the bf16-rounded inputs: only FP32 accumulation error
    R, Ab = oracle.spmm_f64(a.rowptr, a.colind, vb, Bb)
    assert oracle.scaled_err(got, R, Ab).max() < 1e-5
    # against FP64 of the original FP32 inputs: the bf16 storage error
    R64, A64 = oracle.spmm_f64(a.rowptr, a.colind, a.val, B)
    assert oracle.scaled_err(got, R64, A64).max() < 1e-2
    A.sync_status()


def test_native_kernels_ran():
    assert N.total_launches() > 0


def _variant_ids(prefix, dtype=torch.float32):
    return [i + 1 for i, n in enumerate(A.spmm_variants(dtype)) if n.startswith(prefix)]


@pytest.mark.parametrize("dtype", [torch.float32, torch.bfloat16])
def test_bulk_staged_variants_bit_exact(oracle, dtype):
    cases = [S.uniform_csr(300, 4096, 12000, seed=41), S.powerlaw_csr(3000, 2.0, 9.0, seed=42)]
    for a, N_ in zip(cases, (4096, 64)):
        B = S.dense_uniform((a.n_cols, N_), 43)
        rp, ci, v = csr_dev(a)
        if dtype == torch.float32:
            ref = oracle.spmm_fma_chain_f32(a.rowptr, a.colind, a.val, B)
        else:
            ref = oracle.spmm_fma_chain_f32(a.rowptr, a.colind, oracle.bf16_round(a.val),
                                            oracle.bf16_round(B))
        vd, Bd = v.to(dtype), to_dev(B).to(dtype)
        ran = 0
        for var in _variant_ids("bulk", dtype):
            try:
                C = A.spmm(rp, ci, vd, Bd, variant=var)
            except N.NativeError as e:
                assert e.status == 3
                continue
            ran += 1
            assert np.array_equal(bits(C), bits(ref)), A.spmm_variants(dtype)[var - 1]
            C0 = torch.ones_like(C)
            A.spmm(rp, ci, vd, Bd, C=C0, beta=1.0, variant=var)
            ref1 = oracle.spmm_fma_chain_f32(a.rowptr, a.colind, oracle.bf16_round(a.val) if dtype != torch.float32 else a.val,
                                             oracle.bf16_round(B) if dtype != torch.float32 else B,
                                             C=np.ones(ref.shape, np.float32))
            assert np.array_equal(bits(C0), bits(ref1))
        assert ran >= 2
    A.sync_status()


def test_nnzsplit_variants_skewed_rows(oracle):
    # one row with 50,000 entries among short rows, plus empty rows
    rng = np.random.default_rng(44)
    lens = rng.integers(0, 6, 4000)
    lens[1234] = 50000
    lens[:10] = 0
    rp = np.zeros(4001, np.int32)
    np.cumsum(lens, out=rp[1:])
    ci = np.concatenate([np.sort(rng.choice(60000, l, replace=False)) for l in lens]).astype(np.int32)
    a = S.CSR(rp, ci, rng.uniform(-1, 1, ci.size).astype(np.float32), 4000, 60000)
    for N_ in (64, 256):
        B = S.dense_uniform((60000, N_), 45)
        C64, A64 = oracle.spmm_f64(a.rowptr, a.colind, a.val, B)
        chain = oracle.spmm_fma_chain_f32(a.rowptr, a.colind, a.val, B)
        rpd, cid, vd = csr_dev(a)
        Bd = to_dev(B)
        whole = np.diff(a.rowptr) <= 128  # rows that fit in one chunk of the smallest size
        for var in _variant_ids("nnzsplit"):
            if not A.spmm_variant_supported(var, N_):
                continue  # the 32-entry-chunk kernels serve N <= 64 only
            C = A.spmm(rpd, cid, vd, Bd, variant=var)
            got = C.cpu().numpy()
            assert oracle.scaled_err(got, C64, A64).max() < 1e-5
            C2 = A.spmm(rpd, cid, vd, Bd, variant=var)
            assert torch.equal(C, C2)  # deterministic
            # short rows are usually inside one chunk: those are bit-identical to the chain
            same = (got.view(np.uint32) == chain.view(np.uint32)).all(axis=1)
            assert same[whole].mean() > 0.9
            assert (got[:10] == 0).all()
            Cb = torch.full_like(C, 2.0)
            A.spmm(rpd, cid, vd, Bd, C=Cb, beta=0.5, variant=var)
            assert oracle.scaled_err(Cb.cpu().numpy(), C64 + 1.0, A64 + 1.0).max() < 1e-5
    A.sync_status()


@pytest.mark.parametrize("op", ["sum", "max"])
def test_reduce_aggregations(oracle, op):
    """Unweighted copy-sum / copy-max and the weighted forms, bit-exact against the CSR-order
    restatement (sum adds in order without fusing, as the reference's topo kernels do)."""
    a = S.powerlaw_csr(3000, 2.0, 9.0, seed=51, n_cols=2500)
    for N_ in (1, 47, 64, 300):
        B = S.dense_uniform((2500, N_), 52)
        rp, ci, v = csr_dev(a)
        for val in (None, a.val):
            got = A.spmm_reduce(rp, ci, to_dev(B), val=None if val is None else v, op=op)
            ref = oracle.spmm_reduce_f32(a.rowptr, a.colind, B, val=val, op=op)
            assert np.array_equal(bits(got), bits(ref)), (op, N_, val is None)
    A.sync_status()


def test_reduce_long_rows(oracle):
    """Rows past 256 entries (one past 16,384) go to the long-row kernel with the reduction as
    its chain step: sum, weighted sum, max and the DGL max stay bit-exact against the CSR-order
    restatement, for 16-byte (N = 64, 300) and 4-byte (N = 47) copies."""
    a = _skewed(41)
    rp, ci, v = csr_dev(a)
    for N_ in (47, 64, 300):
        B = S.dense_uniform((a.n_cols, N_), 42 + N_) * 30000.0 - 15000.0  # some below -10000
        B = B.astype(np.float32)
        Bd = to_dev(B)
        for op in ("sum", "max", "max_dgl"):
            for val in (None, a.val):
                got = A.spmm_reduce(rp, ci, Bd, val=None if val is None else v, op=op)
                ref = oracle.spmm_reduce_f32(a.rowptr, a.colind, B, val=val, op=op)
                assert np.array_equal(bits(got), bits(ref)), (op, N_, val is None)
    A.sync_status()


def test_reduce_max_dgl(oracle):
    """The reference's DGL copy-max (binary_reduce_max.cu: start at -10000, acc > x ? acc : x):
    empty rows give -10000, values below -10000 never show unless they follow a NaN entry (which
    the entry after it replaces). Bit-exact against the oracle: NaN payloads included where
    values pass through unchanged; where a NaN comes from a product, the same positions are NaN
    (the payload of a NaN product differs between the GPU and the host)."""
    a = S.powerlaw_csr(2000, 2.0, 7.0, seed=61, n_cols=1500)
    rng = np.random.default_rng(62)
    for N_ in (1, 31, 64, 130):
        B = S.dense_uniform((1500, N_), 63) * 30000.0 - 15000.0  # about half below -10000
        B[rng.integers(0, 1500, 40), rng.integers(0, N_, 40)] = np.nan
        B = B.astype(np.float32)
        rp, ci, v = csr_dev(a)
        for val in (None, a.val):
            got = A.spmm_reduce(rp, ci, to_dev(B), val=None if val is None else v, op="max_dgl")
            ref = oracle.spmm_reduce_f32(a.rowptr, a.colind, B, val=val, op="max_dgl")
            g, r = got.cpu().numpy(), ref
            if val is None:  # values pass through unchanged: bit for bit, NaN payloads included
                assert np.array_equal(bits(got), bits(ref)), (N_, val is None)
            else:  # a product with a NaN: the GPU's NaN is canonical, the host keeps the operand's
                assert np.array_equal(np.isnan(g), np.isnan(r)), N_
                ok = ~np.isnan(r)
                assert np.array_equal(g[ok].view(np.uint32), r[ok].view(np.uint32)), N_
            empty = np.diff(a.rowptr) == 0
            assert empty.any() and (got.cpu().numpy()[empty] == -10000.0).all()
            # rows that gather no NaN never fall below -10000 (after a NaN entry, the next
            # entry replaces it whatever its value)
            rows = np.repeat(np.arange(a.n_rows), np.diff(a.rowptr))
            has_nan = np.zeros(a.n_rows, bool)
            np.logical_or.at(has_nan, rows, np.isnan(B[a.colind]).any(axis=1))
            assert (got.cpu().numpy()[~has_nan] >= -10000.0).all()
            assert has_nan.any()
    A.sync_status()


def _skewed(seed, n_rows=3000, n_cols=40000, long_lens=(50000, 4097, 2048, 257, 256, 300)):
    """Short rows plus rows at and past the long-row threshold (256 entries): one long enough
    to cross many (colind, val) chunks of 2048 entries."""
    rng = np.random.default_rng(seed)
    lens = rng.integers(0, 40, n_rows)
    for i, l in enumerate(long_lens):
        lens[7 + 211 * i] = min(l, n_cols)
    lens[:5] = 0
    rp = np.zeros(n_rows + 1, np.int32)
    np.cumsum(lens, out=rp[1:])
    ci = np.concatenate([np.sort(rng.choice(n_cols, l, replace=False)) for l in lens]).astype(np.int32)
    return S.CSR(rp, ci, rng.uniform(-1, 1, ci.size).astype(np.float32), n_rows, n_cols)


@pytest.mark.parametrize("N_", [47, 64, 256, 300])
def test_long_rows_row_split_bit_exact(oracle, N_):
    """Rows longer than 256 entries go to the long-row kernel; every row-split variant stays
    bit-identical to the reference's chain, for 16-byte and 4-byte copy layouts (N = 47 and 300
    give 4-byte copies), with beta = 1 accumulation, and call after call."""
    a = _skewed(7 + N_)
    B = S.dense_uniform((a.n_cols, N_), 8)
    ref = oracle.spmm_fma_chain_f32(a.rowptr, a.colind, a.val, B)
    ref2 = oracle.spmm_fma_chain_f32(a.rowptr, a.colind, a.val, B, C=ref)
    rp, ci, v = csr_dev(a)
    Bd = to_dev(B)
    names = A.spmm_variants()
    for var in [0] + _variant_ids("rowsplit"):
        try:
            C = A.spmm(rp, ci, v, Bd, variant=var)
        except N.NativeError as e:
            assert e.status == 3
            continue
        assert np.array_equal(bits(C), bits(ref)), names[var - 1] if var else "default"
        A.spmm(rp, ci, v, Bd, C=C, beta=1.0, variant=var)
        assert np.array_equal(bits(C), bits(ref2)), names[var - 1] if var else "default"
    A.sync_status()


def test_huge_rows_first_bit_exact(oracle):
    """Rows past 16,384 entries are listed from the end of the long-row list and taken first,
    among many rows just past the long-row threshold: bit-identical for fp32 and bf16 storage,
    two 64-column slices per row, and the list counters start from zero on the next call."""
    rng = np.random.default_rng(11)
    n_rows, n_cols = 400, 60000
    lens = rng.integers(200, 320, n_rows)
    lens[[3, 50, 51, 399]] = [60000, 16385, 20000, 33333]
    rp_h = np.zeros(n_rows + 1, np.int32)
    np.cumsum(lens, out=rp_h[1:])
    ci_h = np.concatenate([np.sort(rng.choice(n_cols, l, replace=False)) for l in lens]).astype(np.int32)
    a = S.CSR(rp_h, ci_h, rng.uniform(-1, 1, ci_h.size).astype(np.float32), n_rows, n_cols)
    B = S.dense_uniform((n_cols, 128), 12)
    ref = oracle.spmm_fma_chain_f32(a.rowptr, a.colind, a.val, B)
    rp, ci, v = csr_dev(a)
    Bd = to_dev(B)
    for _ in range(2):
        C = A.spmm(rp, ci, v, Bd)
        assert np.array_equal(bits(C), bits(ref))
    vb, Bb = oracle.bf16_round(a.val), oracle.bf16_round(B)
    refb = oracle.spmm_fma_chain_f32(a.rowptr, a.colind, vb, Bb)
    C = A.spmm(rp, ci, v.to(torch.bfloat16), Bd.to(torch.bfloat16))
    assert np.array_equal(bits(C), bits(refb))
    A.sync_status()


def test_long_rows_strided_and_bf16(oracle):
    a = _skewed(99)
    rp, ci, v = csr_dev(a)
    # B and C inside wider buffers (ldb = 72, ldc = 80)
    Bw = S.dense_uniform((a.n_cols, 72), 3)
    ref = oracle.spmm_fma_chain_f32(a.rowptr, a.colind, a.val, np.ascontiguousarray(Bw[:, :64]))
    Cw = torch.zeros((a.n_rows, 80), device=dev())
    A.spmm(rp, ci, v, to_dev(Bw)[:, :64], C=Cw[:, 8:72])
    assert np.array_equal(bits(Cw[:, 8:72].contiguous()), bits(ref))
    assert torch.count_nonzero(Cw[:, :8]) == 0 and torch.count_nonzero(Cw[:, 72:]) == 0
    # bf16 storage: the same chain over the bf16-rounded inputs
    names = A.spmm_variants(torch.bfloat16)
    for N_ in (64, 256, 46, 47):
        B = S.dense_uniform((a.n_cols, N_), N_)
        vb, Bb = oracle.bf16_round(a.val), oracle.bf16_round(B)
        refb = oracle.spmm_fma_chain_f32(a.rowptr, a.colind, vb, Bb)
        vd, Bd = v.to(torch.bfloat16), to_dev(B).to(torch.bfloat16)
        for var in [0] + (_variant_ids("rowsplit", torch.bfloat16) if N_ == 64 else []):
            try:
                C = A.spmm(rp, ci, vd, Bd, variant=var)
            except N.NativeError as e:
                assert e.status == 3
                continue
            assert np.array_equal(bits(C), bits(refb)), (N_, names[var - 1] if var else "default")
    A.sync_status()


def test_nnzsplit_bf16_variants(oracle):
    """bf16 storage through the entry-balanced kernels (4- and 8-entry load batches): fp32
    accumulation error only, against FP64 of the bf16-rounded inputs; deterministic."""
    a = _skewed(5, n_rows=2000, n_cols=30000, long_lens=(30000, 3000, 700))
    rp, ci, v = csr_dev(a)
    vb = oracle.bf16_round(a.val)
    names = A.spmm_variants(torch.bfloat16)
    for N_ in (64, 46):
        B = S.dense_uniform((a.n_cols, N_), 6 + N_)
        Bb = oracle.bf16_round(B)
        R, Ab = oracle.spmm_f64(a.rowptr, a.colind, vb, Bb)
        vd, Bd = v.to(torch.bfloat16), to_dev(B).to(torch.bfloat16)
        ran = 0
        for var in _variant_ids("nnzsplit", torch.bfloat16):
            try:
                C = A.spmm(rp, ci, vd, Bd, variant=var)
            except N.NativeError as e:
                assert e.status == 3
                continue
            ran += 1
            assert oracle.scaled_err(C.cpu().numpy(), R, Ab).max() < 1e-5, names[var - 1]
            assert torch.equal(C, A.spmm(rp, ci, vd, Bd, variant=var)), names[var - 1]
        assert ran >= 4
    A.sync_status()


@pytest.mark.parametrize("N_", [46, 64, 256])
def test_bf16_output_is_rounded_fp32_output(N_):
    """C in bf16 (as_spmm_csr_bf16_out16) is the same variant's fp32 C rounded to nearest even,
    bit for bit, through the row-split, long-row and entry-balanced kernels (and with the ReLU
    epilogue, relu of it); the bulk-copy variants have no bf16 output."""
    a = _skewed(9, n_rows=2500, n_cols=20000, long_lens=(20000, 3000, 600, 257))
    rp, ci, v = csr_dev(a)
    vd = v.to(torch.bfloat16)
    Bd = to_dev(S.dense_uniform((a.n_cols, N_), 10 + N_)).to(torch.bfloat16)
    names = A.spmm_variants(torch.bfloat16)
    ran = 0
    for var in range(1, len(names) + 1):
        try:
            C32 = A.spmm(rp, ci, vd, Bd, variant=var)
        except N.NativeError as e:
            assert e.status == 3
            continue
        try:
            C16 = A.spmm(rp, ci, vd, Bd, variant=var, out_dtype=torch.bfloat16)
        except N.NativeError as e:
            assert e.status == 3 and names[var - 1].startswith("bulk"), names[var - 1]
            continue
        ran += 1
        assert C16.dtype == torch.bfloat16
        assert torch.equal(C16.view(torch.int16), C32.to(torch.bfloat16).view(torch.int16)), \
            names[var - 1]
        R16 = A.spmm(rp, ci, vd, Bd, variant=var, out_dtype=torch.bfloat16, relu=True)
        assert torch.equal(R16, torch.relu(C16)), names[var - 1]  # the ReLU epilogue
    assert ran >= 20
    C0 = A.spmm(rp, ci, vd, Bd, out_dtype=torch.bfloat16)  # library choice
    assert torch.equal(C0.view(torch.int16), A.spmm(rp, ci, vd, Bd).to(torch.bfloat16).view(torch.int16))
    with pytest.raises(ValueError):
        A.spmm(rp, ci, vd, Bd, C=torch.empty_like(C0), beta=1.0, out_dtype=torch.bfloat16)
    A.sync_status()


@pytest.mark.parametrize("dtype", [torch.float32, torch.bfloat16])
@pytest.mark.parametrize("N_", [16, 48, 64, 128])
def test_multi_entry_variants(oracle, dtype, N_):
    """The multi-entry kernels (a warp per chunk, 32 / group sub-groups each taking every
    sub-group-th entry): fp32 accumulation error only, deterministic, beta and the bf16
    output as the others, rows that span many chunks included."""
    a = _skewed(30 + N_, n_rows=2500, n_cols=20000, long_lens=(20000, 3000, 600, 257))
    rp, ci, v = csr_dev(a)
    B = S.dense_uniform((a.n_cols, N_), 31 + N_)
    if dtype == torch.bfloat16:
        vh, Bh = oracle.bf16_round(a.val), oracle.bf16_round(B)
    else:
        vh, Bh = a.val, B
    R, Ab = oracle.spmm_f64(a.rowptr, a.colind, vh, Bh)
    vd, Bd = to_dev(vh).to(dtype), to_dev(Bh).to(dtype)
    ran = 0
    for var in _variant_ids("nnzme", dtype):
        if not A.spmm_variant_supported(var, N_, dtype):
            continue
        ran += 1
        C = A.spmm(rp, ci, vd, Bd, variant=var)
        assert oracle.scaled_err(C.cpu().numpy(), R, Ab).max() < 1e-5
        assert torch.equal(C, A.spmm(rp, ci, vd, Bd, variant=var))
        Cb = torch.full_like(C, 2.0)
        A.spmm(rp, ci, vd, Bd, C=Cb, beta=0.5, variant=var)
        assert oracle.scaled_err(Cb.cpu().numpy(), R + 1.0, Ab + 1.0).max() < 1e-5
        assert (C[:5] == 0).all()  # empty rows
        if dtype == torch.bfloat16:
            C16 = A.spmm(rp, ci, vd, Bd, variant=var, out_dtype=torch.bfloat16)
            assert torch.equal(C16.view(torch.int16), C.to(torch.bfloat16).view(torch.int16))
    assert ran >= 3
    A.sync_status()
