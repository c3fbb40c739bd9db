"""The CPU oracle against the reference: golden vectors made from the reference's own
kernels (always), and the reference compiled here from its sources (when present)."""
import ctypes

import numpy as np
import pytest

from armsparse_gb300 import synthetic as S


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def test_spmm_chain_matches_rowbasespmm3_golden(oracle, golden):
    g = golden["spmm_rowbasespmm3"]
    for i in range(int(g["n_cases"])):
        M, K, N = g[f"c{i}_shape"]
        rp, ci, v, B = g[f"c{i}_rowptr"], g[f"c{i}_colind"], g[f"c{i}_val"], g[f"c{i}_B"]
        C = oracle.spmm_fma_chain_f32(rp, ci, v, B, threads=2)
        assert np.array_equal(C.view(np.uint32), g[f"c{i}_C"].view(np.uint32)), i
        C2 = oracle.spmm_fma_chain_f32(rp, ci, v, B, C=C, threads=2)
        assert np.array_equal(C2.view(np.uint32), g[f"c{i}_C_twice"].view(np.uint32)), i
        # rowBaseSpmm2 (SDMM.cpp:65-89): one fused saxpy step per entry and column, in CSR
        # order -- the same chain
        assert np.array_equal(C.view(np.uint32), g[f"c{i}_C_saxpy"].view(np.uint32)), i
        # origin() (SDMM.cpp:422-448): same terms, its own compiled summation; agrees to
        # FP32 rounding
        C64, A64 = oracle.spmm_f64(rp, ci, v, B, threads=1)
        assert oracle.scaled_err(g[f"c{i}_C_origin"], C64, A64).max() < 1e-5


def test_spmm_f64_close_to_golden(oracle, golden):
    g = golden["spmm_rowbasespmm3"]
    for i in range(int(g["n_cases"])):
        rp, ci, v, B = g[f"c{i}_rowptr"], g[f"c{i}_colind"], g[f"c{i}_val"], g[f"c{i}_B"]
        C64, A64 = oracle.spmm_f64(rp, ci, v, B, threads=1)
        assert oracle.scaled_err(g[f"c{i}_C"], C64, A64).max() < 1e-5


def test_vcsr4_layout_and_spmv_golden(oracle, golden):
    g = golden["spmv_vcsr4"]
    for i in range(int(g["n_cases"])):
        vr, vc, vv = oracle.csr_to_vcsr4(g[f"c{i}_rowptr"], g[f"c{i}_colind"], g[f"c{i}_val"])
        assert np.array_equal(vr, g[f"c{i}_vrowptr"])
        assert np.array_equal(vc, g[f"c{i}_vcolind"])
        assert np.array_equal(vv.view(np.uint32), g[f"c{i}_vval"].view(np.uint32))
        y = oracle.spmv_vcsr4_f32(vr, vc, vv, g[f"c{i}_x"], fused=True, threads=1)
        # the reference build here fuses vmlaq_f32 (-ffp-contract=fast with FMA available)
        assert np.array_equal(y.view(np.uint32), g[f"c{i}_y"].view(np.uint32)), i


def test_csr2csc_matches_fast_transpose_golden(oracle, golden):
    g = golden["transpose_triplets"]
    for i in range(int(g["n_cases"])):
        dense = g[f"c{i}_dense"]
        M, N = dense.shape
        trip = g[f"c{i}_triplets"].reshape(-1, 3)
        nnz = trip[0, 2]
        rows, cols, vals = trip[1:nnz + 1, 0], trip[1:nnz + 1, 1], trip[1:nnz + 1, 2]
        rp = np.zeros(M + 1, np.int32)
        np.cumsum(np.bincount(rows, minlength=M), out=rp[1:])
        cp, ri, cv = oracle.csr2csc(rp, cols, vals.astype(np.float32), N)
        res = g[f"c{i}_transposed"].reshape(-1, 3)
        assert res[0].tolist() == [N, M, nnz]
        # transposed triplets: (col, row, value) in column-major order
        assert np.array_equal(res[1:nnz + 1, 0], np.repeat(np.arange(N), np.diff(cp)))
        assert np.array_equal(res[1:nnz + 1, 1], ri)
        assert np.array_equal(res[1:nnz + 1, 2], cv.astype(np.int32))


def test_csr2csc_matches_scipy(oracle):
    sp = pytest.importorskip("scipy.sparse")
    a = S.powerlaw_csr(500, 2.0, 6.0, seed=3, n_cols=300)
    cp, ri, cv = oracle.csr2csc(a.rowptr, a.colind, a.val, a.n_cols)
    m = sp.csr_matrix((a.val, a.colind, a.rowptr), shape=a.shape).tocsc()
    assert np.array_equal(cp, m.indptr) and np.array_equal(ri, m.indices)
    assert np.array_equal(cv.view(np.uint32), m.data.astype(np.float32).view(np.uint32))


@pytest.mark.parametrize("M,K,N,nnz,seed", [(300, 200, 64, 3000, 0), (100, 80, 7, 900, 1),
                                             (33, 40, 3, 200, 2), (128, 128, 130, 2000, 3)])
def test_spmm_chain_against_compiled_reference(oracle, M, K, N, nnz, seed):
    ref = oracle.ref_lib("sdmm")
    if ref is None:
        pytest.skip("reference sources not compiled here")
    a = S.uniform_csr(M, K, nnz, seed, values="ref_int")
    B = S.dense_uniform((K, N), seed + 10)
    mine = oracle.spmm_fma_chain_f32(a.rowptr, a.colind, a.val, B, threads=2)
    C = np.zeros((M, N), np.float32)
    rp, ci, v, Bc = a.rowptr.copy(), a.colind.copy(), a.val.copy(), B.copy()
    ref.ref_rowBaseSpmm3(_p(rp), _p(ci), _p(v), _p(Bc), _p(C), M, K, N, 2)
    assert np.array_equal(mine.view(np.uint32), C.view(np.uint32))


def test_spmv_against_compiled_reference(oracle):
    ref = oracle.ref_lib("spmv")
    if ref is None:
        pytest.skip("reference sources not compiled here")
    a = S.uniform_csr(200, 256, 3000, 5)
    vr, vc, vv = oracle.csr_to_vcsr4(a.rowptr, a.colind, a.val)
    x = S.dense_uniform(256, 6)
    y = np.zeros(200, np.float32)
    ref.ref_sparse_dense_vector(_p(x.copy()), _p(y), _p(vr.copy()), _p(vc.copy()),
                                _p(vv.copy()), 200, 2)
    mine = oracle.spmv_vcsr4_f32(vr, vc, vv, x, fused=True, threads=2)
    assert np.array_equal(mine.view(np.uint32), y.view(np.uint32))


def test_sddmm_oracles_agree(oracle):
    a = S.uniform_csr(64, 48, 600, 7, values="u0515")
    X = S.dense_normal((64, 40), 8)
    Y = S.dense_normal((48, 40), 9)
    o64, ab = oracle.sddmm_f64(a.rowptr, a.colind, X, Y, aval=a.val)
    o32 = oracle.sddmm_f32_lanes(a.rowptr, a.colind, X, Y, aval=a.val)
    assert oracle.scaled_err(o32, o64, ab).max() < 1e-5
    for K in (40, 3, 130, 600):  # the GPU kernel's order: group sizes 4, 1, 16 and 32 lanes
        Xk, Yk = S.dense_normal((64, K), 10 + K), S.dense_normal((48, K), 20 + K)
        r64, rab = oracle.sddmm_f64(a.rowptr, a.colind, Xk, Yk, aval=a.val)
        og = oracle.sddmm_f32_group(a.rowptr, a.colind, Xk, Yk, aval=a.val)
        assert oracle.scaled_err(og, r64, rab).max() < 1e-5
    # against a dense formula
    rows = np.repeat(np.arange(64), np.diff(a.rowptr))
    dense = (X.astype(np.float64) @ Y.astype(np.float64).T)[rows, a.colind] * a.val
    assert np.allclose(o64, dense, rtol=1e-12, atol=1e-12)


def test_sddmm_slices_order(oracle):
    """The fused pass's dot-product order (lane slices, then a butterfly): within FP32 error of
    FP64, deterministic, placed through a permutation, and equal to a plain loop restatement."""
    a = S.uniform_csr(60, 50, 500, 17)
    for G, E, CPL, K in ((32, 2, 1, 48), (8, 8, 1, 48), (16, 4, 2, 100), (32, 8, 1, 256)):
        X, Y = S.dense_normal((60, K), K), S.dense_normal((50, K), K + 1)
        r64, ab = oracle.sddmm_f64(a.rowptr, a.colind, X, Y)
        got = oracle.sddmm_f32_slices(a.rowptr, a.colind, X, Y, G, E, CPL)
        assert oracle.scaled_err(got, r64, ab).max() < 1e-5
        perm = np.random.default_rng(K).permutation(got.size).astype(np.int32)
        placed = oracle.sddmm_f32_slices(a.rowptr, a.colind, X, Y, G, E, CPL, perm=perm)
        assert np.array_equal(placed[perm].view(np.uint32), got.view(np.uint32))
    # a plain restatement for one shape (fmaf = a product exact in double, then one rounding)
    G, E, CPL, K = 8, 4, 2, 40
    X, Y = S.dense_normal((60, K), 3), S.dense_normal((50, K), 4)
    got = oracle.sddmm_f32_slices(a.rowptr, a.colind, X, Y, G, E, CPL)
    rows = np.repeat(np.arange(60), np.diff(a.rowptr))
    for e in range(0, a.colind.size, 37):
        x, y = X[rows[e]], Y[a.colind[e]]
        lanes = []
        for l in range(G):
            acc = np.float32(0)
            for j in range(CPL):
                c = (j * G + l) * E
                for i in range(E):
                    if c + i < K:
                        acc = np.float32(np.float64(y[c + i]) * np.float64(x[c + i]) + np.float64(acc))
            lanes.append(acc)
        off = G // 2
        while off:
            lanes = [np.float32(lanes[l] + lanes[l ^ off]) for l in range(G)]
            off //= 2
        assert lanes[0] == got[e]


def test_entry_balanced_order(oracle):
    """The entry-balanced kernels' order: one sub-chain is the plain chain for rows inside a
    chunk, every form stays within FP32 error of FP64 (short and long spans, beta), and
    sub-chains of 2 and 4 reorder only within a segment."""
    rng = np.random.default_rng(5)
    lens = rng.integers(0, 12, 900)
    lens[10], lens[400], lens[401] = 5000, 700, 129  # spans > 8 chunks, 2-8 chunks, a boundary
    rp = np.zeros(901, np.int32)
    np.cumsum(lens, out=rp[1:])
    ci = np.concatenate([np.sort(rng.choice(6000, l, replace=False)) for l in lens]).astype(np.int32)
    val = rng.uniform(-1, 1, ci.size).astype(np.float32)
    for N_ in (8, 6, 40):
        B = S.dense_uniform((6000, N_), N_)
        chain = oracle.spmm_fma_chain_f32(rp, ci, val, B)
        r64, ab = oracle.spmm_f64(rp, ci, val, B)
        for ch in (128, 1024):
            c_first, c_last = rp[:-1] // ch, np.maximum(rp[1:] - 1, rp[:-1]) // ch
            inside = c_first == c_last
            for sub in (1, 2, 4):
                got = oracle.spmm_nnz_order_f32(rp, ci, val, B, ch, sub)
                assert oracle.scaled_err(got, r64, ab).max() < 1e-5
                if sub == 1:
                    assert np.array_equal(got[inside].view(np.uint32),
                                          chain[inside].view(np.uint32))
            C0 = S.dense_uniform((900, N_), 7)
            got = oracle.spmm_nnz_order_f32(rp, ci, val, B, ch, 1, C=C0, beta=0.5)
            assert oracle.scaled_err(got, r64 + 0.5 * C0, ab + 0.5 * np.abs(C0)).max() < 1e-5


def test_scaled_err_metric(oracle):
    ref = np.array([1.0, 0.0, -2.0])
    ab = np.array([1.0, 4.0, 2.0])
    e = oracle.scaled_err(ref + np.array([1e-6, 1e-6, 0.0]), ref, ab)
    assert e[0] == pytest.approx(1e-6) and e[1] == pytest.approx(2.5e-7) and e[2] == 0.0


def test_rel_err_metric(oracle):
    ref = np.array([1.0, 0.0, 1e-9, -2.0])
    ab = np.array([1.0, 1.0, 1.0, 2.0])
    got = ref + np.array([1e-6, 1e-7, 1e-7, 0.0])
    e = oracle.rel_err(got, ref, ab)
    assert e[0] == pytest.approx(1e-6)
    assert e[1] == pytest.approx(1e-7 / 2 ** -20)
    assert e[3] == 0.0


def test_bf16_round(oracle):
    x = np.array([1.0, 1.00390625, 1.005859375, -3.3, 65504.0], np.float32)
    r = oracle.bf16_round(x)
    # 1 + 2^-8 is a tie -> even (1.0); 1 + 1.5*2^-8 rounds up to 1 + 2^-7
    assert r[0] == 1.0 and r[1] == 1.0 and r[2] == np.float32(1.0078125)
    assert (r.view(np.uint32) & 0xFFFF).max() == 0


def test_spgemm_dense_matches_sparse_matrix_mul3_golden(oracle, golden):
    """The sparse x sparse -> dense restatement against the reference's sparse_matrix_mul3
    (SpMM.cpp:309-327) run here: bit-identical, also for the driver's accumulate pattern."""
    g = golden["spgemm_dense"]
    for i in range(int(g["n_cases"])):
        M, K, N = g[f"c{i}_shape"]
        args = [g[f"c{i}_{x}"] for x in ("a_rowptr", "a_colind", "a_val", "b_rowptr",
                                         "b_colind", "b_val")]
        C = oracle.spgemm_dense_f32(*args, int(N), threads=2)
        assert np.array_equal(C.view(np.uint32), g[f"c{i}_C"].view(np.uint32)), i
        C2 = oracle.spgemm_dense_f32(*args, int(N), C=C, threads=2)
        assert np.array_equal(C2.view(np.uint32), g[f"c{i}_C_twice"].view(np.uint32)), i
        R, Ab = oracle.spgemm_dense_f64(*args, int(N))
        assert oracle.scaled_err(C, R, Ab).max() < 1e-5


def test_spgemm_dense_against_compiled_reference(oracle):
    ref = oracle.ref_lib("spgemm")
    if ref is None:
        pytest.skip("reference sources not compiled here")
    a = S.uniform_csr(120, 90, 1500, 3)
    b = S.uniform_csr(90, 70, 1200, 4)
    mine = oracle.spgemm_dense_f32(a.rowptr, a.colind, a.val, b.rowptr, b.colind, b.val, 70,
                                   threads=2)
    C = np.zeros((120, 70), np.float32)
    arrs = [x.copy() for x in (a.rowptr, a.colind, a.val, b.rowptr, b.colind, b.val)]
    ref.ref_sparse_matrix_mul3(*[_p(x) for x in arrs], _p(C), 120, 90, 70, 2)
    assert np.array_equal(mine.view(np.uint32), C.view(np.uint32))


def _dgl_copy_max(rowptr, colind, B):
    """The reference's copy-max kernel read line by line (gcn/dgl-custom/binary_reduce_max.cu):
    acc1 = max_init() = -10000 (:22-24, :158); for ptr in [lb, hb): acc1 = max_reduce(acc1,
    B[A_indices[ptr]*k + col]) with max_reduce(acc, x) = acc > x ? acc : x (:18-20, :160-165);
    C = acc1 (:166). Pure Python over float32 scalars, for small cases."""
    M, N = rowptr.size - 1, B.shape[1]
    C = np.empty((M, N), np.float32)
    for r in range(M):
        for j in range(N):
            acc = np.float32(-10000)
            for p in range(rowptr[r], rowptr[r + 1]):
                x = B[colind[p], j]
                acc = acc if acc > x else x
            C[r, j] = acc
    return C


def test_reduce_max_dgl_restates_reference_loop(oracle):
    a = S.powerlaw_csr(300, 2.0, 5.0, seed=71, n_cols=200)
    rng = np.random.default_rng(72)
    B = (rng.uniform(-30000, 20000, (200, 5))).astype(np.float32)
    B[rng.integers(0, 200, 12), rng.integers(0, 5, 12)] = np.nan
    got = oracle.spmm_reduce_f32(a.rowptr, a.colind, B, op="max_dgl")
    ref = _dgl_copy_max(a.rowptr, a.colind, B)
    assert np.array_equal(got.view(np.uint32), ref.view(np.uint32))
    assert (np.diff(a.rowptr) == 0).any()


def test_rowpair_layout_and_spmm_match_reference_golden(oracle, golden):
    """The oracle's row-pair layout (built from CSR) and its DataReuseSpmm order against what
    the reference's own toDataReuseFormat / DataReuseSpmm (suitesparse_sdmm.cpp) produced from
    the dense matrices -- bit for bit."""
    g = golden["rowpair_reuse"]
    for i in range(int(g["n_cases"])):
        rp2, ci2, v2, f2 = oracle.csr_to_rowpair(g[f"c{i}_rowptr"], g[f"c{i}_colind"],
                                                 g[f"c{i}_val"])
        assert np.array_equal(rp2, g[f"c{i}_rowptr2"]), i
        assert np.array_equal(ci2, g[f"c{i}_colind2"]), i
        assert np.array_equal(v2.view(np.uint32), g[f"c{i}_val2"].view(np.uint32)), i
        assert np.array_equal(f2, g[f"c{i}_flag2"]), i
        assert f2.any()  # the cases do share columns within pairs
        C = oracle.spmm_rowpair_f32(rp2, ci2, v2, f2, g[f"c{i}_B"], threads=3)
        assert np.array_equal(C.view(np.uint32), g[f"c{i}_C"].view(np.uint32)), i
        # even rows keep the CSR chain; odd rows that share a column generally do not
        chain = oracle.spmm_fma_chain_f32(g[f"c{i}_rowptr"], g[f"c{i}_colind"], g[f"c{i}_val"],
                                          g[f"c{i}_B"])
        assert np.array_equal(C[0::2].view(np.uint32), chain[0::2].view(np.uint32)), i
