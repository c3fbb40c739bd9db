"""Matrix Market reading on the host (files written by the test)."""
import numpy as np
import pytest

from armsparse_gb300.mtx import read_mtx


def _write(path, text):
    path.write_text(text)
    return str(path)


def test_general_real_with_duplicates(tmp_path):
    p = _write(tmp_path / "a.mtx", "%%MatrixMarket matrix coordinate real general\n"
               "% comment\n3 4 5\n1 2 1.5\n3 4 -2\n1 2 0.5\n2 1 3\n1 1 4\n")
    a = read_mtx(p, duplicates="sum")
    assert a.shape == (3, 4)
    assert a.rowptr.tolist() == [0, 2, 3, 4]
    assert a.colind.tolist() == [0, 1, 0, 3]
    assert a.val.tolist() == [4.0, 2.0, 3.0, -2.0]


def test_symmetric_pattern_expands_both_triangles(tmp_path):
    p = _write(tmp_path / "s.mtx", "%%MatrixMarket matrix coordinate pattern symmetric\n"
               "3 3 3\n1 1\n2 1\n3 2\n")
    a = read_mtx(p, duplicates="sum")
    dense = np.zeros((3, 3))
    dense[np.repeat(np.arange(3), np.diff(a.rowptr)), a.colind] = a.val
    assert (dense == dense.T).all() and dense.sum() == 5.0 and dense[0, 0] == 1.0
    b = read_mtx(p)  # the reference's reading drops the self-loop
    assert b.nnz == 4 and b.colind.tolist() == [1, 0, 2, 1]


def test_rejects_bad_files(tmp_path):
    with pytest.raises(ValueError):
        read_mtx(_write(tmp_path / "b.mtx", "%%MatrixMarket matrix array real general\n2 2\n1\n2\n3\n4\n"))
    with pytest.raises(ValueError):
        read_mtx(_write(tmp_path / "c.mtx", "%%MatrixMarket matrix coordinate real general\n2 2 1\n3 1 1.0\n"))


def _golden_cases():
    import os
    path = os.path.join(os.path.dirname(__file__), "golden", "mtx_reader.npz")
    g = np.load(path)
    return [(str(g[f"c{i}_name"]), str(g[f"c{i}_text"]), g[f"c{i}_shape"], g[f"c{i}_rows"],
             g[f"c{i}_cols"], g[f"c{i}_vals"]) for i in range(int(g["n_cases"]))]


def _same_up_to_ties(r, c, v, ref_v):
    """Values equal bit for bit, except that within a run of equal (row, column) entries --
    whose order the reference's std::sort leaves unspecified -- they may come in any order."""
    if v.size != ref_v.size:
        return False
    a, b = v.view(np.uint32), ref_v.view(np.uint32)
    start = np.flatnonzero(np.r_[True, (r[1:] != r[:-1]) | (c[1:] != c[:-1]), True])
    return all(np.array_equal(np.sort(a[i:j]), np.sort(b[i:j])) for i, j in zip(start[:-1], start[1:]))


@pytest.mark.parametrize("case", _golden_cases(), ids=lambda c: c[0])
def test_reference_reading_matches_readmtx_golden(tmp_path, case):
    """The default reading equals what the reference's readMtx<float> (gcn/util/util.hpp:
    286-333) left in its vectors for the same file: self-loops and duplicates of symmetric
    files dropped (values misaligned as its compaction leaves them), general files' duplicates
    kept, only `symmetric` expanded -- bit for bit."""
    from armsparse_gb300.mtx import read_mtx_coo_reference
    name, text, shape, rows, cols, vals = case
    p = _write(tmp_path / f"{name}.mtx", text)
    M, N, r, c, v = read_mtx_coo_reference(p)
    assert (M, N) == tuple(shape)
    assert np.array_equal(r, rows) and np.array_equal(c, cols)
    assert _same_up_to_ties(r, c, v, vals)
    a = read_mtx(p)
    assert np.array_equal(np.repeat(np.arange(M), np.diff(a.rowptr)), rows)
    assert np.array_equal(a.colind, cols)


def test_reference_reading_against_compiled_readmtx(tmp_path):
    """Seeded files of every kind through the reference's reader compiled here (skipped where
    its sources are absent), compared bit for bit."""
    from oracle import oracle as O
    from armsparse_gb300.mtx import read_mtx_coo_reference
    rng = np.random.default_rng(7)
    if O.ref_lib("mtx") is None:
        pytest.skip("reference reader not built (no reference sources)")
    for t in range(12):
        n = int(rng.integers(5, 60))
        k = int(rng.integers(1, 150))
        symm = ["general", "symmetric", "skew-symmetric"][t % 3]
        field = ["real", "pattern", "integer"][(t // 3) % 3]
        keys = set()
        for _ in range(k):
            r, c = int(rng.integers(1, n + 1)), int(rng.integers(1, n + 1))
            if symm != "general" and c > r:
                r, c = c, r
            keys.add((r, c))
        lines = []
        for r, c in sorted(keys, key=lambda _: rng.random()):
            val = "" if field == "pattern" else (f" {int(rng.integers(-5, 6))}" if field == "integer"
                                                  else f" {rng.normal():.7g}")
            lines.append(f"{r} {c}{val}")
        # exact duplicate lines (the same value), so that no result depends on the order that
        # std::sort gives equal keys
        lines += lines[: int(rng.integers(0, 6))]
        text = f"%%MatrixMarket matrix coordinate {field} {symm}\n{n} {n} {len(lines)}\n" + \
            "\n".join(lines) + "\n"
        p = _write(tmp_path / f"t{t}.mtx", text)
        M, N, r, c, v = read_mtx_coo_reference(p)
        rm, rn, rr, rc, rv = O.ref_read_mtx(p)
        assert (M, N) == (rm, rn)
        assert np.array_equal(r, rr) and np.array_equal(c, rc), (t, symm, field)
        assert np.array_equal(v.view(np.uint32), rv.view(np.uint32)), (t, symm, field)


def test_sum_reading_keeps_scipy_semantics(tmp_path):
    p = _write(tmp_path / "s.mtx", "%%MatrixMarket matrix coordinate real symmetric\n"
               "3 3 4\n1 1 2\n2 1 3\n2 1 1\n3 3 5\n")
    a = read_mtx(p, duplicates="sum")
    dense = np.zeros((3, 3))
    dense[np.repeat(np.arange(3), np.diff(a.rowptr)), a.colind] = a.val
    assert dense.tolist() == [[2, 4, 0], [4, 0, 0], [0, 0, 5]]
    b = read_mtx(p)  # the reference's reading: no diagonal, duplicates dropped
    assert b.colind.tolist() == [1, 0] and b.rowptr.tolist() == [0, 1, 2, 2]
