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
    a = read_mtx(p)
    assert a.shape == (3, 4)
    assert a.rowptr.tolist() == [0, 2, 3, 4]
    assert a.colind.tolist() == [0, 1, 0, 3]
    assert a.val.tolist() == [4.0, 2.0, 3.0, -2.0]


def test_symmetric_pattern_expands_both_triangles(tmp_path):
    p = _write(tmp_path / "s.mtx", "%%MatrixMarket matrix coordinate pattern symmetric\n"
               "3 3 3\n1 1\n2 1\n3 2\n")
    a = read_mtx(p)
    dense = np.zeros((3, 3))
    dense[np.repeat(np.arange(3), np.diff(a.rowptr)), a.colind] = a.val
    assert (dense == dense.T).all() and dense.sum() == 5.0 and dense[0, 0] == 1.0


def test_rejects_bad_files(tmp_path):
    with pytest.raises(ValueError):
        read_mtx(_write(tmp_path / "b.mtx", "%%MatrixMarket matrix array real general\n2 2\n1\n2\n3\n4\n"))
    with pytest.raises(ValueError):
        read_mtx(_write(tmp_path / "c.mtx", "%%MatrixMarket matrix coordinate real general\n2 2 1\n3 1 1.0\n"))
