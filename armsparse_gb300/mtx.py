"""Matrix Market reader -> CSR (host side).

Follows what the reference's readers do with SuiteSparse files (gcn/util/util.hpp:286-333 and
the drivers' ad-hoc parsers, suitesparse_spmm.cpp:323-340): the coordinate format, 1-based
indices, `pattern` entries read as 1, `symmetric` / `skew-symmetric` / `hermitian` files
expanded to both triangles (diagonal once), duplicate entries summed (as scipy's COO -> CSR
conversion on the GCN path does, gcn_custom.py:45-48). Output: int32 rowptr/colind with
columns ascending in every row, float32 values.
"""
from __future__ import annotations

import numpy as np

from .synthetic import CSR


def read_mtx(path: str) -> CSR:
    with open(path) as f:
        header = f.readline().split()
        if len(header) < 5 or header[0] != "%%MatrixMarket" or header[1] != "matrix":
            raise ValueError(f"{path}: not a MatrixMarket matrix file")
        fmt, field, symm = header[2].lower(), header[3].lower(), header[4].lower()
        if fmt != "coordinate":
            raise ValueError(f"{path}: only the coordinate format is supported")
        if field not in ("real", "integer", "pattern", "double"):
            raise ValueError(f"{path}: unsupported field {field}")
        line = f.readline()
        while line.startswith("%") or not line.strip():
            line = f.readline()
        M, N, L = (int(x) for x in line.split()[:3])
        ncol = 2 if field == "pattern" else 3
        data = np.loadtxt(f, ndmin=2, usecols=range(ncol)) if L > 0 else np.zeros((0, ncol))
    if data.shape[0] != L:
        raise ValueError(f"{path}: expected {L} entries, found {data.shape[0]}")
    r = data[:, 0].astype(np.int64) - 1
    c = data[:, 1].astype(np.int64) - 1
    v = np.ones(L, np.float64) if field == "pattern" else data[:, 2].astype(np.float64)
    if ((r < 0) | (r >= M) | (c < 0) | (c >= N)).any():
        raise ValueError(f"{path}: index out of range")
    if symm in ("symmetric", "skew-symmetric", "hermitian"):
        off = r != c
        sign = -1.0 if symm == "skew-symmetric" else 1.0
        r, c, v = (np.concatenate([r, c[off]]), np.concatenate([c, r[off]]),
                   np.concatenate([v, sign * v[off]]))
    keys = r * N + c
    order = np.argsort(keys, kind="stable")
    keys, v = keys[order], v[order]
    uniq, start = np.unique(keys, return_index=True)
    vals = np.add.reduceat(v, start) if v.size else v
    rows, cols = uniq // N, (uniq % N).astype(np.int32)
    rowptr = np.zeros(M + 1, np.int64)
    np.cumsum(np.bincount(rows, minlength=M), out=rowptr[1:])
    return CSR(rowptr.astype(np.int32), cols, vals.astype(np.float32), M, N)
