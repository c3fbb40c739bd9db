"""Matrix Market reader -> CSR (host side).

Two readings of a coordinate file:

``duplicates="reference"`` (default) -- what the reference's reader does (``readMtx``,
gcn/util/util.hpp:286-333, with the NIST banner and size parsers of gcn/util/mmio.hpp:215-336):

* the banner's object must be ``matrix`` and its format ``coordinate`` (case-insensitive); the
  field is ``real`` (each value read as a float32, as ``fscanf("%f")`` does), ``integer``
  (``%d``, then converted) or ``pattern`` (every value 1);
* indices are 1-based; entries are whitespace-separated tokens after the size line;
* only a ``symmetric`` file is expanded (``makeSymmetric``, util.hpp:218-284): every
  off-diagonal entry (r, c, v) gains its mirror (c, r, v); the entries are sorted by (row,
  column); self-loops are dropped, and of equal (row, column) entries only the first in
  sorted order stays -- duplicates are dropped, not summed. The reference's compaction loop
  (util.hpp:262-276) moves row and column indices but not values, so after the first dropped
  entry each kept entry carries the value at its own position in the sorted list: the value
  array is the sorted values cut to the kept count. That is restated here; for ``pattern``
  files (every value 1), the GCN graphs' case, it changes nothing;
* ``general``, ``skew-symmetric`` and ``hermitian`` files are read as stored (the reference
  expands only ``symmetric``), sorted by (row, column), duplicates kept as separate entries;
* where the reference's ``std::sort`` leaves entries with equal (row, column) in an
  unspecified order, this reader keeps them in file order (stable sort).

``duplicates="sum"`` -- the scipy COO -> CSR reading of the GCN path (gcn_custom.py:45-48):
``symmetric`` / ``skew-symmetric`` / ``hermitian`` files expanded to both triangles (the
diagonal once, skew mirrors negated), duplicate entries summed, the diagonal kept.

Both reject what the reference would mis-read: ``complex`` fields (its reader reads no entries
for them), the ``array`` format, indices outside the stated shape, and files with fewer
entries than the size line states. Output: int32 rowptr/colind (columns ascending in every
row), float32 values.
"""
from __future__ import annotations

import decimal

import numpy as np

from .synthetic import CSR


def _parse_f32(tokens) -> np.ndarray:
    """Decimal strings -> float32, each rounded once to nearest (as strtof / fscanf "%f" do).

    Parsing goes through float64; a float64 that lands exactly halfway between two float32
    values may stand for a decimal slightly above or below that point, so those few are
    decided on the exact decimal value instead of by round-half-even."""
    d = np.array(tokens, dtype=np.float64)
    with np.errstate(over="ignore"):
        f = d.astype(np.float32)
    fd = f.astype(np.float64)
    other = np.where(fd < d, np.nextafter(f, np.float32(np.inf)), np.nextafter(f, np.float32(-np.inf)))
    od = other.astype(np.float64)
    with np.errstate(invalid="ignore"):
        tie = np.isfinite(d) & np.isfinite(od) & (fd != d) & (np.abs(d - fd) == np.abs(od - d))
    for i in np.flatnonzero(tie):
        exact, mid = decimal.Decimal(tokens[i]), decimal.Decimal(float(d[i]))
        if exact != mid:
            f[i] = max(f[i], other[i]) if exact > mid else min(f[i], other[i])
    return f


def _read_coordinate(path: str):
    """Banner, shape and the raw (row, col, value) lists of a coordinate file (0-based)."""
    with open(path) as fh:
        banner = fh.readline().split()
        if len(banner) < 5 or not banner[0].startswith("%%MatrixMarket"):
            raise ValueError(f"{path}: not a MatrixMarket file")
        obj, fmt, field, symm = (t.lower() for t in banner[1:5])
        if obj != "matrix":
            raise ValueError(f"{path}: not a MatrixMarket matrix file")
        if fmt != "coordinate":
            raise ValueError(f"{path}: only the coordinate format is supported")
        if field not in ("real", "integer", "pattern", "double"):
            raise ValueError(f"{path}: unsupported field {field}")
        line = fh.readline()
        while line and (line.startswith("%") or not line.strip()):
            line = fh.readline()
        size = line.split()
        if len(size) < 3:
            raise ValueError(f"{path}: missing size line")
        M, N, L = (int(x) for x in size[:3])
        tokens = fh.read().split()
    per = 2 if field == "pattern" else 3
    if len(tokens) < per * L:
        raise ValueError(f"{path}: expected {L} entries, found {len(tokens) // per}")
    t = tokens[: per * L]
    r = np.array(t[0::per], dtype=np.int64) - 1
    c = np.array(t[1::per], dtype=np.int64) - 1
    if field == "pattern":
        v = np.ones(L, np.float32)
    elif field == "integer":
        v = np.array(t[2::per], dtype=np.int64).astype(np.float32)
    else:
        v = _parse_f32(t[2::per])
    if L and ((r < 0) | (r >= M) | (c < 0) | (c >= N)).any():
        raise ValueError(f"{path}: index out of range")
    return M, N, symm, r, c, v


def _to_csr(M, N, rows, cols, vals) -> CSR:
    rowptr = np.zeros(M + 1, np.int64)
    np.cumsum(np.bincount(rows, minlength=M), out=rowptr[1:])
    return CSR(rowptr.astype(np.int32), np.asarray(cols, np.int32),
               np.asarray(vals, np.float32), M, N)


def read_mtx_coo_reference(path: str):
    """(M, N, rows, cols, vals) exactly as the reference's readMtx leaves its three vectors
    (util.hpp:286-333): see the module docstring."""
    M, N, symm, r, c, v = _read_coordinate(path)
    if symm == "symmetric" and r.size:
        off = r != c
        r, c, v = (np.concatenate([r, c[off]]), np.concatenate([c, r[off]]),
                   np.concatenate([v, v[off]]))
        order = np.lexsort((c, r))  # stable: ties keep their order
        r, c, v = r[order], c[order], v[order]
        dup = np.zeros(r.size, bool)
        dup[1:] = (r[1:] == r[:-1]) & (c[1:] == c[:-1])
        keep = ~dup & (r != c)
        r, c = r[keep], c[keep]
        v = v[: r.size]  # the compaction moves indices only (util.hpp:262-276)
    else:
        order = np.lexsort((c, r))
        r, c, v = r[order], c[order], v[order]
    return M, N, r, c, v


def read_mtx(path: str, duplicates: str = "reference") -> CSR:
    """A Matrix Market coordinate file as CSR; ``duplicates`` is "reference" or "sum" (see the
    module docstring)."""
    if duplicates == "reference":
        M, N, r, c, v = read_mtx_coo_reference(path)
        return _to_csr(M, N, r, c, v)
    if duplicates != "sum":
        raise ValueError('duplicates must be "reference" or "sum"')
    M, N, symm, r, c, v = _read_coordinate(path)
    v = v.astype(np.float64)
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
    return _to_csr(M, N, uniq // N, (uniq % N).astype(np.int32), vals.astype(np.float32))
