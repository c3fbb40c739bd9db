"""Seeded synthetic sparse inputs.

Every generator returns CSR arrays with int32 ``rowptr``/``colind``, unique column ids per
row and columns ascending within each row (the order the reference's ``toCSR`` produces,
SDMM.cpp:355-370). The shapes follow the workloads the reference's drivers and GCN scripts
run: uniform random patterns (``prepareSparse``, SDMM.cpp:329-342, here without its
duplicate draws), power-law and banded matrices for the kernel-selector sweep, and an
undirected power-law graph with self-loops for the GCN (``proc``,
gcn/pytorch-custom/gcn_custom.py:38-58).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class CSR:
    rowptr: np.ndarray
    colind: np.ndarray
    val: np.ndarray
    n_rows: int
    n_cols: int

    @property
    def nnz(self) -> int:
        return int(self.colind.size)

    @property
    def shape(self):
        return (self.n_rows, self.n_cols)


def _from_sorted_keys(keys: np.ndarray, n_rows: int, n_cols: int) -> tuple[np.ndarray, np.ndarray]:
    rows = (keys // n_cols).astype(np.int64)
    cols = (keys % n_cols).astype(np.int32)
    counts = np.bincount(rows, minlength=n_rows)
    rowptr = np.zeros(n_rows + 1, np.int64)
    np.cumsum(counts, out=rowptr[1:])
    if rowptr[-1] >= 2 ** 31:
        raise ValueError("nnz does not fit int32 indices")
    return rowptr.astype(np.int32), cols


def _sorted_unique(keys: np.ndarray) -> np.ndarray:
    """Sorted distinct values (sort + neighbour compare; faster than np.unique here)."""
    keys = np.sort(keys)
    if keys.size < 2:
        return keys
    keep = np.empty(keys.size, bool)
    keep[0] = True
    np.not_equal(keys[1:], keys[:-1], out=keep[1:])
    return keys[keep]


def uniform_csr(n_rows: int, n_cols: int, nnz: int, seed: int = 0, values: str = "u11") -> CSR:
    """``nnz`` distinct positions drawn uniformly without replacement."""
    rng = np.random.default_rng(seed)
    total = n_rows * n_cols
    if nnz > total:
        raise ValueError("nnz larger than the matrix")
    if nnz > total // 4:
        keys = np.sort(rng.permutation(total)[:nnz])
    else:
        keys = _sorted_unique(rng.integers(0, total, size=int(nnz * 1.1) + 16, dtype=np.int64))
        while keys.size < nnz:
            more = rng.integers(0, total, size=nnz - keys.size + 64, dtype=np.int64)
            keys = _sorted_unique(np.concatenate([keys, more]))
        keys = np.sort(rng.permutation(keys)[:nnz])
    rowptr, colind = _from_sorted_keys(keys, n_rows, n_cols)
    return CSR(rowptr, colind, make_values(rng, nnz, values), n_rows, n_cols)


def make_values(rng: np.random.Generator, n: int, kind: str) -> np.ndarray:
    if kind == "u11":
        return rng.uniform(-1.0, 1.0, n).astype(np.float32)
    if kind == "u0515":
        return rng.uniform(0.5, 1.5, n).astype(np.float32)
    if kind == "ones":
        return np.ones(n, np.float32)
    if kind == "ref_int":
        # the reference drivers' value rule: (rand()%20000-10000)/1000 (SDMM.cpp:335)
        return ((rng.integers(0, 20000, n) - 10000) / 1000.0).astype(np.float32)
    raise ValueError(kind)


def _rows_with_lengths(rng, lengths: np.ndarray, n_cols: int) -> tuple[np.ndarray, np.ndarray]:
    """Distinct uniform column ids per row with the given lengths, ascending in each row."""
    lengths = np.minimum(lengths.astype(np.int64), n_cols)
    rowptr = np.zeros(lengths.size + 1, np.int64)
    np.cumsum(lengths, out=rowptr[1:])
    nnz = int(rowptr[-1])
    # rows holding more than an eighth of the columns draw without replacement (rejection
    # would need many refill rounds for them); the rest draw with rejection below
    big = np.flatnonzero(lengths > max(n_cols // 8, 64))
    small = lengths.copy()
    small[big] = 0
    row_of = np.repeat(np.arange(lengths.size, dtype=np.int64), small)
    cols = rng.integers(0, n_cols, size=row_of.size, dtype=np.int64)
    parts = [row_of * n_cols + cols]
    for r in big:
        parts.append(r * n_cols + rng.choice(n_cols, int(lengths[r]), replace=False).astype(np.int64))
    keys = _sorted_unique(np.concatenate(parts) if big.size else parts[0])
    # refill duplicates until every row has its length (a few rounds at most)
    for _ in range(64):
        got = np.bincount(keys // n_cols, minlength=lengths.size)
        short = lengths - got
        if not short.any():
            break
        need = np.repeat(np.arange(lengths.size, dtype=np.int64), short)
        extra = need * n_cols + rng.integers(0, n_cols, size=need.size, dtype=np.int64)
        keys = _sorted_unique(np.concatenate([keys, extra]))
    return _from_sorted_keys(keys, lengths.size, n_cols)


def powerlaw_csr(n: int, exponent: float, mean_nnz: float, seed: int = 0,
                 n_cols: int | None = None, values: str = "u11") -> CSR:
    """Row lengths from a discrete power law P(len = d) ~ d^-exponent, rescaled so that the
    mean row length is ``mean_nnz``; column ids uniform."""
    rng = np.random.default_rng(seed)
    n_cols = n if n_cols is None else n_cols
    u = rng.random(n)
    raw = (1.0 - u) ** (-1.0 / (exponent - 1.0))  # Pareto(x_min = 1)
    lengths = raw * (mean_nnz / raw.mean())
    lengths = np.clip(np.floor(lengths + rng.random(n)), 0, n_cols).astype(np.int64)
    rowptr, colind = _rows_with_lengths(rng, lengths, n_cols)
    return CSR(rowptr, colind, make_values(rng, colind.size, values), n, n_cols)


def banded_csr(n: int, bandwidth: int, seed: int = 0, fill: float = 1.0,
               values: str = "u11") -> CSR:
    """Entries within |i - j| <= bandwidth // 2, each kept with probability ``fill``."""
    rng = np.random.default_rng(seed)
    half = bandwidth // 2
    offs = np.arange(-half, bandwidth - half, dtype=np.int64)
    rows = np.repeat(np.arange(n, dtype=np.int64), offs.size)
    cols = rows + np.tile(offs, n)
    keep = (cols >= 0) & (cols < n)
    if fill < 1.0:
        keep &= rng.random(keep.size) < fill
    keys = rows[keep] * n + cols[keep]
    rowptr, colind = _from_sorted_keys(keys, n, n)
    return CSR(rowptr, colind, make_values(rng, colind.size, values), n, n)


def powerlaw_graph(n_nodes: int, n_edges: int, exponent: float = 2.1, seed: int = 0,
                   undirected: bool = True, self_loops: bool = True) -> CSR:
    """Graph adjacency (values 1) with power-law degrees (Chung-Lu style endpoint sampling).

    ``n_edges`` counts directed entries before self-loops; for ``undirected`` graphs both
    (u, v) and (v, u) are stored, so about n_edges / 2 distinct pairs are drawn. Duplicate
    edges are merged (the reference's scipy COO -> CSR conversion sums them,
    gcn_custom.py:45-48; here they are drawn again so that nnz is exact)."""
    rng = np.random.default_rng(seed)
    w = (1.0 - rng.random(n_nodes)) ** (-1.0 / (exponent - 1.0))
    p = w / w.sum()
    cdf = np.cumsum(p)
    cdf[-1] = 1.0
    target = n_edges // 2 if undirected else n_edges
    keys = np.empty(0, np.int64)
    for _ in range(200):
        need = target - keys.size
        if need <= 0:
            break
        m = int(need * 1.2) + 64
        u = np.searchsorted(cdf, rng.random(m)).astype(np.int64)
        v = np.searchsorted(cdf, rng.random(m)).astype(np.int64)
        ok = u != v
        u, v = u[ok], v[ok]
        if undirected:
            u, v = np.minimum(u, v), np.maximum(u, v)
        fresh = np.setdiff1d(_sorted_unique(u * n_nodes + v), keys, assume_unique=True)
        fresh = rng.permutation(fresh)[:need]
        keys = np.union1d(keys, fresh)
    keys = keys[:target] if keys.size > target else keys
    u, v = keys // n_nodes, keys % n_nodes
    if undirected:
        u, v = np.concatenate([u, v]), np.concatenate([v, u])
    if self_loops:
        ids = np.arange(n_nodes, dtype=np.int64)
        u, v = np.concatenate([u, ids]), np.concatenate([v, ids])
    allk = _sorted_unique(u * n_nodes + v)
    rowptr, colind = _from_sorted_keys(allk, n_nodes, n_nodes)
    return CSR(rowptr, colind, np.ones(colind.size, np.float32), n_nodes, n_nodes)


def dense_uniform(shape, seed: int, lo: float = -1.0, hi: float = 1.0) -> np.ndarray:
    return np.random.default_rng(seed).uniform(lo, hi, shape).astype(np.float32)


def dense_normal(shape, seed: int) -> np.ndarray:
    return np.random.default_rng(seed).standard_normal(shape, dtype=np.float32)


def to_dense(a: CSR) -> np.ndarray:
    d = np.zeros((a.n_rows, a.n_cols), np.float32)
    rows = np.repeat(np.arange(a.n_rows), np.diff(a.rowptr))
    d[rows, a.colind] = a.val
    return d


# Workloads named by their sizes (the configurations the reference's drivers and GCN run).
def spmm_4096_d001(seed: int = 0) -> CSR:
    """SpMM/SpMV driver shape: 4096 x 4096, density 0.01 (167,772 entries), values U(-1,1)."""
    return uniform_csr(4096, 4096, int(0.01 * 4096 * 4096), seed)


def sddmm_4096_d01(seed: int = 0) -> CSR:
    """SDDMM pattern: 4096 x 4096, density 0.1 (1,677,721 entries), values U(0.5,1.5)."""
    return uniform_csr(4096, 4096, int(0.1 * 4096 * 4096), seed, values="u0515")


# ---- generators on the GPU (for the selector sweep: hundreds of matrices up to 1M rows) -------
def _csr_from_sorted_keys_torch(keys, n_rows, n_cols):
    import torch
    rows = keys // n_cols
    cols = (keys % n_cols).to(torch.int32)
    counts = torch.bincount(rows, minlength=n_rows)
    rowptr = torch.zeros(n_rows + 1, dtype=torch.int64, device=keys.device)
    rowptr[1:] = torch.cumsum(counts, 0)
    return rowptr.to(torch.int32), cols


def powerlaw_csr_device(n, exponent, mean_nnz, seed, device, n_cols=None):
    """Same distribution as powerlaw_csr (Pareto row lengths rescaled to the mean, uniform
    column ids), drawn with a seeded torch generator on the device; duplicate column ids in a
    row are merged, so rows may come out slightly shorter than drawn."""
    import torch
    n_cols = n if n_cols is None else n_cols
    g = torch.Generator(device=device).manual_seed(seed)
    u = torch.rand(n, generator=g, device=device, dtype=torch.float64)
    raw = (1.0 - u) ** (-1.0 / (exponent - 1.0))
    lengths = raw * (mean_nnz / raw.mean())
    lengths = torch.clamp(torch.floor(lengths + torch.rand(n, generator=g, device=device,
                                                           dtype=torch.float64)), 0, n_cols).long()
    rows = torch.repeat_interleave(torch.arange(n, device=device), lengths)
    cols = torch.randint(0, n_cols, (rows.numel(),), generator=g, device=device)
    keys = torch.unique(rows * n_cols + cols)  # sorted
    rowptr, colind = _csr_from_sorted_keys_torch(keys, n, n_cols)
    val = torch.rand(colind.numel(), generator=g, device=device) * 2 - 1
    return rowptr, colind, val


def banded_csr_device(n, bandwidth, seed, device):
    import torch
    g = torch.Generator(device=device).manual_seed(seed)
    half = bandwidth // 2
    offs = torch.arange(-half, bandwidth - half, device=device)
    rows = torch.arange(n, device=device).repeat_interleave(offs.numel())
    cols = rows + offs.repeat(n)
    keep = (cols >= 0) & (cols < n)
    keys = rows[keep] * n + cols[keep]
    rowptr, colind = _csr_from_sorted_keys_torch(keys, n, n)
    val = torch.rand(colind.numel(), generator=g, device=device) * 2 - 1
    return rowptr, colind, val


def powerlaw_graph_device(n_nodes, n_edges, exponent, seed, device, self_loops=True):
    """Directed power-law graph on the device (Chung-Lu endpoint sampling with Pareto weights,
    both endpoints drawn from the same weights), duplicates merged, self-loops added; CSR
    (rowptr, colind) with values 1. For the large GCN layer: 2.4M nodes, 62M edges."""
    import torch
    g = torch.Generator(device=device).manual_seed(seed)
    w = (1.0 - torch.rand(n_nodes, generator=g, device=device, dtype=torch.float64)) ** \
        (-1.0 / (exponent - 1.0))
    cdf = torch.cumsum(w / w.sum(), 0)
    cdf[-1] = 1.0
    u = torch.searchsorted(cdf, torch.rand(n_edges, generator=g, device=device, dtype=torch.float64))
    v = torch.searchsorted(cdf, torch.rand(n_edges, generator=g, device=device, dtype=torch.float64))
    u = u.clamp_(max=n_nodes - 1)
    v = v.clamp_(max=n_nodes - 1)
    keys = u * n_nodes + v
    if self_loops:
        ids = torch.arange(n_nodes, device=device)
        keys = torch.cat([keys, ids * n_nodes + ids])
    keys = torch.unique(keys)
    rowptr, colind = _csr_from_sorted_keys_torch(keys, n_nodes, n_nodes)
    return rowptr, colind, torch.ones(colind.numel(), device=device)
