"""Row sharding of the sparse operand across ranks (no data-path collective).

The path shards by rows: SpMM / SpMV give rank r the CSR rows [row_begin[r], row_begin[r+1])
of A with B (or x) replicated, so each rank writes its own rows of C and nothing is exchanged;
SDDMM shards the same way (each entry belongs to one row). The split balances stored entries,
not rows, so power-law graphs do not leave one rank with the heavy rows -- the GPU analogue of
the reference's nnz-balanced NUMA split (numaAware/balanceNUMAAwareSPDM.cpp:251-271), minus its
partial-C sum reduction (a row split needs none).
"""
from __future__ import annotations

import numpy as np


def balanced_row_blocks(rowptr, world: int) -> np.ndarray:
    """row_begin[0..world]: contiguous row blocks with about nnz / world entries each (rows are
    never split, so a block can exceed the share by at most one row)."""
    rowptr = np.asarray(rowptr, dtype=np.int64)
    M = rowptr.size - 1
    nnz = int(rowptr[-1])
    targets = (np.arange(1, world, dtype=np.int64) * nnz) // world
    cuts = np.searchsorted(rowptr, targets, side="left")
    cuts = np.clip(cuts, 0, M)
    return np.concatenate([[0], np.maximum.accumulate(cuts), [M]]).astype(np.int64)


def shard_csr(rowptr, colind, val, row_begin, rank: int):
    """The CSR block of rank `rank` (row pointer rebased to 0)."""
    rowptr = np.asarray(rowptr)
    r0, r1 = int(row_begin[rank]), int(row_begin[rank + 1])
    e0, e1 = int(rowptr[r0]), int(rowptr[r1])
    return (np.ascontiguousarray(rowptr[r0:r1 + 1] - e0, dtype=np.int32),
            np.ascontiguousarray(colind[e0:e1]), np.ascontiguousarray(val[e0:e1]))
