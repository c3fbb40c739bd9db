"""Row sharding on two CPU ranks (gloo): each rank computes its nnz-balanced row block of
C = A*B with the oracle's rowBaseSpmm3 restatement and the blocks are all-gathered; the result
is bit-identical to the unsharded product (a row split changes no summation order)."""
import os
import socket

import numpy as np
import pytest
import torch
import torch.distributed as dist
import torch.multiprocessing as mp

from armsparse_gb300 import shard
from armsparse_gb300 import synthetic as S


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _worker(rank, world, port, result_path):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from oracle import oracle as O
    a = S.powerlaw_csr(3000, 2.0, 12.0, seed=5, n_cols=2000)
    B = S.dense_uniform((2000, 24), 6)
    rb = shard.balanced_row_blocks(a.rowptr, world)
    rp, ci, v = shard.shard_csr(a.rowptr, a.colind, a.val, rb, rank)
    mine = torch.from_numpy(O.spmm_fma_chain_f32(rp, ci, v, B, threads=1))
    # gather variable-size row blocks: pad to the largest block
    rows = [int(rb[r + 1] - rb[r]) for r in range(world)]
    pad = torch.zeros(max(rows), 24)
    pad[: mine.shape[0]] = mine
    parts = [torch.zeros(max(rows), 24) for _ in range(world)]
    dist.all_gather(parts, pad)
    if rank == 0:
        C = torch.cat([p[:n] for p, n in zip(parts, rows)]).numpy()
        full = O.spmm_fma_chain_f32(a.rowptr, a.colind, a.val, B, threads=1)
        np.save(result_path, np.stack([C, full]))
    dist.barrier()
    dist.destroy_process_group()


def test_balanced_blocks_cover_rows_and_balance_entries():
    a = S.powerlaw_csr(10000, 1.9, 20.0, seed=1)
    for world in (1, 2, 3, 8):
        rb = shard.balanced_row_blocks(a.rowptr, world)
        assert rb[0] == 0 and rb[-1] == a.n_rows and np.all(np.diff(rb) >= 0)
        per = np.diff(a.rowptr[rb])
        longest = int(np.diff(a.rowptr).max())
        assert per.max() <= a.nnz / world + longest


def test_two_rank_row_sharded_spmm_matches_unsharded(tmp_path):
    out = str(tmp_path / "res.npy")
    mp.spawn(_worker, args=(2, _free_port(), out), nprocs=2, join=True)
    C, full = np.load(out)
    assert np.array_equal(C.view(np.uint32), full.view(np.uint32))
