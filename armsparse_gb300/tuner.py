"""Exhaustive autotuner for the SpMM kernel variants (and the SDDMM paths).

The nearest reference logic is a static dispatch on the dense width (k < 32 / k < 64 / else
in gcn/pytorch-custom/spmm_kernel.cu:437-457, and k % 4 / k % 2 in sddmm.cu:438-455). Here
every variant that can run the arguments is timed with CUDA events on the current stream,
L2 flushed before every repetition, and the median is kept. The tuner is the fallback when
no learned selector is loaded and the yardstick the selector is scored against.
"""
from __future__ import annotations

import math
import statistics
from dataclasses import dataclass

import numpy as np
import torch

from . import _native as N
from . import sparse as S

_FLUSH = {}


def _flush_buffer(device: torch.device, nbytes: int = 256 << 20) -> torch.Tensor:
    key = (device.index, nbytes)
    if key not in _FLUSH:
        _FLUSH[key] = torch.empty(nbytes, dtype=torch.uint8, device=device)
    return _FLUSH[key]


def time_cuda(fn, reps: int = 5, warmup: int = 1, flush: bool = True,
              device: torch.device | None = None) -> float:
    """Median milliseconds of fn() over reps, each bracketed by CUDA events on the current
    stream (L2 flushed before each repetition when flush is set)."""
    device = device or torch.device("cuda", torch.cuda.current_device())
    stream = torch.cuda.current_stream(device)
    buf = _flush_buffer(device) if flush else None
    for _ in range(warmup):
        fn()
    times = []
    for i in range(reps):
        if buf is not None:
            buf.fill_(i & 0xFF)
        s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        s.record(stream)
        fn()
        e.record(stream)
        e.synchronize()
        times.append(s.elapsed_time(e))
    return statistics.median(times)


@dataclass
class Timing:
    variant: int
    name: str
    ms: float | None  # None: the variant cannot run these arguments


def autotune_spmm(rowptr, colind, val, B, C=None, variants=None, reps: int = 5,
                  flush: bool = True, max_ratio: float | None = None) -> list[Timing]:
    """Time every SpMM variant (or the given ids) on these arguments. With max_ratio, a
    variant whose first timed run is more than max_ratio x the best time so far keeps that
    single measurement (it cannot be the pick; this bounds the sweep time)."""
    names = S.spmm_variants(B.dtype)
    ids = variants or list(range(1, len(names) + 1))
    M = rowptr.numel() - 1
    if C is None:
        C = torch.empty((M, B.shape[1]), dtype=torch.float32, device=B.device)
    out = []
    best_ms = None
    for v in ids:
        try:
            S.spmm(rowptr, colind, val, B, C=C, variant=v)
        except N.NativeError as e:
            if e.status == 3:  # AS_ERR_UNSUPPORTED
                out.append(Timing(v, names[v - 1], None))
                continue
            raise
        fn = lambda: S.spmm(rowptr, colind, val, B, C=C, variant=v)
        ms = time_cuda(fn, reps=1, warmup=0, flush=flush, device=B.device)
        if not (max_ratio and best_ms is not None and ms > max_ratio * best_ms):
            ms = time_cuda(fn, reps=reps, warmup=0, flush=flush, device=B.device)
        best_ms = ms if best_ms is None else min(best_ms, ms)
        out.append(Timing(v, names[v - 1], ms))
    return out


def best(timings: list[Timing]) -> Timing:
    ok = [t for t in timings if t.ms is not None]
    return min(ok, key=lambda t: t.ms)


# ------------------------------------------------------------------------------------------
# Cheap matrix features (inputs of the learned selector)
# ------------------------------------------------------------------------------------------
HIST_BINS = 12  # row-length histogram over log2 buckets: 0, 1, 2-3, 4-7, ..., >= 1024


def features(rowptr: np.ndarray, n_cols: int, N: int, dtype_bf16: bool) -> np.ndarray:
    """rows, nnz, mean/std/max row length, coefficient of variation, a normalised log2 row-
    length histogram, dense width N and the storage dtype -- all O(rows) from rowptr."""
    rowptr = np.asarray(rowptr, dtype=np.int64)
    lens = np.diff(rowptr).astype(np.float64)
    M = lens.size
    nnz = float(rowptr[-1]) if M else 0.0
    mean = lens.mean() if M else 0.0
    std = lens.std() if M else 0.0
    mx = lens.max() if M else 0.0
    b = np.zeros(HIST_BINS)
    if M:
        idx = np.where(lens <= 0, 0, np.minimum(np.floor(np.log2(np.maximum(lens, 1))) + 1,
                                                 HIST_BINS - 1)).astype(np.int64)
        b = np.bincount(idx, minlength=HIST_BINS)[:HIST_BINS] / M
    f = [np.log2(M + 1), np.log2(nnz + 1), np.log2(n_cols + 1), np.log2(mean + 1),
         np.log2(std + 1), np.log2(mx + 1), std / (mean + 1e-9), np.log2(N), float(dtype_bf16),
         float(N % 4 == 0), float(N % 8 == 0)]
    return np.concatenate([np.asarray(f, np.float64), b]).astype(np.float32)


N_FEATURES = 11 + HIST_BINS


# ------------------------------------------------------------------------------------------
# SDDMM paths
# ------------------------------------------------------------------------------------------
def sddmm_paths() -> list[str]:
    """Names of the SDDMM paths a fp32 call can take: "simt" (CUDA-core FP32 dot products,
    as_sddmm_csr_f32) and "tc1".."tcN" (the tcgen05 split-bf16 kernel variants,
    as_sddmm_csr_bf16x3_v). The reference has one kind only, picked by K % 4 / K % 2
    (gcn/pytorch-custom/sddmm.cu:438-455)."""
    n = int(N.load().as_sddmm_bf16x3_variant_count())
    return ["simt"] + [f"tc{v}" for v in range(1, n + 1)]


def run_sddmm_path(name: str, rowptr, colind, X, Y, aval=None, out=None):
    """One SDDMM through the named path (see sddmm_paths)."""
    if name == "simt":
        return S.sddmm(rowptr, colind, X, Y, aval=aval, out=out)
    return S.sddmm(rowptr, colind, X, Y, aval=aval, out=out, tensor_cores=True,
                   variant=int(name[2:]))


def autotune_sddmm(rowptr, colind, X, Y, aval=None, paths=None, reps: int = 5,
                   flush: bool = True, max_ratio: float | None = None) -> list[Timing]:
    """Time every SDDMM path on these arguments (median of reps, L2 flushed); the Timing's
    ``variant`` is the index into sddmm_paths()."""
    names = sddmm_paths()
    paths = paths or names
    out = torch.empty(colind.numel(), dtype=torch.float32, device=X.device)
    res, best_ms = [], None
    for name in paths:
        fn = lambda: run_sddmm_path(name, rowptr, colind, X, Y, aval, out)
        try:
            fn()
        except N.NativeError as e:
            if e.status == 3:  # AS_ERR_UNSUPPORTED
                res.append(Timing(names.index(name), name, None))
                continue
            raise
        ms = time_cuda(fn, reps=1, warmup=0, flush=flush, device=X.device)
        if not (max_ratio and best_ms is not None and ms > max_ratio * best_ms):
            ms = time_cuda(fn, reps=reps, warmup=0, flush=flush, device=X.device)
        best_ms = ms if best_ms is None else min(best_ms, ms)
        res.append(Timing(names.index(name), name, ms))
    return res


SDDMM_TILE = (128, 256)  # output tile of the tcgen05 kernels (rows x columns)
N_SDDMM_FEATURES = 10


def sddmm_features(rowptr: torch.Tensor, colind: torch.Tensor, n_cols: int, K: int) -> np.ndarray:
    """Inputs of the learned SDDMM path choice: log2 of rows, columns, K and entries; density;
    mean and coefficient of variation of the row lengths; the fraction of 128 x 256 output
    tiles that hold an entry and the work those tiles carry per entry (the dense tiles the
    tensor-core path computes divided by the entries it keeps: its wasted-work factor) -- the
    last two from one pass over the pattern on the device."""
    M = rowptr.numel() - 1
    nnz = int(colind.numel())
    lens = (rowptr[1:] - rowptr[:-1]).double()
    mean = float(lens.mean()) if M else 0.0
    cv = float(lens.std(unbiased=False) / (lens.mean() + 1e-9)) if M else 0.0
    tr, tc = SDDMM_TILE
    n_tiles_c = (n_cols + tc - 1) // tc
    n_tiles = max(1, ((M + tr - 1) // tr) * n_tiles_c)
    if nnz:
        rows = torch.repeat_interleave(torch.arange(M, device=rowptr.device),
                                       (rowptr[1:] - rowptr[:-1]).long())
        tiles = (rows // tr) * n_tiles_c + (colind.long() // tc)
        occupied = int(torch.unique(tiles).numel())
    else:
        occupied = 0
    density = nnz / max(1.0, float(M) * n_cols)
    waste = occupied * tr * tc / max(1, nnz)
    f = [math.log2(M + 1), math.log2(n_cols + 1), math.log2(K + 1), math.log2(nnz + 1),
         density, math.log2(mean + 1), cv, occupied / n_tiles, math.log2(waste + 1),
         math.log2(K * nnz + 1)]
    return np.asarray(f, np.float32)


# ------------------------------------------------------------------------------------------
# Storage formats
# ------------------------------------------------------------------------------------------
def autotune_formats(rowptr, colind, val, B, reps: int = 5, exact: bool = True,
                     variant: int = 0) -> dict:
    """Time one SpMM (fp32) in each storage format the library has, the conversion from CSR
    done once beforehand and timed separately:
      "csr"     -- the CSR kernels (``variant``, 0 = library default);
      "vcsr4"   -- the reference's 1x4-blocked layout (toVectorAwareCSR, SpMV.cpp:15-38);
      "rowpair" -- the reference's row-pair reuse layout (toDataReuseFormat,
                   suitesparse_sdmm.cpp:150-179), only when ``exact`` is False: its odd rows
                   sum in DataReuseSpmm's order, not the CSR order.
    "csr" and "vcsr4" give the same bits. Returns {"times": {format: {"ms", "convert_ms"}},
    "pick": fastest format}; a caller that reuses the matrix converts once and keeps the pick."""
    out = {}
    C = torch.empty((rowptr.numel() - 1, B.shape[1]), dtype=torch.float32, device=B.device)
    out["csr"] = {"ms": time_cuda(lambda: S.spmm(rowptr, colind, val, B, C=C, variant=variant),
                                  reps=reps), "convert_ms": 0.0}
    conv_ms = time_cuda(lambda: S.csr_to_vcsr4(rowptr, colind, val), reps=1, warmup=1)
    vr, vc, vv = S.csr_to_vcsr4(rowptr, colind, val)
    out["vcsr4"] = {"ms": time_cuda(lambda: S.spmm_vcsr4(vr, vc, vv, B, C=C), reps=reps),
                    "convert_ms": conv_ms, "slots_per_entry": vc.numel() / max(1, colind.numel())}
    if not exact:
        conv_ms = time_cuda(lambda: S.csr_to_rowpair(rowptr, colind, val), reps=1, warmup=1)
        r2, c2, v2, f2 = S.csr_to_rowpair(rowptr, colind, val)
        out["rowpair"] = {"ms": time_cuda(lambda: S.spmm_rowpair(r2, c2, v2, f2, B, C=C), reps=reps),
                          "convert_ms": conv_ms,
                          "shared_fraction": float(f2.float().mean()) if f2.numel() else 0.0}
    return {"times": out, "pick": min(out, key=lambda k: out[k]["ms"])}
