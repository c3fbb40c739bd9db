#!/usr/bin/env python3
"""Benchmark of the sparse hot path on one GB300 (or N independent replicas).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload NAME] [--impl ours|reference]

Default workload: the SpMM driver's case -- A 4096 x 4096 CSR, uniform pattern at density
0.01 (167,772 entries), values U(-1,1) fp32, B 4096 x 4096 fp32 U(-1,1), C = A*B. One step =
one SpMM call on inputs resident in HBM; L2 is flushed (a 256 MiB write) between steps,
outside the timed events. Metric: algorithmic GB/s (every array counted once at its storage
size: 4(M+1) + 8 nnz + 4 K N + 4 M N bytes) and the fraction of the measured HBM copy
bandwidth.

``e2e`` runs the same workload through the reference-facing host call (``origin`` from
libarmsparse_drivers.so, the signature of SDMM.cpp:422) with host buffers: host->device
copies of A and B, the kernel, and the device->host copy of C are inside the timed region.

``--impl reference`` times the reference's CPU algorithm (the oracle's restatement of
rowBaseSpmm3, OpenMP over all host cores) on the same workload and metric.

Multi-GPU: the path shards by rows with nothing to exchange, and this build runs replicas
only -- each rank repeats the whole workload on its own GPU (weak scaling); the time is the
maximum over ranks.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

L2_FLUSH_BYTES = 256 << 20
FALLBACK_HBM_GBS = 6800.0
FALLBACK_BF16_TFLOPS = 1900.0


# ------------------------------------------------------------------------------------------
# Workloads
# ------------------------------------------------------------------------------------------
class Workload:
    """Throughput workloads: value = algorithmic bytes / time (GB/s), higher is better."""
    higher_is_better = True
    bound = "hbm"

    def value(self, seconds: float, ws: int = 1) -> float:
        return ws * self.bytes / seconds / 1e9

    def roofline(self, kernel_ms, hbm, bf16, src):
        if self.bound == "tensor":
            achieved = self.flops / (kernel_ms * 1e-3) / 1e12
            return {"bound": "tensor", "achieved": round(achieved, 3), "peak": bf16,
                    "unit": "TFLOP/s", "frac": round(achieved / bf16, 5),
                    "traffic": profiled_traffic(self.profile), "peak_source": src,
                    "kernel": self.kernel,
                    "achieved_is": "algorithmic (sampled) flops 2*nnz*K per step",
                    "executed_tflops": round(self.exec_flops / (kernel_ms * 1e-3) / 1e12, 2),
                    "executed_frac": round(self.exec_flops / (kernel_ms * 1e-3) / 1e12 / bf16, 4)}
        achieved = self.bytes / (kernel_ms * 1e-3) / 1e9
        return {"bound": "hbm", "achieved": round(achieved, 2), "peak": hbm, "unit": "GB/s",
                "frac": round(achieved / hbm, 4), "traffic": profiled_traffic(self.profile),
                "peak_source": src, "kernel": self.kernel}

    def cpu_value(self, threads: int, budget_s: float):
        """The reference algorithm on the host cores for about budget_s seconds."""
        self.cpu_step(threads)  # warm
        t0 = time.perf_counter()
        total, calls = 0, 0
        while True:
            total += self.cpu_step(threads)
            calls += 1
            if time.perf_counter() - t0 >= budget_s:
                break
        dt = time.perf_counter() - t0
        return total / dt / 1e9, f"{calls} full calls in {dt:.1f} s"

    def flush_between_steps(self) -> bool:
        return True


class SpmmF32(Workload):
    name = "spmm_f32"
    metric = "SpMM GB/s (algorithmic bytes) and % HBM roofline"
    unit = "GB/s"
    dtype = "f32"
    kernel = "spmm_rowsplit (the call; its long-row kernel finds no row over 256 entries here)"
    profile = "spmm_rowsplit_f32_4096x4096x4096_d001"
    e2e_api = "libarmsparse_drivers.so origin() (SDMM.cpp:422 signature) with host buffers"

    def __init__(self, seed=0):
        from armsparse_gb300 import synthetic as S
        self.M = self.K = self.N = 4096
        self.a = S.spmm_4096_d001(seed)
        self.B = S.dense_uniform((self.K, self.N), seed + 1)
        nnz = self.a.nnz
        self.bytes = 4 * (self.M + 1) + 8 * nnz + 4 * self.K * self.N + 4 * self.M * self.N
        self.flops = 2 * nnz * self.N
        self.config = {"workload": "spmm_csr_f32 C=A*B, A 4096x4096 uniform density 0.01 "
                                   "(167,772 nnz) U(-1,1), B 4096x4096 U(-1,1)",
                       "M": 4096, "K": 4096, "N": 4096, "nnz": nnz,
                       "alg_bytes_per_step": self.bytes, "alg_flops_per_step": self.flops,
                       "l2": "flushed between steps (256 MiB write, outside the timed events)"}

    def to_device(self, dev):
        import torch
        self.rp = torch.from_numpy(self.a.rowptr).to(dev)
        self.ci = torch.from_numpy(self.a.colind).to(dev)
        self.v = torch.from_numpy(self.a.val).to(dev)
        self.Bd = torch.from_numpy(self.B).to(dev)
        self.C = torch.empty((self.M, self.N), device=dev)

    def step(self):
        import armsparse_gb300 as A
        A.spmm(self.rp, self.ci, self.v, self.Bd, C=self.C)

    # --- end to end through the reference-facing host call ---
    def e2e_setup(self):
        from armsparse_gb300 import build
        self.drv = ctypes.CDLL(os.path.join(ROOT, "armsparse_gb300", build.DRIVERS_NAME))
        self.hC = np.zeros((self.M, self.N), np.float32)
        self.h = [np.ascontiguousarray(x) for x in (self.a.rowptr, self.a.colind, self.a.val, self.B)]
        self.h2d = sum(x.nbytes for x in self.h)
        self.d2h = self.hC.nbytes

    def e2e_step(self):
        p = lambda x: x.ctypes.data_as(ctypes.c_void_p)
        rp, ci, v, B = self.h
        self.drv.as_drv_origin(p(rp), p(ci), p(v), p(B), p(self.hC), self.M, self.K, self.N, 0)
        if self.drv.as_drv_last_status() != 0:
            raise RuntimeError("e2e call failed")

    # --- CPU: the reference algorithm (oracle restatement of rowBaseSpmm3) ---
    def extra(self):
        """The other headline figures, measured in the same process (capped at about a
        minute): bf16-storage SpMM on this matrix, both SDDMM paths on the 4096^3 density 0.1
        case with their error against FP64, and the GCN epoch tuned vs plain."""
        return default_extras(self)

    # --- reference arm on the GPU: the reference's own spmm_cuda kernels ---
    ref_cuda_kernel = ("spmm_cuda (gcn/pytorch-custom/spmm_kernel.cu:425-458: spmm_test2 at this "
                       "width), compiled for sm_103a from the reference's source")

    def ref_cuda_step(self):
        from oracle import ref_gpu
        ref_gpu.spmm_cuda(self.rp, self.ci, self.v, self.Bd, out=self.C)

    def cpu_step(self, threads, rows=None):
        from oracle import oracle as O
        a = self.a
        if rows is None:
            O.spmm_fma_chain_f32(a.rowptr, a.colind, a.val, self.B, threads=threads)
            return self.bytes
        rp = a.rowptr[: rows + 1]
        O.spmm_fma_chain_f32(rp, a.colind, a.val, self.B, threads=threads)
        nnz = int(rp[-1])
        return 4 * (rows + 1) + 8 * nnz + 4 * self.K * self.N + 4 * rows * self.N


def _scaled_err_max(got, ref64, scale64):
    """max |got - ref| / max(|ref|, sum |terms|) over the outputs (FP64 reference)."""
    import torch
    d = (got.double() - ref64).abs() / torch.maximum(ref64.abs(), scale64).clamp_min(1e-300)
    return float(d.max())


def default_extras(wl, budget_s: float = 60.0):
    """Time-capped figures beside the default SpMM line. FP64 references are computed on the
    GPU with torch (sparse fp64 products and this library's fp64 SDDMM), not by the oracle."""
    import torch
    import armsparse_gb300 as A
    from armsparse_gb300 import tuner
    t_start = time.perf_counter()
    dev = wl.Bd.device
    out = {"budget_s": budget_s}

    def left():
        return budget_s - (time.perf_counter() - t_start)

    # SpMM bf16 storage, fp32 accumulate: same matrix and B, rounded
    try:
        v16, B16 = wl.v.to(torch.bfloat16), wl.Bd.to(torch.bfloat16)
        C16 = torch.empty_like(wl.C)
        f32_ms = tuner.time_cuda(lambda: A.spmm(wl.rp, wl.ci, wl.v, wl.Bd, C=wl.C), reps=20)
        bf_ms = tuner.time_cuda(lambda: A.spmm(wl.rp, wl.ci, v16, B16, C=C16), reps=20)
        Acsr = torch.sparse_csr_tensor(wl.rp.long(), wl.ci.long(), wl.v.double(),
                                       size=(wl.M, wl.K))
        Aabs = torch.sparse_csr_tensor(wl.rp.long(), wl.ci.long(), wl.v.double().abs(),
                                       size=(wl.M, wl.K))
        B64 = wl.Bd.double()
        ref, scale = Acsr @ B64, Aabs @ B64.abs()
        err_f32 = _scaled_err_max(wl.C, ref, scale)
        err_bf = _scaled_err_max(C16, ref, scale)
        del ref, scale, Acsr, Aabs, B64
        bytes16 = 4 * (wl.M + 1) + 6 * wl.a.nnz + 2 * wl.K * wl.N + 4 * wl.M * wl.N
        out["spmm_bf16"] = {"ms": round(bf_ms, 5), "gbs": round(bytes16 / (bf_ms * 1e-3) / 1e9, 1),
                            "speedup_vs_f32": round(f32_ms / bf_ms, 3), "f32_ms": round(f32_ms, 5),
                            "max_scaled_err_vs_fp64": err_bf,
                            "f32_max_scaled_err_vs_fp64": err_f32,
                            "error_metric": "|C - C64| / max(|C64|, sum|a*b|), fp64 of the "
                                            "fp32 inputs"}
    except Exception as e:  # noqa: BLE001 -- a failed extra is reported, not fatal
        out["spmm_bf16"] = {"error": repr(e)[:200]}

    # SDDMM 4096^3 density 0.1, both paths
    if left() > 20:
        try:
            sd = SddmmTc()
            sd.to_device(dev)
            res = {}
            for name, tc in (("tc", True), ("f32", False)):
                fn = lambda: A.sddmm(sd.rp, sd.ci, sd.Xd, sd.Yd, aval=sd.v, out=sd.out,
                                     tensor_cores=tc)
                ms = tuner.time_cuda(fn, reps=10)
                fn()
                res[name] = (ms, sd.out.clone())
            X64, Y64, v64 = sd.Xd.double(), sd.Yd.double(), sd.v.double()
            r64 = A.sddmm(sd.rp, sd.ci, X64, Y64, aval=v64)
            s64 = A.sddmm(sd.rp, sd.ci, X64.abs(), Y64.abs(), aval=v64.abs())
            del X64, Y64
            for name, (ms, o) in res.items():
                out[f"sddmm_{name}"] = {
                    "us": round(ms * 1e3, 1),
                    "gflops_algorithmic": round(sd.flops / (ms * 1e-3) / 1e9, 1),
                    "max_scaled_err_vs_fp64": _scaled_err_max(o, r64, s64)}
            out["sddmm_tc"]["executed_tflops"] = round(sd.exec_flops / (res["tc"][0] * 1e-3) / 1e12, 1)
            del sd, r64, s64, res
        except Exception as e:  # noqa: BLE001
            out["sddmm"] = {"error": repr(e)[:200]}
    # GCN epoch: tuned (captured graph, selector kernels) vs plain (eager, library default)
    if left() > 15:
        try:
            g = GcnEpoch()
            g.to_device(dev)
            for _ in range(3):
                g.step()
            graph_ms = tuner.time_cuda(g.step, reps=20, warmup=2, flush=False)
            plain_ms = tuner.time_cuda(g.plain_step, reps=10, warmup=2, flush=False)
            out["gcn_epoch"] = {"tuned_graph_ms": round(graph_ms, 4),
                                "plain_eager_ms": round(plain_ms, 4),
                                "speedup": round(plain_ms / graph_ms, 2)}
            del g
        except Exception as e:  # noqa: BLE001
            out["gcn_epoch"] = {"error": repr(e)[:200]}
    torch.cuda.empty_cache()
    out["elapsed_s"] = round(time.perf_counter() - t_start, 1)
    return out


class _Generic(Workload):
    """End to end through the public Python API: pinned host inputs copied in, the op,
    the output copied back to pinned host memory, all inside the timed region."""
    bound = "hbm"

    def e2e_setup(self):
        import torch
        self.h_in = {k: v.cpu().pin_memory() for k, v in self.inputs().items()}
        self.h_out = torch.empty(self.output().shape, dtype=self.output().dtype).pin_memory()
        self.h2d = sum(t.numel() * t.element_size() for t in self.h_in.values())
        self.d2h = self.h_out.numel() * self.h_out.element_size()

    def e2e_step(self):
        import torch
        for k, t in self.h_in.items():
            self.inputs()[k].copy_(t, non_blocking=True)
        self.step()
        self.h_out.copy_(self.output(), non_blocking=True)
        torch.cuda.current_stream().synchronize()


class SpmmBf16(_Generic, SpmmF32):
    """The SpMM workload above with A's values and B stored as bf16 (fp32 products and
    accumulation, fp32 C): the bf16-storage path of the GCN layers."""
    name = "spmm_bf16"
    metric = "SpMM GB/s (algorithmic bytes), bf16 storage / fp32 accumulate"
    dtype = "bf16 storage, fp32 accumulate"
    profile = "spmm_rowsplit_bf16_4096x4096x4096_d001"
    e2e_api = "armsparse_gb300.spmm with pinned host inputs copied in and C copied back"

    def __init__(self, seed=0):
        super().__init__(seed)
        nnz = self.a.nnz
        self.bytes = 4 * (self.M + 1) + 6 * nnz + 2 * self.K * self.N + 4 * self.M * self.N
        self.config.update(workload="spmm_csr_bf16 C=A*B, A 4096x4096 uniform density 0.01 "
                                    "(167,772 nnz) U(-1,1), B 4096x4096 U(-1,1), values and B "
                                    "rounded to bf16, C fp32", alg_bytes_per_step=self.bytes)

    def to_device(self, dev):
        import torch
        super().to_device(dev)
        self.v = self.v.to(torch.bfloat16)
        self.Bd = self.Bd.to(torch.bfloat16)

    def inputs(self):
        return {"rp": self.rp, "ci": self.ci, "v": self.v, "B": self.Bd}

    def output(self):
        return self.C

    def cpu_step(self, threads, rows=None):
        from oracle import oracle as O
        if not hasattr(self, "_bf"):
            self._bf = (O.bf16_round(self.a.val), O.bf16_round(self.B))
        v, B = self._bf
        a = self.a
        rp = a.rowptr if rows is None else a.rowptr[: rows + 1]
        O.spmm_fma_chain_f32(rp, a.colind, v, B, threads=threads)
        nnz = int(rp[-1])
        m = a.n_rows if rows is None else rows
        return 4 * (m + 1) + 6 * nnz + 2 * self.K * self.N + 4 * m * self.N


class SpmmPowerlaw(_Generic, SpmmF32):
    """SpMM on a skewed matrix: power-law row lengths (exponent 2.0, mean 20 entries per
    row; the longest row holds all 300,000 columns), 300,000 x 300,000, 5.83M entries, N = 128,
    fp32. `value` is the library-default, bit-exact path (row-split kernels, rows past 256
    entries in the long-row kernel); `extra` times the learned selector's pick."""
    name = "spmm_powerlaw"
    metric = "SpMM GB/s (algorithmic bytes), power-law rows, library default (bit-exact)"
    profile = "spmm_long_powerlaw_300k_n128"
    kernel = "spmm_rowsplit + spmm_long (the call)"
    e2e_api = "armsparse_gb300.spmm with pinned host inputs copied in and C copied back"

    def __init__(self, seed=5):
        from armsparse_gb300 import synthetic as S
        self.a = S.powerlaw_csr(300_000, 2.0, 20.0, seed=seed)
        self.M = self.K = 300_000
        self.N = 128
        self.B = S.dense_uniform((self.K, self.N), seed + 1)
        nnz = self.a.nnz
        self.bytes = 4 * (self.M + 1) + 8 * nnz + 4 * self.K * self.N + 4 * self.M * self.N
        self.flops = 2 * nnz * self.N
        lens = np.diff(self.a.rowptr)
        self.config = {"workload": "spmm_csr_f32 C=A*B, A 300,000 x 300,000 with power-law row "
                                   "lengths (exponent 2.0, mean 20, column ids uniform), "
                                   "B 300,000 x 128 U(-1,1)",
                       "M": self.M, "K": self.K, "N": self.N, "nnz": nnz,
                       "longest_row": int(lens.max()), "rows_over_256": int((lens > 256).sum()),
                       "alg_bytes_per_step": self.bytes, "alg_flops_per_step": self.flops,
                       "l2": "flushed between steps (256 MiB write, outside the timed events)"}

    def inputs(self):
        return {"rp": self.rp, "ci": self.ci, "v": self.v, "B": self.Bd}

    def output(self):
        return self.C

    def extra(self):
        from armsparse_gb300 import selector, tuner
        import armsparse_gb300 as A
        sel = selector.Selector.load()
        v = sel.choose(self.rp, self.K, self.N)
        ms = tuner.time_cuda(lambda: A.spmm(self.rp, self.ci, self.v, self.Bd, C=self.C,
                                             variant=v), reps=10)
        return {"selector_pick": A.spmm_variants()[v - 1], "selector_ms": round(ms, 4),
                "selector_gbs": round(self.bytes / (ms * 1e-3) / 1e9, 1)}


class SpgemmDense(_Generic):
    """Sparse x sparse -> dense as the SpMM driver times it (SpMM.cpp:105-160): A and B
    4096 x 4096 at density 0.01, C += A * B (sparse_matrix_mul3, SpMM.cpp:309-327)."""
    name = "spgemm"
    metric = "SpGEMM (sparse x sparse -> dense) GB/s (algorithmic bytes)"
    unit = "GB/s"
    dtype = "f32"
    kernel = "spgemm_dense"
    profile = "spgemm_dense_4096_d001"

    def __init__(self, seed=0):
        from armsparse_gb300 import synthetic as S
        self.M = self.K = self.N = 4096
        self.a = S.spmm_4096_d001(seed)
        self.b = S.spmm_4096_d001(seed + 1)
        self.C0 = np.zeros((self.M, self.N), np.float32)
        na, nb = self.a.nnz, self.b.nnz
        self.bytes = 4 * (self.M + 1) + 8 * na + 4 * (self.K + 1) + 8 * nb + 8 * self.M * self.N
        self.config = {"workload": "spgemm_csr_dense_f32 C += A*B, A and B 4096x4096 uniform "
                                   "density 0.01 (167,772 entries each) U(-1,1), C dense fp32",
                       "M": 4096, "K": 4096, "N": 4096, "nnz_a": na, "nnz_b": nb,
                       "alg_bytes_per_step": self.bytes,
                       "l2": "flushed between steps (256 MiB write, outside the timed events)"}

    def to_device(self, dev):
        import torch
        t = lambda x: torch.from_numpy(x).to(dev)
        self.A = (t(self.a.rowptr), t(self.a.colind), t(self.a.val))
        self.B = (t(self.b.rowptr), t(self.b.colind), t(self.b.val))
        self.C = t(self.C0)

    def inputs(self):
        return {"arp": self.A[0], "aci": self.A[1], "av": self.A[2], "brp": self.B[0],
                "bci": self.B[1], "bv": self.B[2]}

    def output(self):
        return self.C

    def step(self):
        import armsparse_gb300 as A
        A.spgemm_dense(*self.A, *self.B, self.N, C=self.C, beta=1.0)

    def cpu_step(self, threads, rows=None):
        from oracle import oracle as O
        a, b = self.a, self.b
        O.spgemm_dense_f32(a.rowptr, a.colind, a.val, b.rowptr, b.colind, b.val, self.N,
                           threads=threads)
        return self.bytes


class _SddmmRefCuda:
    ref_cuda_kernel = ("sddmm_cuda_csr (gcn/pytorch-custom/sddmm.cu:459-483: sddmmCSR2Scale), "
                       "compiled for sm_103a from the reference's source; unscaled, on the "
                       "pattern cut to a multiple of 16 entries (its tail blocks read past row "
                       "ends otherwise)")

    def ref_cuda_step(self):
        from oracle import ref_gpu
        if not hasattr(self, "_ref16"):
            import torch
            n16 = self.a.nnz - self.a.nnz % 16
            self._ref16 = (torch.clamp(self.rp, max=n16), self.ci[:n16],
                           torch.empty(n16, device=self.Xd.device))
        rp, ci, out = self._ref16
        ref_gpu.sddmm_cuda_csr(rp, ci, self.Xd, self.Yd, out=out)


class SddmmTc(_Generic, _SddmmRefCuda):
    name = "sddmm_tc"
    metric = "SDDMM GB/s (algorithmic bytes), tensor-core split-bf16 path"
    unit = "GB/s"
    dtype = "bf16x3 (fp32 in/out, fp32 accumulate)"
    kernel = ("the whole as_sddmm_csr_bf16x3 call: fp32 -> bf16 hi/lo split of X and Y, "
              "tile pre-pass, sddmm_tc_persistent")
    profile = "sddmm_tc_persistent_4096x4096x4096_d01"
    bound = "tensor"
    tensor_cores = True

    def __init__(self, seed=0):
        from armsparse_gb300 import synthetic as S
        self.M = self.N = self.K = 4096
        self.a = S.sddmm_4096_d01(seed)
        self.X = S.dense_normal((self.M, self.K), seed + 1)
        self.Y = S.dense_normal((self.N, self.K), seed + 2)
        nnz = self.a.nnz
        self.bytes = 4 * (self.M + 1) + 4 * nnz + 4 * nnz + 4 * nnz + 4 * self.M * self.K + \
            4 * self.N * self.K
        self.flops = 2 * nnz * self.K
        self.exec_flops = 3 * 2 * self.M * self.N * self.K
        self.config = {"workload": "sddmm_csr out[e]=val[e]*<X[r],Y[c]>, pattern 4096x4096 "
                                   "uniform density 0.1 (1,677,721 nnz) val U(0.5,1.5), "
                                   "X,Y 4096x4096 N(0,1), K=4096",
                       "M": 4096, "N": 4096, "K": 4096, "nnz": nnz,
                       "alg_bytes_per_step": self.bytes, "alg_flops_per_step": self.flops,
                       "path": "tensor cores (tcgen05, split-bf16 x3)" if self.tensor_cores
                       else "FP32 CUDA cores",
                       "l2": "flushed between steps (256 MiB write, outside the timed events)"}

    def to_device(self, dev):
        import torch
        self.rp = torch.from_numpy(self.a.rowptr).to(dev)
        self.ci = torch.from_numpy(self.a.colind).to(dev)
        self.v = torch.from_numpy(self.a.val).to(dev)
        self.Xd = torch.from_numpy(self.X).to(dev)
        self.Yd = torch.from_numpy(self.Y).to(dev)
        self.out = torch.empty(self.a.nnz, device=dev)

    def inputs(self):
        return {"rp": self.rp, "ci": self.ci, "v": self.v, "X": self.Xd, "Y": self.Yd}

    def output(self):
        return self.out

    variant = 0  # tensor-core kernel variant (0 = library choice); set by --tc-variant

    def step(self):
        import armsparse_gb300 as A
        A.sddmm(self.rp, self.ci, self.Xd, self.Yd, aval=self.v, out=self.out,
                tensor_cores=self.tensor_cores, variant=self.variant)

    def cpu_step(self, threads, rows=None):
        from oracle import oracle as O
        a = self.a
        if rows is None:
            O.sddmm_f32_lanes(a.rowptr, a.colind, self.X, self.Y, aval=a.val, threads=threads)
            return self.bytes
        rp = a.rowptr[: rows + 1]
        O.sddmm_f32_lanes(rp, a.colind, self.X[:rows], self.Y, aval=a.val, threads=threads)
        nnz = int(rp[-1])
        return 4 * (rows + 1) + 12 * nnz + 4 * rows * self.K + 4 * self.N * self.K


class SddmmF32(SddmmTc):
    name = "sddmm_f32"
    metric = "SDDMM GB/s (algorithmic bytes), FP32 CUDA-core path"
    dtype = "f32"
    kernel = "sddmm_group (a lane group per edge)"
    profile = "sddmm_group_f32_4096x4096x4096_d01"
    bound = "hbm"
    tensor_cores = False


class _CpuSpmm:
    """out = A * feat on the host with the oracle's restatement of the GCN op's kernel
    (csr_spmm_kernel, gcn/pytorch-custom/spmm.cpp:49-71) -- the reference arm of the GCN
    workload; backward uses the CSC arrays as op.py:30 does."""

    @staticmethod
    def make(threads):
        import torch
        from oracle import oracle as O

        class F(torch.autograd.Function):
            @staticmethod
            def forward(ctx, feat, csr, csc):
                ctx.csc = csc
                rp, ci, v = csr
                return torch.from_numpy(O.spmm_fma_chain_f32(rp, ci, v, feat.detach().numpy(),
                                                             threads=threads))

            @staticmethod
            def backward(ctx, g):
                cp, ri, v = ctx.csc
                return (torch.from_numpy(O.spmm_fma_chain_f32(cp, ri, v, g.contiguous().numpy(),
                                                              threads=threads)), None, None)
        return F


class GcnEpoch(Workload):
    """One full-batch training epoch of the 2-layer GCN (gcn_custom.py:122-126) on the
    PubMed-shaped synthetic graph: 19,717 nodes, 88,648 directed edges + self-loops =
    108,365 entries, 500 features (10 % non-zero), hidden 64, 3 classes, Adam."""
    name = "gcn_epoch"
    metric = "GCN training epoch time (ms), 2-layer, 19,717 nodes, 500->64->3"
    unit = "ms/epoch"
    dtype = "f32"
    kernel = "SpMM of layer 1 (N = 64)"
    profile = "gcn_spmm_19717_n64"
    higher_is_better = False

    def __init__(self, seed=0):
        from armsparse_gb300 import synthetic as S
        self.a = S.powerlaw_graph(19717, 88648, seed=seed)
        rng = np.random.default_rng(seed + 1)
        x = np.zeros((19717, 500), np.float32)
        m = rng.random(x.shape) < 0.1
        x[m] = rng.random(int(m.sum())).astype(np.float32)
        self.x = x
        self.y = rng.integers(0, 3, 19717)
        train = np.zeros(19717, bool)
        for c in range(3):
            train[np.flatnonzero(self.y == c)[:60]] = True
        self.train = train
        nnz = self.a.nnz
        self.spmm_bytes = 4 * (19717 + 1) + 8 * nnz + 2 * 19717 * 64 * 4
        self.bytes = self.spmm_bytes
        self.config = {"workload": "GCN 2-layer training epoch, synthetic power-law graph "
                                   "19,717 nodes / 108,365 nnz (incl. self-loops), 500->64->3, "
                                   "Adam lr 0.01, dropout 0.5",
                       "nodes": 19717, "nnz": nnz, "features": 500, "hidden": 64, "classes": 3,
                       "l2": "flushed between epochs (256 MiB write, outside the timed events)"}

    def value(self, seconds, ws=1):
        return seconds * 1e3

    def to_device(self, dev):
        import torch
        from armsparse_gb300 import gcn
        self.dev = dev
        self.xd = torch.from_numpy(self.x).to(dev)
        self.yd = torch.from_numpy(self.y).to(dev)
        self.td = torch.from_numpy(self.train).to(dev)
        self.g = gcn.Graph.from_csr(self.a, dev)
        self.g_plain = gcn.Graph.from_csr(self.a, dev)
        try:
            from armsparse_gb300 import selector
            self.g.selector = selector.Selector.load()
            self.config["kernels"] = "learned selector (armsparse_gb300/selector_model.json)"
        except (OSError, ValueError):
            self.config["kernels"] = "library default (no selector model file)"
        torch.manual_seed(0)
        self.model = gcn.Net(500, 64, 3).to(dev)
        self.opt = gcn.make_optimizer(self.model)
        torch.manual_seed(0)
        self.model_plain = gcn.Net(500, 64, 3).to(dev)
        self.opt_plain = gcn.make_optimizer(self.model_plain)
        self.plan = self.g.plan(64, torch.float32), self.g.plan(3, torch.float32)
        # the features are 10 % non-zero: the tuned path keeps them as CSR, so the first
        # layer's X @ W is an SpMM (and its weight gradient an SpMM with X^T)
        self.feats = gcn.SparseFeatures(self.xd, self.g.selector)
        torch.manual_seed(0)
        self.model_graph = gcn.Net(500, 64, 3).to(dev)
        self.captured = gcn.CapturedEpoch(self.model_graph,
                                          gcn.make_optimizer(self.model_graph, capturable=True),
                                          self.feats, self.g, self.yd, self.td)
        self.config["execution"] = ("selector-tuned kernels, features as CSR (X @ W as SpMM), "
                                    "the epoch recorded once as a CUDA graph and replayed "
                                    "(eager epochs reported in extra)")

    def step(self):
        self.loss = self.captured()

    def launches_per_replay(self):
        return self.captured.launches

    def eager_step(self):
        from armsparse_gb300 import gcn
        return gcn.train_epoch(self.model, self.opt, self.feats, self.g, self.yd, self.td)

    def plain_step(self):
        from armsparse_gb300 import gcn
        return gcn.train_epoch(self.model_plain, self.opt_plain, self.xd, self.g_plain, self.yd,
                               self.td)

    def roofline_ms(self, epoch_ms):
        """Time of the dominant kernel of this project in the epoch: the layer-1 aggregation
        (SpMM, N = 64), timed alone with CUDA events."""
        import torch
        import armsparse_gb300 as A
        from armsparse_gb300 import tuner
        B = torch.rand(19717, 64, device=self.dev)
        C = torch.empty_like(B)
        v = self.plan[0][0]
        return tuner.time_cuda(lambda: A.spmm(self.g.rowptr, self.g.colind, self.g.values, B,
                                              C=C, variant=v), reps=20)

    def e2e_setup(self):
        # the features arrive as CSR from pinned host memory (same pattern every epoch)
        self.hcsr = [t.cpu().pin_memory() for t in (self.feats.rowptr, self.feats.colind,
                                                     self.feats.values)]
        self.h2d = sum(t.numel() * t.element_size() for t in self.hcsr)
        self.d2h = 4

    def e2e_step(self):
        f = self.feats
        f.rowptr.copy_(self.hcsr[0], non_blocking=True)
        f.colind.copy_(self.hcsr[1], non_blocking=True)
        f.load_values(self.hcsr[2])
        self.step()
        float(self.loss)

    # --- reference arm: the same network on the host cores ---
    def _cpu_setup(self, threads):
        if getattr(self, "_cpu", None) is not None:
            return
        import torch
        from oracle import oracle as O
        torch.set_num_threads(threads)
        a = self.a
        cp, ri, cv = O.csr2csc(a.rowptr, a.colind, a.val, a.n_cols)
        self._csr = (a.rowptr, a.colind, a.val)
        self._csc = (cp, ri, cv)
        self._F = _CpuSpmm.make(threads)
        g = torch.Generator().manual_seed(0)
        glorot = lambda i, o: ((torch.rand(i, o, generator=g) * 2 - 1) *
                               (6.0 / (i + o)) ** 0.5).requires_grad_(True)
        self._W1, self._W2 = glorot(500, 64), glorot(64, 3)
        self._b1 = torch.zeros(64, requires_grad=True)
        self._b2 = torch.zeros(3, requires_grad=True)
        deg_r = np.diff(a.rowptr).astype(np.float32)
        deg_c = np.diff(cp).astype(np.float32)
        self._in = torch.from_numpy(1 / np.sqrt(deg_r))[:, None]
        self._out = torch.from_numpy(1 / np.sqrt(deg_c))[:, None]
        self._x = torch.from_numpy(self.x)
        self._y = torch.from_numpy(self.y)
        self._t = torch.from_numpy(self.train)
        self._opt = torch.optim.Adam([dict(params=[self._W1, self._b1], weight_decay=5e-4),
                                      dict(params=[self._W2, self._b2], weight_decay=0)], lr=0.01)
        self._cpu = True

    def cpu_step(self, threads):
        import torch
        import torch.nn.functional as Fn
        self._cpu_setup(threads)
        conv = lambda x, W, b: self._F.apply((x @ W) * self._out, self._csr, self._csc) * self._in + b
        self._opt.zero_grad()
        h = Fn.dropout(Fn.relu(conv(self._x, self._W1, self._b1)), training=True)
        out = Fn.log_softmax(conv(h, self._W2, self._b2), dim=1)
        Fn.nll_loss(out[self._t], self._y[self._t]).backward()
        self._opt.step()
        return 1

    def cpu_aggregate(self, total, seconds, steps):
        return seconds / steps * 1e3

    def cpu_value(self, threads, budget_s):
        self.cpu_step(threads)
        t0 = time.perf_counter()
        n = 0
        while True:
            self.cpu_step(threads)
            n += 1
            if time.perf_counter() - t0 >= budget_s:
                break
        dt = time.perf_counter() - t0
        return dt / n * 1e3, f"{n} training epochs in {dt:.1f} s (torch CPU + restated csr_spmm_kernel)"

    def extra(self):
        """Plain path (library default kernels) vs the tuned path: epoch time and losses over
        20 epochs from the same initial weights."""
        import torch
        from armsparse_gb300 import gcn, tuner
        plain_ms = tuner.time_cuda(self.plain_step, reps=20, warmup=2, flush=False)
        tuned_ms = tuner.time_cuda(self.eager_step, reps=20, warmup=2, flush=False)
        graph_ms = tuner.time_cuda(self.step, reps=20, warmup=2, flush=False)
        torch.manual_seed(1)
        m1 = gcn.Net(500, 64, 3).to(self.dev)
        torch.manual_seed(1)
        m2 = gcn.Net(500, 64, 3).to(self.dev)
        o1, o2 = gcn.make_optimizer(m1), gcn.make_optimizer(m2)
        l1, l2 = [], []  # eager: the same dropout masks for both paths
        for _ in range(20):
            torch.manual_seed(_)
            l1.append(float(gcn.train_epoch(m1, o1, self.xd, self.g_plain, self.yd, self.td)))
            torch.manual_seed(_)
            l2.append(float(gcn.train_epoch(m2, o2, self.feats, self.g, self.yd, self.td)))
        return {"plain_ms_per_epoch": round(plain_ms, 4),
                "plain": "eager epochs, library-default kernels",
                "tuned_eager_ms_per_epoch": round(tuned_ms, 4),
                "tuned_graph_ms_per_epoch": round(graph_ms, 4),
                "speedup_tuned_graph_vs_plain": round(plain_ms / graph_ms, 2),
                "plan_layer1": self.plan[0], "plan_layer2": self.plan[1],
                "loss_max_abs_diff_20_epochs": max(abs(a - b) for a, b in zip(l1, l2))}


class GcnLarge(Workload):
    """One full-batch forward + backward of a 2-layer GCN on a large power-law graph (2.4M
    nodes, 62M directed edges, exponent 2.1, + self-loops), 100-dim features, hidden 256, 47
    classes, with the edge values trainable (their gradient is an SDDMM at the pattern).
    Tuned path: learned-selector kernels; features, layer activations and the SpMM/SDDMM
    operands in bf16 storage with fp32 accumulation (the dense products on bf16 tensor cores;
    the 47 class scores carried 48 wide, the loss over the 47); each layer's backward runs
    A^T dOut and the edge-value SDDMM in one pass over the CSC (dOut's rows gathered once);
    plain path (reported in `extra`): fp32 throughout, library-default (bit-exact) kernels."""
    name = "gcn_large"
    metric = "GCN forward+backward time (ms), 2.4M nodes / 62M edges, 100->256->47"
    unit = "ms/step"
    dtype = "bf16 storage, fp32 accumulate"
    kernel = "SpMM of layer 1 (N = 256)"
    profile = "gcn_large_spmm_n256"
    higher_is_better = False
    scale = 1.0  # --scale: nodes and edges x scale (a smaller graph of the same shape, for ncu)

    def __init__(self, seed=0):
        self.seed = seed
        self.n_nodes = int(2_400_000 * self.scale)
        self.n_edges = int(62_000_000 * self.scale)
        self.config = {"workload": "GCN 2-layer forward+backward with trainable edge values, "
                                   f"power-law graph {self.n_nodes:,} nodes, {self.n_edges:,} "
                                   "directed edges (exp. 2.1) + self-loops, 100->256->47",
                       "nodes": self.n_nodes, "edges": self.n_edges, "features": 100, "hidden": 256,
                       "classes": 47, "l2": "inputs far larger than L2 (B alone is 0.5-2.4 GB)"}

    def value(self, seconds, ws=1):
        return seconds * 1e3

    def flush_between_steps(self):
        return False

    def to_device(self, dev):
        import torch
        from armsparse_gb300 import gcn
        from armsparse_gb300 import synthetic as S
        self.dev = dev
        rp, ci, val = S.powerlaw_graph_device(self.n_nodes, self.n_edges, 2.1, self.seed, dev)
        n = self.n_nodes
        self.nnz = ci.numel()
        self.config["nnz"] = self.nnz
        # the first layer's SpMM: rowptr, colind + bf16 values, bf16 B read once, bf16 C written
        self.bytes = 4 * (n + 1) + 6 * self.nnz + 2 * n * 256 * 2
        deg = (rp[1:] - rp[:-1]).float()
        self.g = gcn.Graph(rp, ci, (val / deg.sqrt().repeat_interleave(rp[1:] - rp[:-1])).contiguous())
        self.g_plain = gcn.Graph(rp, ci, self.g.values)
        try:
            from armsparse_gb300 import selector
            self.g.selector = selector.Selector.load()
        except (OSError, ValueError):
            pass
        gen = torch.Generator(device=dev).manual_seed(self.seed + 1)
        self.x = torch.rand(n, 100, generator=gen, device=dev)
        # the features in bf16 storage, 100 columns padded to 104 (208-byte rows: 16-byte
        # aligned, so cuBLAS can pick its sm_103 kernels; the zero columns meet zero rows of W1)
        self.xb = torch.nn.functional.pad(self.x, (0, 4)).to(torch.bfloat16)
        self.y = torch.randint(0, 47, (n,), generator=gen, device=dev)
        torch.manual_seed(0)
        self.W1 = (torch.randn(100, 256, device=dev) * 0.1).requires_grad_(True)
        self.W2 = (torch.randn(256, 47, device=dev) * 0.1).requires_grad_(True)
        self.w = self.g.values.clone().requires_grad_(True)

    def _layer(self, g, x, W, dtype, plan, fuse=False, relu=False):
        from armsparse_gb300 import gcn
        colptr, rowind, vcsc = g.csc
        h = x @ W.to(dtype)  # bf16 layers: a bf16 tensor-core GEMM with fp32 accumulation
        return gcn.SPMMFunction.apply(g.rowptr, g.colind, colptr, rowind, h, self.w, vcsc, plan,
                                      g.csc_pos if fuse else None, relu)

    def _step(self, g, dtype, tuned):
        import torch
        import torch.nn.functional as Fn
        from armsparse_gb300 import gcn
        p1 = g.plan(256, dtype, fused=True) if tuned else None
        x = self.xb if dtype == torch.bfloat16 else self.x
        W1 = Fn.pad(self.W1, (0, 0, 0, 4)) if dtype == torch.bfloat16 else self.W1
        # tuned: the ReLU is applied in the SpMM's store
        h = self._layer(g, x, W1, dtype, p1, tuned, True) if tuned else \
            Fn.relu(self._layer(g, x, W1, dtype, p1))
        if tuned:
            # the 47 class scores are carried 48 wide (one zero weight column): rows of 96
            # bytes, 16-byte aligned, so the SpMMs load whole vectors; the loss (log_softmax
            # and the mean NLL in one kernel each way) reads the 47
            p2 = g.plan(48, dtype, fused=True)
            out = self._layer(g, h, Fn.pad(self.W2, (0, 1)), dtype, p2, True)
            loss = gcn.SoftmaxXent.apply(out, self.y, 47)
        else:
            out = self._layer(g, h, self.W2, dtype, None).float()
            # the model's log_softmax then the mean NLL (gcn_custom.py's loss); nll_mean in
            # place of F.nll_loss, whose one-block reduction takes milliseconds on 2.4M rows
            loss = gcn.nll_mean(Fn.log_softmax(out, dim=1), self.y)
        loss.backward()
        self.W1.grad = self.W2.grad = self.w.grad = None
        return loss.detach()

    def step(self):
        import torch
        self.loss = self._step(self.g, torch.bfloat16, True)

    def roofline_ms(self, step_ms):
        import torch
        import armsparse_gb300 as A
        from armsparse_gb300 import tuner
        # the first layer's forward SpMM as the step runs it: bf16 B, bf16 C with the ReLU
        B = torch.rand(self.g.n_rows, 256, device=self.dev).to(torch.bfloat16)
        C = torch.empty(self.g.n_rows, 256, device=self.dev, dtype=torch.bfloat16)
        v = self.g.plan(256, torch.bfloat16)[0]
        vb = self.g.values.to(torch.bfloat16)
        return tuner.time_cuda(lambda: A.spmm(self.g.rowptr, self.g.colind, vb, B, C=C,
                                              variant=v, out_dtype=torch.bfloat16, relu=True),
                               reps=5, flush=False)

    def e2e_setup(self):
        self.hx = self.xb.cpu().pin_memory()  # the bf16 features the tuned step reads
        self.h2d = self.hx.numel() * 2
        self.d2h = 4

    def e2e_step(self):
        self.xb.copy_(self.hx, non_blocking=True)
        self.step()
        float(self.loss)

    def cpu_step(self, threads):
        raise NotImplementedError("no CPU arm at this size (hours on the host cores)")

    def cpu_value(self, threads, budget_s):
        return None, "not run: the reference's CPU path at 62M edges takes hours"

    def extra(self):
        import torch
        from armsparse_gb300 import tuner
        plain_ms = tuner.time_cuda(lambda: self._step(self.g_plain, torch.float32, False),
                                   reps=3, warmup=1, flush=False)
        tuned_ms = tuner.time_cuda(lambda: self._step(self.g, torch.bfloat16, True), reps=3,
                                   warmup=1, flush=False)
        return {"plain_fp32_ms": round(plain_ms, 3), "tuned_bf16_ms": round(tuned_ms, 3),
                "speedup": round(plain_ms / tuned_ms, 3),
                "plan_256": self.g.plan(256, torch.bfloat16, fused=True),
                "plan_48": self.g.plan(48, torch.bfloat16, fused=True)}


class SpmvF32(_Generic):
    """y = A*x on the SpMV driver's matrix (4096 x 4096, density 0.01, 167,772 entries): a
    1.4 MB problem, bound by launch latency; `extra` reports the per-call time when 100 calls
    are replayed from a CUDA graph, and the 1x4-blocked layout of the reference."""
    name = "spmv"
    metric = "SpMV GB/s (algorithmic bytes), CSR fp32"
    unit = "GB/s"
    dtype = "f32"
    kernel = "spmv_csr"
    profile = "spmv_csr_4096_d001"

    def __init__(self, seed=0):
        from armsparse_gb300 import synthetic as S
        self.a = S.spmm_4096_d001(seed)
        self.x = S.dense_uniform(4096, seed + 1)
        nnz = self.a.nnz
        self.bytes = 4 * 4097 + 8 * nnz + 4 * 4096 + 4 * 4096
        self.config = {"workload": "spmv_csr y=A*x, A 4096x4096 uniform density 0.01 (167,772 nnz)",
                       "M": 4096, "K": 4096, "nnz": nnz, "alg_bytes_per_step": self.bytes,
                       "l2": "flushed between steps (256 MiB write, outside the timed events)"}

    def to_device(self, dev):
        import torch
        self.dev = dev
        t = lambda a: torch.from_numpy(a).to(dev)
        self.rp, self.ci, self.v, self.xd = t(self.a.rowptr), t(self.a.colind), t(self.a.val), t(self.x)
        self.y = torch.empty(4096, device=dev)

    def inputs(self):
        return {"rp": self.rp, "ci": self.ci, "v": self.v, "x": self.xd}

    def output(self):
        return self.y

    def step(self):
        import armsparse_gb300 as A
        A.spmv(self.rp, self.ci, self.v, self.xd, y=self.y)

    def cpu_step(self, threads, rows=None):
        from oracle import oracle as O
        if not hasattr(self, "_v4"):
            self._v4 = O.csr_to_vcsr4(self.a.rowptr, self.a.colind, self.a.val)
        vr, vc, vv = self._v4
        O.spmv_vcsr4_f32(vr, vc, vv, self.x, threads=threads)
        return self.bytes

    def extra(self):
        import torch
        import armsparse_gb300 as A
        from oracle import oracle as O
        vr, vc, vv = O.csr_to_vcsr4(self.a.rowptr, self.a.colind, self.a.val)
        t = lambda a: torch.from_numpy(a).to(self.dev)
        vrd, vcd, vvd = t(vr), t(vc), t(vv)
        yv = torch.empty(4096, device=self.dev)
        s = torch.cuda.Stream(self.dev)
        out = {}
        for name, fn in (("csr", self.step),
                         ("vcsr4", lambda: A.spmv_vcsr4(vrd, vcd, vvd, self.xd, y=yv))):
            with torch.cuda.stream(s):
                fn()
                s.synchronize()
                g = torch.cuda.CUDAGraph()
                with torch.cuda.graph(g, stream=s):
                    for _ in range(100):
                        fn()
            g.replay()
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(10):
                g.replay()
            e1.record()
            e1.synchronize()
            us = e0.elapsed_time(e1) * 1e3 / 1000
            out[f"{name}_graph_us_per_call"] = round(us, 3)
            out[f"{name}_graph_gbs"] = round(self.bytes / (us * 1e-6) / 1e9, 1)
        return out


class Csr2Csc(_Generic):
    """CSR -> CSC of a power-law matrix with 1M rows and ~20M entries (3 radix passes)."""
    name = "csr2csc"
    metric = "CSR->CSC GB/s (algorithmic bytes)"
    unit = "GB/s"
    dtype = "int32 + f32 payload"
    kernel = "radix_scatter"
    profile = "csr2csc_powerlaw_1m_20m"
    cpu_threads_used = 1

    def __init__(self, seed=0):
        from armsparse_gb300 import synthetic as S
        self.a = S.powerlaw_csr(1_000_000, 2.1, 20.0, seed=seed)
        n, nnz = self.a.n_rows, self.a.nnz
        self.bytes = 4 * (n + 1) + 8 * nnz + 4 * (n + 1) + 8 * nnz
        self.config = {"workload": "csr2csc of a power-law matrix 1M x 1M (exp. 2.1, mean 20 "
                                   "entries/row), fp32 values", "n": n, "nnz": nnz,
                       "alg_bytes_per_step": self.bytes,
                       "l2": "flushed between steps (256 MiB write, outside the timed events)"}

    def to_device(self, dev):
        import torch
        t = lambda a: torch.from_numpy(a).to(dev)
        self.rp, self.ci, self.v = t(self.a.rowptr), t(self.a.colind), t(self.a.val)
        self.res = None

    def inputs(self):
        return {"rp": self.rp, "ci": self.ci, "v": self.v}

    def output(self):
        return self.res[1] if self.res is not None else self.ci

    def step(self):
        import armsparse_gb300 as A
        self.res = A.csr2csc(self.rp, self.ci, self.v, self.a.n_cols)

    def cpu_step(self, threads, rows=None):
        from oracle import oracle as O
        O.csr2csc(self.a.rowptr, self.a.colind, self.a.val, self.a.n_cols)
        return self.bytes

    def cpu_value(self, threads, budget_s):
        v, sample = Workload.cpu_value(self, threads, budget_s)
        return v, sample + " (single-threaded counting transpose)"


WORKLOADS = {c.name: c for c in [SpmmF32, SpmmBf16, SpmmPowerlaw, SpgemmDense, SddmmTc, SddmmF32, GcnEpoch, GcnLarge, SpmvF32,
                                 Csr2Csc]}



# ------------------------------------------------------------------------------------------
# Measurement helpers
# ------------------------------------------------------------------------------------------
def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d.get("hbm_gbs", FALLBACK_HBM_GBS), d.get("bf16_tflops", FALLBACK_BF16_TFLOPS), "measured"
    return FALLBACK_HBM_GBS, FALLBACK_BF16_TFLOPS, "fallback"


def profiled_traffic(profile: str):
    """dram bytes per launch from the committed ncu summary (profiles/<profile>.md), if any."""
    path = os.path.join(ROOT, "profiles", profile + ".md")
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.strip().startswith("traffic_bytes_per_launch:"):
            try:
                return int(line.split(":", 1)[1].strip().split()[0])
            except ValueError:
                return None
    return None


class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "50"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, ValueError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        self.out = ""
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
                self.out, _ = self.proc.communicate()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in (self.out or "").strip().splitlines():
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


# ------------------------------------------------------------------------------------------
# Arms
# ------------------------------------------------------------------------------------------
def run_reference(args, wl_cls):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    from oracle import oracle as O
    O.build()
    wl = wl_cls()
    threads = os.cpu_count() or 1
    for _ in range(args.warmup):
        wl.cpu_step(threads)
    t0 = time.perf_counter()
    total = 0
    for _ in range(args.steps):
        total += wl.cpu_step(threads)
    dt = time.perf_counter() - t0
    value = wl.cpu_aggregate(total, dt, args.steps) if hasattr(wl, "cpu_aggregate") else total / dt / 1e9
    line = {
        "impl": "reference", "metric": wl.metric, "value": round(value, 3), "unit": wl.unit,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(dt / args.steps * 1e3, 3), "higher_is_better": wl.higher_is_better,
        "scaling": "weak", "vs_baseline": None, "dtype": wl.dtype, "data": "synthetic (seeded)",
        "config": dict(wl.config, parallelism=f"replicas x{ws}"),
        "cpu_baseline": {"value": round(value, 3), "unit": wl.unit, "cores": threads,
                         "kind": "port",
                         "sample": f"the whole workload per step, {args.steps} steps, "
                                   "oracle restatement of the reference kernel, OpenMP"},
        "e2e": {"value": round(value, 3), "unit": wl.unit, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    gpu = reference_cuda(args, wl)
    if gpu is not None:
        line["reference_cuda"] = gpu
    print(json.dumps(line), flush=True)
    return 0


def reference_cuda(args, wl):
    """The reference's own CUDA kernels for this workload on this machine's GPU (where the
    workload has them and their cubins were built): K timed steps after W warm-ups, L2
    flushed between steps, CUDA events; None otherwise."""
    if not hasattr(wl, "ref_cuda_step"):
        return None
    try:
        import torch
        from oracle import ref_gpu
        if not (torch.cuda.is_available() and ref_gpu.available()):
            return {"unavailable": "no GPU or reference cubins not built"}
        from armsparse_gb300 import tuner
        dev = torch.device("cuda", 0)
        wl.to_device(dev)
        ms = tuner.time_cuda(wl.ref_cuda_step, reps=max(3, args.steps), warmup=max(3, args.warmup))
        return {"kernel": wl.ref_cuda_kernel, "ms_per_step": round(ms, 5),
                "value": round(wl.value(ms * 1e-3), 3), "unit": wl.unit,
                "l2": "flushed between steps"}
    except Exception as e:  # noqa: BLE001 -- the CPU line stands without it
        return {"unavailable": repr(e)[:200]}


def cpu_baseline(wl, budget_s=10.0):
    threads = os.cpu_count() or 1
    v, sample = wl.cpu_value(threads, budget_s)
    cores = getattr(wl, "cpu_threads_used", threads)
    return {"value": None if v is None else round(v, 3), "unit": wl.unit, "cores": cores,
            "kind": "port",
            "sample": sample + " (oracle restatement of the reference kernel, OpenMP over all "
                               "host cores)"}


def run_ours(args, wl_cls):
    import torch
    import torch.distributed as dist
    import armsparse_gb300 as A
    from armsparse_gb300 import _native as N

    ws, rank, local = dist_env()
    if ws > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    wl = wl_cls()
    wl.to_device(dev)
    flush = torch.empty(L2_FLUSH_BYTES, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)

    for _ in range(max(args.warmup, 3)):
        if wl.flush_between_steps():
            flush.fill_(1)
        wl.step()
    torch.cuda.synchronize(dev)

    def barrier():
        if ws > 1:
            dist.barrier()
        torch.cuda.synchronize(dev)

    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(args.steps)]
    l0 = N.total_launches()
    barrier()
    nvtx = _nvtx()
    with ClockSampler(local) as clk:
        nvtx.range_push("timed")  # lets a profiler select the timed steps (ncu --nvtx-include)
        t0 = time.perf_counter()
        for i in range(args.steps):
            if wl.flush_between_steps():
                flush.fill_(i & 0xFF)
            evs[i][0].record(stream)
            wl.step()
            evs[i][1].record(stream)
        torch.cuda.synchronize(dev)
        wall = time.perf_counter() - t0
        nvtx.range_pop()
    barrier()
    launches = N.total_launches() - l0
    if hasattr(wl, "launches_per_replay"):  # steps replayed from a CUDA graph
        launches += args.steps * wl.launches_per_replay()
    times = [s.elapsed_time(e) for s, e in evs]  # ms
    kernel_ms = sum(times) / len(times)
    if ws > 1:
        t = torch.tensor([kernel_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        kernel_ms = float(t.item())
    value = wl.value(kernel_ms * 1e-3, ws)

    # end to end through the reference-facing host call
    wl.e2e_setup()
    for _ in range(2):
        wl.e2e_step()
    barrier()
    e2e_steps = max(3, min(args.steps, 10))
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        wl.e2e_step()
    e2e_s = (time.perf_counter() - t0) / e2e_steps
    if ws > 1:
        t = torch.tensor([e2e_s], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_s = float(t.item())
    e2e_value = wl.value(e2e_s, ws)

    hbm, bf16, src = measured_peaks()
    roof = wl.roofline(wl.roofline_ms(kernel_ms) if hasattr(wl, "roofline_ms") else kernel_ms,
                       hbm, bf16, src)
    line = {
        "metric": wl.metric, "value": round(value, 3), "unit": wl.unit, "n_gpus": ws,
        "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": round(kernel_ms, 5),
        "higher_is_better": wl.higher_is_better, "scaling": "weak", "vs_baseline": None,
        "dtype": wl.dtype,
        "data": "synthetic (seeded)", "config": dict(wl.config, parallelism=f"replicas x{ws}"),
        "roofline": roof,
        "e2e": {"value": round(e2e_value, 3), "unit": wl.unit,
                "h2d_bytes_per_step": wl.h2d, "d2h_bytes_per_step": wl.d2h,
                "ms_per_step": round(e2e_s * 1e3, 3),
                "api": getattr(wl, "e2e_api", "armsparse_gb300 Python API, pinned host buffers")},
        "gpu_launches": launches,
        "clocks": clk.summary(),
        "wall_s_timed_region": round(wall, 4),
    }
    if hasattr(wl, "extra") and not args.no_extra:
        line["extra"] = wl.extra()
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(wl, args.cpu_seconds)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        dist.destroy_process_group()
    return 0


def _nvtx():
    """torch's NVTX ranges, or a stand-in that does nothing where the build lacks them."""
    import torch

    class _Off:
        @staticmethod
        def range_push(_):
            pass

        @staticmethod
        def range_pop():
            pass
    try:
        torch.cuda.nvtx.range_push("probe")
        torch.cuda.nvtx.range_pop()
        return torch.cuda.nvtx
    except Exception:  # noqa: BLE001 -- any failure means no ranges
        return _Off


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="spmm_f32")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-extra", action="store_true",
                    help="skip the extra figures (profiler runs of the headline step alone)")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--tc-variant", type=int, default=0,
                    help="tensor-core SDDMM kernel variant (0 = library choice)")
    ap.add_argument("--scale", type=float, default=1.0,
                    help="gcn_large only: nodes and edges times this (a smaller graph of the "
                         "same shape, for profiler captures); the headline uses 1")
    args = ap.parse_args()
    wl_cls = WORKLOADS[args.workload]
    if hasattr(wl_cls, "variant"):
        wl_cls.variant = args.tc_variant
    if hasattr(wl_cls, "scale"):
        wl_cls.scale = args.scale
    if args.impl == "reference":
        return run_reference(args, wl_cls)
    return run_ours(args, wl_cls)


if __name__ == "__main__":
    sys.exit(main())
