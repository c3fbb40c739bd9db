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
class SpmmF32:
    name = "spmm_f32"
    metric = "SpMM GB/s (algorithmic bytes) and % HBM roofline"
    unit = "GB/s"
    dtype = "f32"
    kernel = "spmm_rowsplit"
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


class _Generic:
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


class SddmmTc(_Generic):
    name = "sddmm_tc"
    metric = "SDDMM GB/s (algorithmic bytes), tensor-core split-bf16 path"
    unit = "GB/s"
    dtype = "bf16x3 (fp32 in/out, fp32 accumulate)"
    kernel = "sddmm_tc_kernel"
    profile = "sddmm_tc_kernel_4096x4096x4096_d01"
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

    def step(self):
        import armsparse_gb300 as A
        A.sddmm(self.rp, self.ci, self.Xd, self.Yd, aval=self.v, out=self.out,
                tensor_cores=self.tensor_cores)

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
    kernel = "sddmm_f32_lane"
    profile = "sddmm_f32_lane_4096x4096x4096_d01"
    bound = "hbm"
    tensor_cores = False


WORKLOADS = {c.name: c for c in [SpmmF32, SddmmTc, SddmmF32]}



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
    value = total / dt / 1e9
    line = {
        "impl": "reference", "metric": wl.metric, "value": round(value, 3), "unit": wl.unit,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(dt / args.steps * 1e3, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": wl.dtype, "data": "synthetic (seeded)",
        "config": wl.config,
        "cpu_baseline": {"value": round(value, 3), "unit": wl.unit, "cores": threads,
                         "kind": "port",
                         "sample": f"the whole workload per step, {args.steps} steps, "
                                   "oracle restatement of the reference kernel, OpenMP"},
        "e2e": {"value": round(value, 3), "unit": wl.unit, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def cpu_baseline(wl, budget_s=10.0):
    threads = os.cpu_count() or 1
    wl.cpu_step(threads)  # warm
    t0 = time.perf_counter()
    total, calls = 0, 0
    while True:
        total += wl.cpu_step(threads)
        calls += 1
        if time.perf_counter() - t0 >= budget_s:
            break
    dt = time.perf_counter() - t0
    return {"value": round(total / dt / 1e9, 3), "unit": wl.unit, "cores": threads,
            "kind": "port",
            "sample": f"{calls} full calls in {dt:.1f} s (oracle restatement of the reference "
                      "kernel, OpenMP over all host cores)"}


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
    with ClockSampler(local) as clk:
        t0 = time.perf_counter()
        for i in range(args.steps):
            flush.fill_(i & 0xFF)
            evs[i][0].record(stream)
            wl.step()
            evs[i][1].record(stream)
        torch.cuda.synchronize(dev)
        wall = time.perf_counter() - t0
    barrier()
    launches = N.total_launches() - l0
    times = [s.elapsed_time(e) for s, e in evs]  # ms
    kernel_ms = sum(times) / len(times)
    if ws > 1:
        t = torch.tensor([kernel_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        kernel_ms = float(t.item())
    value = ws * wl.bytes / (kernel_ms * 1e-3) / 1e9

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
    e2e_value = ws * wl.bytes / e2e_s / 1e9

    hbm, bf16, src = measured_peaks()
    if getattr(wl, "bound", "hbm") == "tensor":
        achieved = wl.flops / (kernel_ms * 1e-3) / 1e12
        roof = {"bound": "tensor", "achieved": round(achieved, 3), "peak": bf16,
                "unit": "TFLOP/s", "frac": round(achieved / bf16, 5),
                "traffic": profiled_traffic(wl.profile), "peak_source": src, "kernel": wl.kernel,
                "achieved_is": "algorithmic (sampled) flops 2*nnz*K per step",
                "executed_tflops": round(wl.exec_flops / (kernel_ms * 1e-3) / 1e12, 2),
                "executed_frac": round(wl.exec_flops / (kernel_ms * 1e-3) / 1e12 / bf16, 4)}
    else:
        achieved = wl.bytes / (kernel_ms * 1e-3) / 1e9
        roof = {"bound": "hbm", "achieved": round(achieved, 2), "peak": hbm, "unit": "GB/s",
                "frac": round(achieved / hbm, 4), "traffic": profiled_traffic(wl.profile),
                "peak_source": src, "kernel": wl.kernel}
    line = {
        "metric": wl.metric, "value": round(value, 3), "unit": wl.unit, "n_gpus": ws,
        "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": round(kernel_ms, 5),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": wl.dtype,
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
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(wl, args.cpu_seconds)
    if rank == 0:
        print(json.dumps(line), flush=True)
    if ws > 1:
        dist.destroy_process_group()
    return 0


def main():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="spmm_f32")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    args = ap.parse_args()
    wl_cls = WORKLOADS[args.workload]
    if args.impl == "reference":
        return run_reference(args, wl_cls)
    return run_ours(args, wl_cls)


if __name__ == "__main__":
    sys.exit(main())
