"""Learned SpMM kernel selector: a small MLP over cheap matrix features.

The reference picks a kernel only by the dense width (k < 32 / k < 64 / else,
gcn/pytorch-custom/spmm_kernel.cu:437-457). Here:

1. ``sweep`` runs the exhaustive autotuner (tuner.autotune_spmm) over seeded synthetic
   matrices -- power-law and banded, n from 1k to 1M rows, dense width N in {16..256},
   fp32 and bf16 -- on a fixed candidate set of kernel variants, and records (features,
   time of every candidate);
2. ``train`` fits an MLP (features -> one score per candidate) with soft targets
   t_v ~ exp(-(time_v / best - 1) / tau), on the GPU, with this project's own kernels
   (include/armsparse_mlp.h: linear forward/backward, softmax cross entropy, Adam);
3. ``Selector.choose`` evaluates the network on the host (a few thousand multiply-adds) and
   returns the variant id; the autotuner stays the fallback and the yardstick the picks are
   scored against (``evaluate`` reports picked time / best time).

Model files are JSON (weights, feature normalisation, candidate names, format version).
"""
from __future__ import annotations

import ctypes
import json
import math
import os

import numpy as np
import torch

from . import _native as N
from . import sparse as S
from . import tuner

FORMAT = "armsparse-selector-1"
DEFAULT_MODEL = os.path.join(os.path.dirname(os.path.abspath(__file__)), "selector_model.json")

# Candidate variants (names exist for both dtypes). Chosen to span the three families: the
# register row-split kernels at several lane-group sizes, vector widths and unroll depths,
# the shared-memory-staged kernels, and the entry-balanced kernels for skewed rows.
CANDIDATES = [
    "rowsplit_v8_g32_c4_u4", "rowsplit_v16_g32_c2_u4", "rowsplit_v16_g32_c1_u4",
    "rowsplit_v8_g32_c2_u4", "rowsplit_v16_g16_c1_u4", "rowsplit_v16_g8_c1_u4",
    "rowsplit_v4_g32_c2_u8", "rowsplit_v4_g32_c1_u8", "rowsplit_v4_g16_c2_u8",
    "rowsplit_v8_g32_c2_u8", "rowsplit_v4_g8_c1_u8",
    "bulk_lb32_s4",
    "nnzsplit_v4_g32_c1_ch128", "nnzsplit_v4_g32_c2_ch128", "nnzsplit_v16_g32_c1_ch128",
    "nnzsplit_v16_g16_c1_ch128", "nnzsplit_v16_g32_c1_ch1024", "nnzsplit_v4_g32_c2_ch1024",
    "nnzsplit_v16_g32_c2_ch1024", "nnzsplit_v4_g32_c1_ch1024",
    "rowsplit_v16_g32_c2_u8", "nnzsplit_v16_g32_c1_ch256_u8", "nnzsplit_v4_g32_c2_ch256_u8",
    "nnzsplit_v16_g32_c1_ch1024_u8", "nnzsplit_v4_g32_c2_ch1024_u8",
    "nnzsplit_v4_g32_c1_ch32", "nnzsplit_v4_g32_c2_ch32", "nnzsplit_v16_g32_c1_ch32",
    "nnzme_v8_g16_ch1024", "nnzme_v16_g8_ch1024", "nnzme_v16_g16_ch1024",
]


def is_exact(name: str) -> bool:
    """Whether a variant's outputs are each the CSR-order fused chain (bit-identical to the
    reference's rowBaseSpmm3 and to the library default): the row-split and bulk-copy
    families. The entry-balanced ones reorder the sums of rows that cross a chunk."""
    return name.startswith(("rowsplit", "bulk"))


def variant_ids(names, dtype):
    table = {n: i + 1 for i, n in enumerate(S.spmm_variants(dtype))}
    return [table[n] for n in names]


# ------------------------------------------------------------------------------------------
# Sweep
# ------------------------------------------------------------------------------------------
def sweep_configs(n_matrices=300, seed=0, max_nnz=8_000_000):
    """Seeded matrix descriptions: half power-law (exponent U[1.8, 2.5], mean nnz/row
    U[2, 200]), half banded (bandwidth U[3, 64]); n log-uniform in [1e3, 1e6]; N in
    {16, 32, 64, 128, 256}; dtype fp32 or bf16. The mean row length is reduced where needed so
    that nnz stays under max_nnz (sweep time)."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n_matrices):
        n = int(10 ** rng.uniform(3, 6))
        kind = "powerlaw" if i % 2 == 0 else "banded"
        cfg = {"id": i, "kind": kind, "n": n, "N": int(rng.choice([16, 32, 64, 128, 256])),
               "dtype": "bf16" if rng.random() < 0.5 else "fp32", "seed": 1000 + i}
        if kind == "powerlaw":
            cfg["exponent"] = float(rng.uniform(1.8, 2.5))
            cfg["mean"] = float(min(rng.uniform(2, 200), max_nnz / n))
        else:
            cfg["bandwidth"] = int(min(rng.integers(3, 65), max(3, max_nnz // n)))
        out.append(cfg)
    return out


def make_matrix(cfg, device):
    from . import synthetic as syn
    if cfg["kind"] == "powerlaw":
        return syn.powerlaw_csr_device(cfg["n"], cfg["exponent"], cfg["mean"], cfg["seed"], device)
    return syn.banded_csr_device(cfg["n"], cfg["bandwidth"], cfg["seed"], device)


def sweep(configs, device=None, reps=3, log=None):
    """Autotune every config over CANDIDATES; returns a list of records."""
    device = device or torch.device("cuda", 0)
    records = []
    for cfg in configs:
        rowptr, colind, val = make_matrix(cfg, device)
        dt = torch.bfloat16 if cfg["dtype"] == "bf16" else torch.float32
        g = torch.Generator(device=device).manual_seed(cfg["seed"] + 7)
        B = (torch.rand(cfg["n"], cfg["N"], generator=g, device=device) * 2 - 1).to(dt)
        ids = variant_ids(CANDIDATES, dt)
        t = tuner.autotune_spmm(rowptr, colind, val.to(dt), B, variants=ids, reps=reps,
                                max_ratio=4.0)
        feats = tuner.features(rowptr.cpu().numpy(), cfg["n"], cfg["N"], dt == torch.bfloat16)
        rec = {"cfg": cfg, "features": feats.tolist(), "nnz": int(colind.numel()),
               "times_ms": [x.ms for x in t]}
        records.append(rec)
        if log:
            ok = [x for x in t if x.ms is not None]
            b = min(ok, key=lambda x: x.ms)
            log(f"{cfg['id']:4d} {cfg['kind']:8s} n={cfg['n']:8d} nnz={rec['nnz']:9d} N={cfg['N']:3d} "
                f"{cfg['dtype']} best={b.name} {b.ms * 1e3:.1f}us")
        del rowptr, colind, val, B
    return records


# ------------------------------------------------------------------------------------------
# Network (trained with the project's own kernels)
# ------------------------------------------------------------------------------------------
def soft_targets(times, tau=0.1):
    t = np.array([np.inf if x is None else x for x in times], np.float64)
    best = t.min()
    s = np.where(np.isfinite(t), np.exp(-(t / best - 1.0) / tau), 0.0)
    return s / s.sum()


class _Lib:
    def __init__(self, device):
        self.L = N.load()
        self.ctx = N.context(device.index)
        self.stream = torch.cuda.current_stream(device).cuda_stream

    def call(self, name, *args):
        N.check(getattr(self.L, name)(self.ctx.handle, *args, self.stream), name)


class MLP:
    """features -> hidden -> hidden -> candidates, ReLU, on the GPU."""

    def __init__(self, n_in, n_out, hidden=64, seed=0, device=None):
        self.device = device or torch.device("cuda", 0)
        g = torch.Generator().manual_seed(seed)
        dims = [n_in, hidden, hidden, n_out]
        self.params = []
        for i in range(3):
            a = math.sqrt(6.0 / (dims[i] + dims[i + 1]))
            W = (torch.rand(dims[i + 1], dims[i], generator=g) * 2 - 1) * a
            self.params += [W.to(self.device).contiguous(), torch.zeros(dims[i + 1], device=self.device)]
        self.m = [torch.zeros_like(p) for p in self.params]
        self.v = [torch.zeros_like(p) for p in self.params]
        self.step = 0
        self.lib = _Lib(self.device)

    def forward(self, X):
        """Returns (logits, activations) for backward."""
        acts = [X]
        h = X
        for i in range(3):
            W, b = self.params[2 * i], self.params[2 * i + 1]
            out = torch.empty(h.shape[0], W.shape[0], device=self.device)
            self.lib.call("as_mlp_linear_fwd", h.shape[0], W.shape[1], W.shape[0], h.data_ptr(),
                          W.data_ptr(), b.data_ptr(), out.data_ptr(), int(i < 2))
            acts.append(out)
            h = out
        return h, acts

    def loss_and_grads(self, X, T):
        Bn = X.shape[0]
        Z, acts = self.forward(X)
        loss = torch.empty(Bn, device=self.device)
        dZ = torch.empty_like(Z)
        self.lib.call("as_mlp_softmax_xent", Bn, Z.shape[1], Z.data_ptr(), T.data_ptr(),
                      loss.data_ptr(), dZ.data_ptr(), ctypes.c_float(1.0 / Bn))
        grads = [None] * 6
        d = dZ
        for i in (2, 1, 0):
            W = self.params[2 * i]
            x_in = acts[i]
            dW = torch.empty_like(W)
            db = torch.empty(W.shape[0], device=self.device)
            dX = torch.empty_like(x_in) if i > 0 else None
            self.lib.call("as_mlp_linear_bwd", Bn, W.shape[1], W.shape[0], d.data_ptr(),
                          x_in.data_ptr(), W.data_ptr(), x_in.data_ptr() if i > 0 else None,
                          dX.data_ptr() if dX is not None else None, dW.data_ptr(), db.data_ptr())
            grads[2 * i], grads[2 * i + 1] = dW, db
            d = dX
        return loss.mean(), grads

    def adam_step(self, grads, lr=3e-3, wd=1e-4):
        self.step += 1
        for p, g, m, v in zip(self.params, grads, self.m, self.v):
            self.lib.call("as_mlp_adam", p.numel(), p.data_ptr(), g.data_ptr(), m.data_ptr(),
                          v.data_ptr(), ctypes.c_float(lr), ctypes.c_float(0.9),
                          ctypes.c_float(0.999), ctypes.c_float(1e-8), ctypes.c_float(wd),
                          self.step)

    def host_weights(self):
        return [p.detach().cpu().numpy().astype(np.float64) for p in self.params]


def train(records, epochs=3000, hidden=64, lr=3e-3, seed=0, tau=0.1, device=None, log=None,
          candidates=None, fmt=FORMAT):
    """Fit the selector on sweep records (full batch); returns a model dict. ``candidates``
    (default: the SpMM CANDIDATES) names the network's outputs, one per timed path."""
    candidates = candidates or CANDIDATES
    device = device or torch.device("cuda", 0)
    X = np.array([r["features"] for r in records], np.float64)
    mu, sd = X.mean(axis=0), X.std(axis=0) + 1e-6
    Xn = torch.tensor((X - mu) / sd, dtype=torch.float32, device=device)
    T = torch.tensor(np.stack([soft_targets(r["times_ms"], tau) for r in records]),
                     dtype=torch.float32, device=device)
    net = MLP(X.shape[1], len(candidates), hidden, seed, device)
    for ep in range(epochs):
        loss, grads = net.loss_and_grads(Xn, T)
        net.adam_step(grads, lr=lr)
        if log and (ep % 500 == 0 or ep == epochs - 1):
            log(f"epoch {ep:5d} loss {float(loss):.4f}")
    W = net.host_weights()
    return {"format": fmt, "candidates": list(candidates), "mu": mu.tolist(), "sd": sd.tolist(),
            "weights": [w.tolist() for w in W], "hidden": hidden, "tau": tau,
            "n_train": len(records)}


def host_forward(model, feats):
    x = (np.asarray(feats, np.float64) - np.array(model["mu"])) / np.array(model["sd"])
    W = [np.array(w, np.float64) for w in model["weights"]]
    h = x
    for i in range(3):
        h = h @ W[2 * i].T + W[2 * i + 1]
        if i < 2:
            h = np.maximum(h, 0.0)
    return h


def evaluate(model, records):
    """Mean and worst (picked time / best time) over records, and the same for the fixed
    width rule the reference uses (its dispatch on N)."""
    picked, fixed = [], []
    for r in records:
        t = np.array([np.inf if x is None else x for x in r["times_ms"]])
        best = t.min()
        scores = host_forward(model, r["features"])
        scores = np.where(np.isfinite(t), scores, -np.inf)
        picked.append(t[int(np.argmax(scores))] / best)
        fixed.append(t[CANDIDATES.index(width_rule(r["cfg"]["N"]))] / best
                     if np.isfinite(t[CANDIDATES.index(width_rule(r["cfg"]["N"]))]) else np.nan)
    picked, fixed = np.array(picked), np.array(fixed)
    return {"mlp_mean": float(np.mean(picked)), "mlp_geomean": float(np.exp(np.mean(np.log(picked)))),
            "mlp_worst": float(np.max(picked)),
            "rule_mean": float(np.nanmean(fixed)), "rule_geomean": float(np.exp(np.nanmean(np.log(fixed)))),
            "n": len(records)}


def width_rule(N):
    """The method without the network: a static choice by the dense width only -- the
    reference's own selection logic (gcn/pytorch-custom/spmm_kernel.cu:437-457: k < 32,
    k < 64, else) mapped to this build's best kernel for each width class on uniform rows."""
    if N < 32:
        return "rowsplit_v4_g16_c2_u8"
    if N < 64:
        return "rowsplit_v4_g32_c1_u8"
    return "rowsplit_v4_g32_c2_u8" if N < 512 else "rowsplit_v8_g32_c4_u4"


def narrower_feasible(names, name, N, dtype):
    """The variant with `name`'s family, lane group, vectors per lane and unroll/chunk but the
    narrowest vector width that can run width N, or 0."""
    parts = name.split("_")
    if parts[0] not in ("rowsplit", "nnzsplit"):
        return 0
    for vb in (4, 2):
        alt = "_".join([parts[0], f"v{vb}"] + parts[2:])
        if alt in names:
            vid = names.index(alt) + 1
            if S.spmm_variant_supported(vid, N, dtype):
                return vid
    return 0


class Selector:
    def __init__(self, model: dict):
        if model.get("format") != FORMAT:
            raise ValueError("unknown selector model format")
        self.model = model
        self._cache = {}

    @classmethod
    def load(cls, path: str = DEFAULT_MODEL) -> "Selector":
        with open(path) as f:
            return cls(json.load(f))

    def save(self, path: str) -> None:
        with open(path, "w") as f:
            json.dump(self.model, f)

    def choose(self, rowptr, n_cols: int, N: int, dtype=torch.float32, key=None,
               exact: bool = False) -> int:
        """Variant id for an SpMM with this matrix and dense width (cached by ``key``). With
        ``exact`` only kernels whose every output is the reference's CSR-order chain are
        considered (the row-split and bulk families: bit-identical to the library default)."""
        if key is not None and (key, N, dtype, exact) in self._cache:
            return self._cache[(key, N, dtype, exact)]
        rp = rowptr.cpu().numpy() if isinstance(rowptr, torch.Tensor) else np.asarray(rowptr)
        feats = tuner.features(rp, n_cols, N, dtype == torch.bfloat16)
        order = np.argsort(-host_forward(self.model, feats))
        ids = variant_ids(self.model["candidates"], dtype)
        # best-scored candidate that can run this width (vector kernels need N % vector width);
        # an infeasible pick falls back to the same kernel shape with narrower vectors
        v = 0
        names = S.spmm_variants(dtype)
        for i in order:
            cand = ids[int(i)]
            if exact and not is_exact(self.model["candidates"][int(i)]):
                continue
            if S.spmm_variant_supported(cand, N, dtype):
                v = cand
                break
            alt = narrower_feasible(names, names[cand - 1], N, dtype)
            if alt:
                v = alt
                break
        if key is not None:
            self._cache[(key, N, dtype, exact)] = v
        return v



# ------------------------------------------------------------------------------------------
# SDDMM path choice: CUDA cores (exact FP32 dot products) or the tcgen05 split-bf16 kernels
# ------------------------------------------------------------------------------------------
SDDMM_FORMAT = "armsparse-sddmm-selector-1"
DEFAULT_SDDMM_MODEL = os.path.join(os.path.dirname(os.path.abspath(__file__)),
                                   "sddmm_selector_model.json")


def sddmm_sweep_configs(n_patterns=160, seed=0, max_nnz=6_000_000, max_dense_bytes=1 << 30):
    """Seeded SDDMM problems: uniform patterns (density log-uniform in [1e-4, 0.3]), banded
    and power-law ones; rows and columns log-uniform in [512, 16384]; K in {32, ..., 2048}.
    Entries are capped at max_nnz and the dense operands at max_dense_bytes (sweep time)."""
    rng = np.random.default_rng(seed)
    kinds = ["uniform", "uniform", "banded", "powerlaw"]
    out = []
    for i in range(n_patterns):
        M = int(2 ** rng.uniform(9, 14))
        Nc = int(2 ** rng.uniform(9, 14))
        K = int(rng.choice([32, 64, 128, 256, 512, 1024, 2048]))
        while (M + Nc) * K * 4 > max_dense_bytes and K > 32:
            K //= 2
        cfg = {"id": i, "kind": kinds[i % 4], "M": M, "N": Nc, "K": K, "seed": 5000 + i}
        if cfg["kind"] == "uniform":
            cfg["density"] = float(min(10 ** rng.uniform(-4, math.log10(0.3)), max_nnz / (M * Nc)))
        elif cfg["kind"] == "banded":
            cfg["bandwidth"] = int(min(rng.integers(3, 257), max(3, max_nnz // M)))
        else:
            cfg["exponent"] = float(rng.uniform(1.8, 2.5))
            cfg["mean"] = float(min(rng.uniform(2, 300), max_nnz / M, Nc / 4))
        out.append(cfg)
    return out


def make_sddmm_pattern(cfg, device):
    """(rowptr, colind) of a sweep problem on the device, columns ascending in each row."""
    from . import synthetic as syn
    M, Nc = cfg["M"], cfg["N"]
    if cfg["kind"] == "powerlaw":
        rp, ci, _ = syn.powerlaw_csr_device(M, cfg["exponent"], cfg["mean"], cfg["seed"], device,
                                            n_cols=Nc)
        return rp, ci
    if cfg["kind"] == "banded":
        g = torch.Generator(device=device).manual_seed(cfg["seed"])
        bw = cfg["bandwidth"]
        rows = torch.arange(M, device=device).repeat_interleave(bw)
        off = torch.randint(-bw, bw + 1, (M * bw,), generator=g, device=device)
        cols = (rows * Nc // M + off).clamp_(0, Nc - 1)
        keys = torch.unique(rows * Nc + cols)
    else:
        g = torch.Generator(device=device).manual_seed(cfg["seed"])
        n = max(1, int(cfg["density"] * M * Nc))
        keys = torch.unique(torch.randint(0, M * Nc, (n,), generator=g, device=device))
    rows, cols = keys // Nc, (keys % Nc).to(torch.int32)
    rowptr = torch.zeros(M + 1, dtype=torch.int64, device=device)
    rowptr[1:] = torch.cumsum(torch.bincount(rows, minlength=M), 0)
    return rowptr.to(torch.int32), cols.contiguous()


def sddmm_sweep(configs, device=None, reps=3, log=None):
    """Time every SDDMM path (tuner.sddmm_paths) on each problem; returns records."""
    device = device or torch.device("cuda", 0)
    paths = tuner.sddmm_paths()
    records = []
    for cfg in configs:
        rowptr, colind = make_sddmm_pattern(cfg, device)
        g = torch.Generator(device=device).manual_seed(cfg["seed"] + 1)
        X = torch.randn(cfg["M"], cfg["K"], generator=g, device=device)
        Y = torch.randn(cfg["N"], cfg["K"], generator=g, device=device)
        t = tuner.autotune_sddmm(rowptr, colind, X, Y, paths=paths, reps=reps, max_ratio=4.0)
        feats = tuner.sddmm_features(rowptr, colind, cfg["N"], cfg["K"])
        rec = {"cfg": cfg, "features": feats.tolist(), "nnz": int(colind.numel()),
               "times_ms": [x.ms for x in t]}
        records.append(rec)
        if log:
            ok = [x for x in t if x.ms is not None]
            b = min(ok, key=lambda x: x.ms)
            log(f"{cfg['id']:4d} {cfg['kind']:8s} {cfg['M']}x{cfg['N']} K={cfg['K']} "
                f"nnz={rec['nnz']} best={b.name} {b.ms * 1e3:.1f}us "
                f"simt={t[0].ms if t[0].ms is None else round(t[0].ms * 1e3, 1)}us")
        del rowptr, colind, X, Y
    return records


def evaluate_sddmm(model, records):
    """Picked time / best time of the network over records (mean, geometric mean, worst),
    against always taking the CUDA-core path -- the reference's only kind of SDDMM kernel
    (gcn/pytorch-custom/sddmm.cu:438-455 chooses among them by K % 4 and K % 2 alone) -- and
    against always taking the library's default tensor-core variant."""
    picked, simt, tc = [], [], []
    names = model["candidates"]
    for r in records:
        t = np.array([np.inf if x is None else x for x in r["times_ms"]])
        best = t.min()
        scores = np.where(np.isfinite(t), host_forward(model, r["features"]), -np.inf)
        picked.append(t[int(np.argmax(scores))] / best)
        simt.append(t[names.index("simt")] / best)
        tc_best = [t[i] for i, n in enumerate(names) if n.startswith("tc")]
        tc.append(tc_best[-1] / best if np.isfinite(tc_best[-1]) else np.nan)
    gm = lambda a: float(np.exp(np.nanmean(np.log(np.asarray(a)))))
    return {"mlp_geomean": gm(picked), "mlp_mean": float(np.mean(picked)),
            "mlp_worst": float(np.max(picked)), "simt_geomean": gm(simt),
            "tc_default_geomean": gm(tc), "n": len(records)}


class SddmmSelector:
    """The learned choice of SDDMM path for a pattern and K: "simt" or "tc<variant>"."""

    def __init__(self, model: dict):
        if model.get("format") != SDDMM_FORMAT:
            raise ValueError("unknown SDDMM selector model format")
        self.model = model

    @classmethod
    def load(cls, path: str = DEFAULT_SDDMM_MODEL) -> "SddmmSelector":
        with open(path) as f:
            return cls(json.load(f))

    def save(self, path: str) -> None:
        with open(path, "w") as f:
            json.dump(self.model, f)

    def choose(self, rowptr, colind, n_cols: int, K: int) -> str:
        feats = tuner.sddmm_features(rowptr, colind, n_cols, K)
        scores = host_forward(self.model, feats)
        names = self.model["candidates"]
        known = set(tuner.sddmm_paths())
        for i in np.argsort(-scores):
            if names[int(i)] in known:
                return names[int(i)]
        return "simt"
