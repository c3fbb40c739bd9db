"""GCN on the sparse hot path: the autograd SpMM op, GCNConv and the 2-layer network.

Mirrors gcn/pytorch-custom/op.py (SPMMFunction :8-37, GCNConv :79-153) and the model/training
of gcn_custom.py (:72-126), GPU-resident, with three changes the reference lacks:

* backward computes dB = A^T * dY with the CSC arrays (as op.py:30 does) AND the gradient of
  the edge values dA[e] = <dY[row(e)], B[col(e)]> as an SDDMM at A's pattern (op.py:31 returns
  None);
* the CSC arrays come from the GPU transpose, computed once per graph and cached
  (``Graph.csc``), instead of a host scipy ``tocsc()`` (gcn_custom.py:52);
* no hidden global state: the reference's backward returns a stale module-level ``grad_feat``
  when called without edge weights (op.py:21, :33-35).

Orientation is explicit: ``rowptr/colind`` is the CSR of A in out = A * x (the reference builds
its "rowptr" from ``tocsc()``, gcn_custom.py:48-55, which only coincides for symmetric graphs).
"""
from __future__ import annotations

import math

import torch
import torch.nn.functional as F
from torch.nn import Parameter

from . import sparse as S
from ._native import NativeError


def _spmm(rowptr, colind, values, feat, variant=0, relu=False):
    """A * feat (relu(A * feat) when relu) for fp32 / fp64 / bf16 features (bf16 values and
    features are multiplied in fp32; the result is returned in the feature dtype)."""
    if feat.dtype == torch.bfloat16:
        vb = values.to(torch.bfloat16)
        try:  # C written in bf16 by the kernel, the ReLU applied in the same store
            return S.spmm(rowptr, colind, vb, feat.contiguous(), variant=variant,
                          out_dtype=torch.bfloat16, relu=relu)
        except NativeError as e:
            if e.status != 3:  # AS_ERR_UNSUPPORTED (a bulk variant): fp32 C, then rounded
                raise
        out = S.spmm(rowptr, colind, vb, feat.contiguous(), variant=variant).to(torch.bfloat16)
    else:
        out = S.spmm(rowptr, colind, values.to(feat.dtype), feat.contiguous(), variant=variant)
    return F.relu(out) if relu else out


class SPMMFunction(torch.autograd.Function):
    """out = A * feat, A given as CSR (rowptr, colind, edge_weight_csr) and as CSC (colptr, rowind,
    edge_weight_csc). Same ``apply`` signature as the reference (op.py:9), plus an optional
    ``variants`` pair (kernel variant ids for the forward CSR product and the backward CSC
    product; 0 = library choice) and an optional ``csc_pos`` (the CSC position of each CSR
    entry, ``Graph.csc_pos``): given it, a backward that needs both gradients runs them in one
    pass over the CSC (``sparse.spmm_sddmm``: dOut's rows gathered once for dB and dA), the
    edge gradient written in CSC order and then gathered into CSR order. ``relu=True`` returns
    relu(A * feat), the ReLU applied in the SpMM's store (its backward masks the gradient by
    the output, as F.relu's does)."""

    @staticmethod
    def forward(ctx, rowptr, colind, colptr, rowind, feat, edge_weight_csr=None,
                edge_weight_csc=None, variants=None, csc_pos=None, relu=False):
        if edge_weight_csr is None:
            raise ValueError("SPMMFunction needs edge values (pass ones for an unweighted graph)")
        fwd_v, bwd_v = variants if variants is not None else (0, 0)
        out = _spmm(rowptr, colind, edge_weight_csr, feat, fwd_v, relu)
        ctx.save_for_backward(rowptr, colind, colptr, rowind, feat, edge_weight_csr,
                              edge_weight_csc, csc_pos, out if relu else None)
        ctx.bwd_variant = bwd_v
        return out

    @staticmethod
    def backward(ctx, grad_out):
        rowptr, colind, colptr, rowind, feat, w_csr, w_csc, csc_pos, out = ctx.saved_tensors
        grad_feat = grad_w = None
        g = grad_out.contiguous()
        if out is not None:  # the ReLU's backward: zero where the output was clamped
            g = torch.ops.aten.threshold_backward(g, out, 0)
        if (csc_pos is not None and ctx.needs_input_grad[4] and ctx.needs_input_grad[5] and
                w_csc is not None and w_csc.numel() == w_csr.numel() and g.dtype == feat.dtype
                and g.dtype in (torch.float32, torch.bfloat16)):
            fused = _spmm_sddmm_t(colptr, rowind, w_csc, g, feat.contiguous(), csc_pos,
                                  ctx.bwd_variant)
            if fused is not None:
                grad_feat, grad_w = fused
                return (None, None, None, None, grad_feat, grad_w.to(w_csr.dtype), None, None,
                        None, None)
        if ctx.needs_input_grad[4]:
            if w_csc is None or w_csc.numel() != w_csr.numel():
                raise RuntimeError("backward of SPMMFunction needs the edge values in CSC order "
                                   "(SPMMFunction.apply(rowptr, colind, colptr, rowind, feat, "
                                   "values_csr, values_csc))")
            grad_feat = _spmm(colptr, rowind, w_csc, g, ctx.bwd_variant)
        if ctx.needs_input_grad[5]:
            if g.dtype == torch.bfloat16 and feat.dtype == torch.bfloat16:
                # bf16 layer: bf16 operands, fp32 products and sums
                grad_w = S.sddmm(rowptr, colind, g, feat.contiguous()).to(w_csr.dtype)
            else:
                gf = g if g.dtype in (torch.float32, torch.float64) else g.float()
                ff = feat if feat.dtype == gf.dtype else feat.to(gf.dtype)
                grad_w = S.sddmm(rowptr, colind, gf, ff.contiguous()).to(w_csr.dtype)
        return None, None, None, None, grad_feat, grad_w, None, None, None, None


def _spmm_sddmm_t(colptr, rowind, w_csc, g, feat, csc_pos, variant):
    """(A^T g, dA) in one pass over the CSC, or None when the backward variant cannot carry
    the SDDMM (not an nnz-split kernel, or its column tile is narrower than the width). dA is
    written in CSC order (coalesced) and gathered into CSR order: measured faster than
    scattering it through the permutation inside the pass."""
    try:
        C, dA_csc = S.spmm_sddmm(colptr, rowind, w_csc.to(g.dtype), g, feat, variant=variant,
                                 out_dtype=g.dtype)
    except NativeError as e:
        if e.status != 3:  # AS_ERR_UNSUPPORTED: run the two products separately
            raise
        return None
    return C, S.gather(dA_csc, csc_pos)


def _time_pick(rowptr, colind, values, n_in: int, width: int, dtype, exact: bool = False) -> int:
    """The fastest of the selector's candidate SpMM kernels on these arrays (timed once);
    with ``exact`` only the bit-exact families (selector.is_exact)."""
    from . import selector as SEL
    from . import tuner
    B = torch.zeros(n_in, width, device=rowptr.device, dtype=dtype)
    names = [n for n in SEL.CANDIDATES if not exact or SEL.is_exact(n)]
    ids = SEL.variant_ids(names, dtype)
    return tuner.best(tuner.autotune_spmm(rowptr, colind, values.to(dtype), B, variants=ids,
                                          reps=3, max_ratio=3.0)).variant


def _nnz_tile(name: str, esz: int) -> int:
    """Column tile (vector elements x lanes x vectors per lane) of an nnz-split or multi-entry
    variant name."""
    f = {p[0]: int(p[1:]) for p in name.split("_")[1:] if p[:1] in "vgc" and p[1:].isdigit()}
    return (f["v"] // esz) * f["g"] * f.get("c", 1)


def _time_pick_fused(colptr, rowind, values, n_out: int, width: int, dtype) -> int:
    """The fastest nnz-split kernel for the fused backward pass (A^T dOut with the edge-value
    SDDMM, ``sparse.spmm_sddmm``) on these arrays, timed once; 0 when none can carry it."""
    from . import tuner
    esz = 4 if dtype == torch.float32 else 2
    dev = colptr.device
    g = torch.zeros(n_out, width, device=dev, dtype=dtype)
    f = torch.zeros(colptr.numel() - 1, width, device=dev, dtype=dtype)
    C = torch.empty(colptr.numel() - 1, width, device=dev, dtype=dtype)  # as the backward writes
    dA = torch.empty(rowind.numel(), device=dev)
    vals = values.to(dtype)
    best, best_ms = 0, float("inf")
    for i, name in enumerate(S.spmm_variants(dtype)):
        v = i + 1
        if (not name.startswith(("nnzsplit", "nnzme")) or _nnz_tile(name, esz) < width
                or not S.spmm_variant_supported(v, width, dtype)):
            continue
        fn = lambda: S.spmm_sddmm(colptr, rowind, vals, g, f, C=C, variant=v, dA=dA,
                                  out_dtype=dtype)
        try:
            fn()
        except NativeError:
            continue
        ms = tuner.time_cuda(fn, reps=3, warmup=1, flush=False)
        if ms < best_ms:
            best, best_ms = v, ms
    return best


class _DenseProduct(torch.autograd.Function):
    """x @ W for a tall dense x and a narrow W. The weight gradient x^T dY reduces over all
    rows into a few outputs (64 x 3 for the GCN's second layer); as one GEMM that runs on a
    single tile for the whole reduction, so it is split into row blocks of kRows, reduced by
    a batched GEMM and a sum."""

    kRows = 1024

    @staticmethod
    def forward(ctx, x, W):
        ctx.save_for_backward(x, W)
        return x @ W

    @staticmethod
    def backward(ctx, g):
        x, W = ctx.saved_tensors
        dx = g @ W.t() if ctx.needs_input_grad[0] else None
        dW = None
        if ctx.needs_input_grad[1]:
            n, r = x.shape[0], _DenseProduct.kRows
            pad = (-n) % r
            xp = torch.nn.functional.pad(x, (0, 0, 0, pad)) if pad else x
            gp = torch.nn.functional.pad(g, (0, 0, 0, pad)) if pad else g
            b = xp.shape[0] // r
            dW = torch.bmm(xp.reshape(b, r, -1).transpose(1, 2), gp.reshape(b, r, -1)).sum(0)
        return dx, dW


class Graph:
    """A sparse adjacency on the GPU with its transpose computed once (GPU, deterministic)."""

    def __init__(self, rowptr: torch.Tensor, colind: torch.Tensor, values: torch.Tensor,
                 n_cols: int | None = None):
        self.rowptr, self.colind, self.values = rowptr, colind, values
        self.n_rows = rowptr.numel() - 1
        self.n_cols = self.n_rows if n_cols is None else n_cols
        self._csc = None
        self._perm = None
        self._csc_pos = None
        self.selector = None  # a selector.Selector: per-width kernel choice (None = library choice)
        # with a selector: True restricts the choice to kernels whose outputs are the CSR-order
        # chains (so training is bit-for-bit the library default's), False lets it take the
        # entry-balanced kernels too (their sums differ in the last bits for rows that cross a
        # chunk, and over hundreds of epochs the losses drift apart by up to ~1e-3)
        self.exact = False
        self._plans = {}

    @property
    def csc(self):
        """(colptr, rowind, values in CSC order), from the transpose that also gives ``perm``."""
        if self._csc is None:
            colptr, rowind, perm = S.csr2csc_perm(self.rowptr, self.colind, self.n_cols)
            self._perm = perm
            self._csc = (colptr, rowind, torch.index_select(self.values, 0, perm))
        return self._csc

    @property
    def perm(self) -> torch.Tensor:
        """The CSR position of each CSC entry (int32): ``values[perm]`` is the values in CSC
        order for any values."""
        self.csc
        return self._perm

    @property
    def csc_pos(self) -> torch.Tensor:
        """The CSC position of each CSR entry (int32, the inverse of ``perm``): the fused
        backward gathers the edge gradient from CSC into CSR order through it."""
        if self._csc_pos is None:
            p = self.perm
            pos = torch.empty_like(p)
            pos[p.long()] = torch.arange(p.numel(), device=p.device, dtype=torch.int32)
            self._csc_pos = pos
        return self._csc_pos

    def plan(self, N: int, dtype=torch.float32, fused: bool = False):
        """(forward, backward) kernel variants for dense width N: the learned selector's pick,
        or -- for widths below the 16..256 it was trained on -- the fastest of its candidate
        kernels timed once on this graph. fused: the backward variant is for the fused pass
        (``SPMMFunction`` given ``perm`` and trainable values) -- the fastest nnz-split kernel
        that carries the SDDMM, timed once."""
        if self.selector is None or dtype == torch.float64:
            return (0, 0)
        if fused and not self.exact:
            key = (N, dtype, "fused")
            if key not in self._plans:
                colptr, rowind, vcsc = self.csc
                bwd = _time_pick_fused(colptr, rowind, vcsc, self.n_rows, N, dtype)
                self._plans[key] = (self.plan(N, dtype)[0], bwd or self.plan(N, dtype)[1])
            return self._plans[key]
        key = (N, dtype, self.exact)
        if key not in self._plans:
            colptr, rowind, vcsc = self.csc
            ex = self.exact
            if N < 16:
                self._plans[key] = (_time_pick(self.rowptr, self.colind, self.values,
                                               self.n_cols, N, dtype, ex),
                                    _time_pick(colptr, rowind, vcsc, self.n_rows, N, dtype, ex))
            else:
                self._plans[key] = (self.selector.choose(self.rowptr, self.n_cols, N, dtype,
                                                         exact=ex),
                                    self.selector.choose(colptr, self.n_rows, N, dtype,
                                                         exact=ex))
        return self._plans[key]

    @classmethod
    def from_csr(cls, a, device) -> "Graph":
        t = lambda x: torch.from_numpy(x).to(device)
        return cls(t(a.rowptr), t(a.colind), t(a.val), a.n_cols)

    def aggregate(self, feat: torch.Tensor) -> torch.Tensor:
        colptr, rowind, vcsc = self.csc
        return SPMMFunction.apply(self.rowptr, self.colind, colptr, rowind, feat, self.values,
                                  vcsc, self.plan(feat.shape[1], feat.dtype), self.csc_pos)


class _FeatureProduct(torch.autograd.Function):
    """X @ W with X sparse (CSR, and its transpose for the backward) and W dense: the SpMM of
    this library in both directions; dW = X^T dY. X takes no gradient."""

    @staticmethod
    def forward(ctx, feats, W):
        ctx.feats = feats
        return S.spmm(feats.rowptr, feats.colind, feats.values, W.contiguous(),
                      variant=feats.plan(W.shape[1], True))

    @staticmethod
    def backward(ctx, grad_out):
        f = ctx.feats
        rp_t, ci_t, v_t = f.transposed
        dW = S.spmm(rp_t, ci_t, v_t, grad_out.contiguous(),
                    variant=f.plan(grad_out.shape[1], False))
        return None, dW


class SparseFeatures:
    """Node features stored as CSR on the GPU: the bag-of-words inputs of citation graphs
    (the reference's PubMed features are TF-IDF vectors, about 10 % non-zero). The first
    layer's X @ W then runs as an SpMM (and its weight gradient as an SpMM with X^T), in
    place of a dense GEMM over mostly zeros. Built from a dense matrix with the GPU
    format builder; the sparsity pattern is fixed, the values can be refreshed in place
    (``load_values``)."""

    def __init__(self, dense: torch.Tensor, selector=None):
        self.shape = tuple(dense.shape)
        self.rowptr, self.colind, self.values = S.dense_to_csr(dense.contiguous())
        self.transposed = S.csr2csc(self.rowptr, self.colind, self.values, self.shape[1])
        self.selector = selector
        self._plans = {}

    def load_values(self, values: torch.Tensor) -> None:
        """New feature values with the same sparsity pattern (CSR order), written into the
        existing buffers (a recorded CUDA graph keeps reading them)."""
        self.values.copy_(values, non_blocking=True)
        self.transposed[2].copy_(S.csr2csc(self.rowptr, self.colind, self.values,
                                           self.shape[1])[2])

    def plan(self, width: int, forward: bool) -> int:
        """Kernel variant for X @ W (forward) or X^T @ dY, chosen once per width by timing the
        selector's candidate kernels on these matrices (X^T has few, very long rows -- outside
        the shapes the learned selector was trained on)."""
        if self.selector is None:
            return 0
        key = (width, forward)
        if key not in self._plans:
            from . import selector as SEL
            from . import tuner
            rp, ci, v = (self.rowptr, self.colind, self.values) if forward else self.transposed
            n_in = self.shape[1] if forward else self.shape[0]
            B = torch.zeros(n_in, width, device=self.device)
            ids = SEL.variant_ids(SEL.CANDIDATES, torch.float32)
            best = tuner.best(tuner.autotune_spmm(rp, ci, v, B, variants=ids, reps=3,
                                                   max_ratio=3.0))
            self._plans[key] = best.variant
        return self._plans[key]

    @property
    def device(self) -> torch.device:
        return self.values.device

    @property
    def dtype(self) -> torch.dtype:
        return self.values.dtype

    def matmul(self, W: torch.Tensor) -> torch.Tensor:
        return _FeatureProduct.apply(self, W)


def glorot_(w: torch.Tensor) -> None:
    """U(-a, a), a = sqrt(6 / (fan_in + fan_out)) (the init op.py:76 imports)."""
    a = math.sqrt(6.0 / (w.size(-2) + w.size(-1)))
    with torch.no_grad():
        w.uniform_(-a, a)


class GCNConv(torch.nn.Module):
    """x -> D_in^-1/2 * A * D_out^-1/2 * (x W) + b, op for op as op.py:112-149: the dense
    product, the pre-scale by 1/sqrt(out-degree) (from colptr), the SpMM, the post-scale by
    1/sqrt(in-degree) (from rowptr), the bias."""

    def __init__(self, in_channels, out_channels, bias=True, normalize=True, cached=True):
        super().__init__()
        self.in_channels, self.out_channels = in_channels, out_channels
        self.normalize, self.cached = normalize, cached
        self.weight = Parameter(torch.empty(in_channels, out_channels))
        self.bias = Parameter(torch.empty(out_channels)) if bias else None
        self.cached_result = None
        self.reset_parameters()

    def reset_parameters(self):
        glorot_(self.weight)
        if self.bias is not None:
            with torch.no_grad():
                self.bias.zero_()
        self.cached_result = None

    @staticmethod
    def deg_inv_sqrt(indptr):
        return (1 / torch.sqrt((indptr[1:] - indptr[:-1]).float())).unsqueeze(dim=1)

    def forward(self, x, rowptr, colind, colptr, rowind, edge_weight_csr, edge_weight_csc,
                variants=None):
        if isinstance(x, SparseFeatures):
            x = x.matmul(self.weight)
        elif x.dim() == 2 and x.shape[0] >= 8 * _DenseProduct.kRows:
            x = _DenseProduct.apply(x, self.weight)
        else:
            x = torch.matmul(x, self.weight)
        if not self.cached or self.cached_result is None:
            if self.normalize:
                in_norm, out_norm = self.deg_inv_sqrt(rowptr), self.deg_inv_sqrt(colptr)
            else:
                in_norm = out_norm = None
            self.cached_result = (in_norm, out_norm)
        in_norm, out_norm = self.cached_result
        if self.normalize:
            x = x * out_norm
        out = SPMMFunction.apply(rowptr, colind, colptr, rowind, x, edge_weight_csr,
                                 edge_weight_csc, variants)
        if self.normalize:
            out = out * in_norm
        if self.bias is not None:
            out = out + self.bias
        return out


class Net(torch.nn.Module):
    """2-layer GCN of gcn_custom.py:72-90: conv -> relu -> dropout -> conv -> log_softmax."""

    def __init__(self, n_features, n_hidden, n_classes, dropout: float = 0.5):
        super().__init__()
        self.conv1 = GCNConv(n_features, n_hidden)
        self.conv2 = GCNConv(n_hidden, n_classes)
        self.dropout = dropout

    def forward(self, x, g: Graph):
        colptr, rowind, vcsc = g.csc
        args = (g.rowptr, g.colind, colptr, rowind, g.values, vcsc)
        x = F.relu(self.conv1(x, *args, variants=g.plan(self.conv1.out_channels, x.dtype)))
        x = F.dropout(x, p=self.dropout, training=self.training)
        x = self.conv2(x, *args, variants=g.plan(self.conv2.out_channels, x.dtype))
        return F.log_softmax(x, dim=1)


def nll_mean(logp: torch.Tensor, y: torch.Tensor) -> torch.Tensor:
    """F.nll_loss(logp, y) (mean over the rows) as a gather and a mean: the same value up to
    fp32 summation order, but both directions run as elementwise and tree-reduction kernels,
    where torch's nll_loss reduces over all rows in one thread block (milliseconds on a
    million-row batch)."""
    return -logp.gather(1, y.unsqueeze(1)).mean()


class SoftmaxXent(torch.autograd.Function):
    """Mean softmax cross-entropy of bf16 class scores (n x width, the first n_classes columns
    are the classes): the model's log_softmax then F.nll_loss (gcn_custom.py:90, :122-126) as
    one forward and one backward kernel of this library (``sparse.softmax_xent``). The
    gradient is bf16, zero in the padding columns."""

    @staticmethod
    def forward(ctx, scores, labels, n_classes: int):
        loss, lse = S.softmax_xent(scores, labels, n_classes)
        ctx.save_for_backward(scores, labels, lse)
        ctx.n_classes = n_classes
        return loss

    @staticmethod
    def backward(ctx, g):
        scores, labels, lse = ctx.saved_tensors
        G = S.softmax_xent_grad(scores, labels, ctx.n_classes, lse, g.float().contiguous())
        return G, None, None


def make_optimizer(model: Net, capturable: bool = False):
    """Adam, lr 0.01, weight decay 5e-4 on the first layer only (gcn_custom.py:116-119).
    capturable keeps Adam's step count on the device so that the step can be recorded in a
    CUDA graph (``CapturedEpoch``)."""
    return torch.optim.Adam([dict(params=model.conv1.parameters(), weight_decay=5e-4),
                             dict(params=model.conv2.parameters(), weight_decay=0)], lr=0.01,
                            capturable=capturable)


def train_epoch(model, opt, x, g, y, train) -> torch.Tensor:
    """One full-batch step (gcn_custom.py:122-126); returns the loss (on the device). ``train``
    is the boolean training mask or the ascending indices of the training nodes (the same
    loss; indices need no host synchronisation, which a boolean mask does)."""
    model.train()
    opt.zero_grad(set_to_none=True)
    out = model(x, g)
    if train.dtype == torch.bool:
        loss = F.nll_loss(out[train], y[train])
    else:
        loss = F.nll_loss(out.index_select(0, train), y.index_select(0, train))
    loss.backward()
    opt.step()
    return loss.detach()


class CapturedEpoch:
    """A training epoch recorded once as a CUDA graph and replayed per call: on a graph of
    PubMed's size an eager epoch is bound by host-side launch overhead (some 80 kernel
    launches through autograd), a replay by the kernels themselves.

    Before recording, ``warmup`` eager epochs run on a side stream (they are real training
    epochs: the weights move), which also settles everything the recording must not do: the
    CSC transpose and the selector's plans are cached on the graph, the library scratch has
    reached its size, Adam's state exists. ``opt`` must be built with ``capturable=True``.
    New node features are fed by copying into ``x`` in place; every replay draws fresh dropout
    masks."""

    def __init__(self, model, opt, x, g: Graph, y, train, warmup: int = 3):
        if train.dtype == torch.bool:
            train = train.nonzero().squeeze(1)
        if not all(group.get("capturable", False) for group in opt.param_groups):
            raise ValueError("CapturedEpoch needs an optimizer built with capturable=True")
        dev = x.device
        side = torch.cuda.Stream(dev)
        side.wait_stream(torch.cuda.current_stream(dev))
        with torch.cuda.stream(side):
            for _ in range(max(1, warmup)):
                train_epoch(model, opt, x, g, y, train)
        torch.cuda.current_stream(dev).wait_stream(side)
        # the recorded kernels read these tensors' memory at every replay: keep them alive
        self.static = (model, opt, x, g, y, train)
        self.graph = torch.cuda.CUDAGraph()
        from . import _native
        before = _native.total_launches()
        with torch.cuda.graph(self.graph):
            self.loss = train_epoch(model, opt, x, g, y, train)
        self.launches = _native.total_launches() - before  # this library's kernels per replay

    def __call__(self) -> torch.Tensor:
        """One epoch; returns the loss tensor (overwritten by the next call)."""
        self.graph.replay()
        return self.loss


def synthetic_task(n_nodes=19717, n_edges=88648, n_features=500, n_classes=3, seed=0,
                   device="cuda"):
    """PubMed-shaped stand-in: power-law undirected graph with self-loops, 10 % non-zero U(0,1)
    features, random labels, 60 training nodes per class (the reference's Planetoid split)."""
    import numpy as np

    from . import synthetic as syn
    a = syn.powerlaw_graph(n_nodes, n_edges, seed=seed)
    rng = np.random.default_rng(seed + 1)
    x = np.zeros((n_nodes, n_features), np.float32)
    mask = rng.random(x.shape) < 0.1
    x[mask] = rng.random(int(mask.sum())).astype(np.float32)
    y = rng.integers(0, n_classes, n_nodes)
    train = np.zeros(n_nodes, bool)
    for c in range(n_classes):
        idx = np.flatnonzero(y == c)[:60]
        train[idx] = True
    dev = torch.device(device)
    g = Graph.from_csr(a, dev)
    return (torch.from_numpy(x).to(dev), g, torch.from_numpy(y).to(dev),
            torch.from_numpy(train).to(dev), a)
