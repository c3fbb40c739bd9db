"""The GCN op on the GPU: the torch extension `spmm`, the autograd SPMMFunction and GCNConv
against golden vectors made by running the reference's own op.py (forward bit-exact, input
gradient bit-exact), FP64 gradcheck on a 500-node subgraph, and run-to-run reproducibility
of GCN training."""
import numpy as np
import pytest
import torch

import armsparse_gb300 as A
from armsparse_gb300 import gcn
from armsparse_gb300 import synthetic as S
from gpu_util import bits, dev, to_dev

pytestmark = pytest.mark.gpu


def test_extension_ops(oracle):
    from armsparse_gb300.torch_ops import spmm
    a = S.uniform_csr(700, 500, 9000, seed=3)
    B = S.dense_uniform((500, 64), 4)
    rp, ci, v, Bd = to_dev(a.rowptr), to_dev(a.colind), to_dev(a.val), to_dev(B)
    out = spmm.csr_spmm(rp, ci, v, Bd)
    assert np.array_equal(bits(out), bits(oracle.spmm_fma_chain_f32(a.rowptr, a.colind, a.val, B)))
    ob = spmm.csr_spmm(rp, ci, v.bfloat16(), Bd.bfloat16())
    assert ob.dtype == torch.float32
    X, Y = S.dense_normal((700, 32), 5), S.dense_normal((500, 32), 6)
    s = spmm.csr_sddmm(rp, ci, to_dev(X), to_dev(Y))
    assert np.array_equal(bits(s), bits(oracle.sddmm_f32_group(a.rowptr, a.colind, X, Y)))
    rows = np.repeat(np.arange(700, dtype=np.int32), np.diff(a.rowptr))
    s2 = spmm.coo_sddmm(to_dev(rows), ci, to_dev(X), to_dev(Y))
    assert torch.equal(s, s2)
    colptr = torch.empty(501, dtype=torch.int32, device=dev())
    rowind = torch.empty(a.nnz, dtype=torch.int32, device=dev())
    cv = spmm.csr2csc(rp, ci, colptr, rowind, v)
    ocp, ori, ocv = oracle.csr2csc(a.rowptr, a.colind, a.val, 500)
    assert np.array_equal(colptr.cpu().numpy(), ocp) and np.array_equal(rowind.cpu().numpy(), ori)
    assert np.array_equal(bits(cv), bits(ocv))
    with pytest.raises(RuntimeError):
        spmm.csr_spmm(rp, ci, v, Bd.double())


def test_spmm_function_matches_reference_op(golden):
    g = golden["gcn_op"]
    rp, ci, cp, ri = (to_dev(g[k]) for k in ("rowptr", "colind", "colptr", "rowind"))
    w, wc = to_dev(g["val"]), to_dev(g["val_csc"])
    f = to_dev(g["feat"]).requires_grad_(True)
    out = gcn.SPMMFunction.apply(rp, ci, cp, ri, f, w, wc)
    out.backward(to_dev(g["grad_out"]))
    assert np.array_equal(bits(out), bits(g["out"]))
    assert np.array_equal(bits(f.grad), bits(g["grad_feat"]))
    # the same through the cached GPU transpose
    G = gcn.Graph(rp, ci, w)
    colptr, rowind, vcsc = G.csc
    assert torch.equal(colptr, cp) and torch.equal(rowind, ri)
    assert np.array_equal(bits(vcsc), bits(g["val_csc"]))


def test_gcnconv_matches_reference_op(golden):
    g = golden["gcn_op"]
    rp, ci, cp, ri = (to_dev(g[k]) for k in ("rowptr", "colind", "colptr", "rowind"))
    w, wc = to_dev(g["val"]), to_dev(g["val_csc"])
    conv = gcn.GCNConv(16, 8).to(dev())
    with torch.no_grad():
        conv.weight.copy_(to_dev(g["W"]))
        conv.bias.copy_(to_dev(g["b"]))
    x = to_dev(g["feat"]).requires_grad_(True)
    y = conv(x, rp, ci, cp, ri, w, wc)
    y.backward(to_dev(g["conv_grad_out"]))
    # the dense x @ W runs in cuBLAS here and in CPU torch in the reference: FP32 rounding only
    for got, ref in ((y, g["conv_out"]), (x.grad, g["conv_grad_x"]),
                     (conv.weight.grad, g["conv_grad_W"]), (conv.bias.grad, g["conv_grad_b"])):
        got = got.detach().cpu().numpy()
        assert np.allclose(got, ref, rtol=1e-5, atol=1e-5 * np.abs(ref).max()), np.abs(got - ref).max()


def _subgraph(a, n):
    """Induced subgraph on the first n nodes (keeps self-loops), CSR."""
    rows = np.repeat(np.arange(a.n_rows), np.diff(a.rowptr))
    keep = (rows < n) & (a.colind < n)
    r, c = rows[keep], a.colind[keep]
    rp = np.zeros(n + 1, np.int32)
    np.cumsum(np.bincount(r, minlength=n), out=rp[1:])
    return S.CSR(rp, c.astype(np.int32), a.val[keep], n, n)


def test_gradcheck_fp64_500_node_subgraph():
    a = _subgraph(S.powerlaw_graph(19717, 88648, seed=9), 500)
    rng = np.random.default_rng(1)
    w = rng.uniform(0.5, 1.5, a.nnz)
    G = gcn.Graph(to_dev(a.rowptr), to_dev(a.colind), to_dev(w.astype(np.float32)))
    colptr, rowind, _ = G.csc
    # CSC values in float64: permute the CSR values the way the transpose does
    perm = np.lexsort((np.repeat(np.arange(500), np.diff(a.rowptr)), a.colind))
    wd = torch.tensor(w, dtype=torch.float64, device=dev(), requires_grad=True)
    wcsc = torch.tensor(w[perm], dtype=torch.float64, device=dev())
    feat = torch.randn(500, 3, dtype=torch.float64, device=dev(), requires_grad=True)
    fn = lambda f, ww: gcn.SPMMFunction.apply(G.rowptr, G.colind, colptr, rowind, f, ww, wcsc)
    assert torch.autograd.gradcheck(fn, (feat, wd), eps=1e-6, atol=1e-8, rtol=1e-6)


def test_edge_value_gradient_is_sddmm(oracle):
    a = S.powerlaw_graph(2000, 12000, seed=4)
    G = gcn.Graph.from_csr(a, dev())
    w = G.values.clone().requires_grad_(True)
    colptr, rowind, vcsc = G.csc
    f = torch.randn(2000, 24, device=dev())
    out = gcn.SPMMFunction.apply(G.rowptr, G.colind, colptr, rowind, f, w, vcsc)
    gy = torch.randn_like(out)
    out.backward(gy)
    ref = oracle.sddmm_f32_group(a.rowptr, a.colind, gy.cpu().numpy(), f.cpu().numpy())
    assert np.array_equal(bits(w.grad), bits(ref))


def test_fused_backward_matches_separate(oracle):
    """With Graph.csc_pos, a backward needing both gradients runs one pass over the CSC: dB is
    the unfused nnz-split SpMM's bits, dA the slices-order oracle's bits in CSR order."""
    a = S.powerlaw_graph(3000, 20000, seed=5)
    G = gcn.Graph.from_csr(a, dev())
    colptr, rowind, vcsc = G.csc
    cp, ri, _ = oracle.csr2csc(a.rowptr, a.colind, a.val, a.n_cols)
    assert np.array_equal(colptr.cpu().numpy(), cp) and np.array_equal(rowind.cpu().numpy(), ri)
    var = A.spmm_variants().index("nnzsplit_v4_g32_c1_ch1024") + 1
    gen = torch.Generator(device=dev()).manual_seed(6)
    f0 = torch.randn(3000, 24, generator=gen, device=dev())
    gy = torch.randn(3000, 24, generator=gen, device=dev())
    grads = []
    for pos in (G.csc_pos, None):
        w = G.values.clone().requires_grad_(True)
        f = f0.clone().requires_grad_(True)
        out = gcn.SPMMFunction.apply(G.rowptr, G.colind, colptr, rowind, f, w, vcsc, (0, var),
                                     pos)
        out.backward(gy)
        grads.append((f.grad, w.grad))
    assert torch.equal(grads[0][0], grads[1][0])
    ref = oracle.sddmm_f32_slices(cp, ri, f0.cpu().numpy(), gy.cpu().numpy(), 32, 1, 1,
                                  perm=G.perm.cpu().numpy())
    assert np.array_equal(bits(grads[0][1]), bits(ref))
    pos = G.csc_pos.cpu().numpy()
    assert np.array_equal(G.perm.cpu().numpy()[pos], np.arange(pos.size))
    r64, ab = oracle.sddmm_f64(a.rowptr, a.colind, gy.cpu().numpy(), f0.cpu().numpy())
    assert oracle.scaled_err(grads[1][1].cpu().numpy(), r64, ab).max() < 1e-5


def test_relu_epilogue_matches_relu_after():
    """SPMMFunction(relu=True) on bf16 features: the output is F.relu of the plain op's and the
    gradients through it are the same bits (the backward masks by the output as F.relu's)."""
    a = S.powerlaw_graph(4000, 30000, seed=8)
    G = gcn.Graph.from_csr(a, dev())
    colptr, rowind, vcsc = G.csc
    gen = torch.Generator(device=dev()).manual_seed(9)
    f0 = torch.randn(4000, 64, generator=gen, device=dev()).to(torch.bfloat16)
    gy = torch.randn(4000, 64, generator=gen, device=dev()).to(torch.bfloat16)
    res = []
    for fused in (True, False):
        f = f0.clone().requires_grad_(True)
        w = G.values.clone().requires_grad_(True)
        if fused:
            out = gcn.SPMMFunction.apply(G.rowptr, G.colind, colptr, rowind, f, w, vcsc, None,
                                         None, True)
        else:
            out = torch.nn.functional.relu(
                gcn.SPMMFunction.apply(G.rowptr, G.colind, colptr, rowind, f, w, vcsc))
        out.backward(gy)
        res.append((out.detach(), f.grad, w.grad))
    assert torch.equal(res[0][0], res[1][0])
    assert torch.equal(res[0][1], res[1][1])
    assert torch.equal(res[0][2], res[1][2])


def test_gcn_training_is_reproducible():
    x, g, y, train, _ = gcn.synthetic_task(seed=0)

    def run():
        torch.manual_seed(0)
        model = gcn.Net(x.shape[1], 64, 3).to(dev())
        opt = gcn.make_optimizer(model)
        return torch.stack([gcn.train_epoch(model, opt, x, g, y, train) for _ in range(10)])

    l1, l2 = run(), run()
    assert torch.equal(l1, l2)
    assert torch.isfinite(l1).all() and l1[-1] < l1[0]


def test_tuned_training_tracks_plain_path():
    """200 full-batch epochs (the loop of gcn_custom.py:143-152; dropout 0.5, Adam as
    :116-119) from the same seed, three ways: the library default (plain: bit-exact row-split
    chains), the learned selector restricted to bit-exact kernels (Graph.exact), and the
    selector free to take its entry-balanced picks. The exact-tuned losses equal the plain ones
    bit for bit at every epoch (so |dloss| <= 1e-4 holds trivially). The free picks reorder
    the sums of rows that cross a chunk: their losses agree to 1e-4 over the first 20 epochs,
    and the 1-ulp differences grow through training (about 2e-3 by epoch 180)."""
    from armsparse_gb300 import selector
    x, g, y, train, _ = gcn.synthetic_task(seed=0)
    idx = train.nonzero().squeeze(1)

    def run(sel, exact=False):
        g.selector = sel
        g.exact = exact
        g._plans = {}
        if sel is not None:  # plans are made (and any candidate timed) before the seed is set
            g.plan(64)
            g.plan(3)
        torch.manual_seed(0)
        model = gcn.Net(x.shape[1], 64, 3).to(dev())
        opt = gcn.make_optimizer(model)
        return torch.stack([gcn.train_epoch(model, opt, x, g, y, idx) for _ in range(200)]).cpu().numpy()

    plain = run(None)
    sel = selector.Selector.load()
    exact = run(sel, exact=True)
    names = A.spmm_variants()
    assert all(selector.is_exact(names[v - 1]) for v in g.plan(64) + g.plan(3) if v)
    assert np.isfinite(plain).all() and plain[-1] < plain[0]
    assert np.array_equal(exact.view(np.uint32), plain.view(np.uint32))
    free = run(sel, exact=False)
    diff = np.abs(plain.astype(np.float64) - free.astype(np.float64))
    assert diff[:20].max() <= 1e-4, float(diff[:20].max())
    assert np.isfinite(free).all() and free[-1] < free[0]
    g.selector, g.exact = None, False
    A.sync_status()


def test_captured_epoch_matches_eager():
    """The CUDA-graph epoch replays the same training step as the eager one: with dropout off
    and the same initial weights, losses agree epoch by epoch; with dropout on, training
    still converges and fresh masks are drawn per replay."""
    from armsparse_gb300 import selector
    x, g, y, train, _ = gcn.synthetic_task(seed=0)
    g.selector = selector.Selector.load()
    idx = train.nonzero().squeeze(1)

    def make(dropout):
        torch.manual_seed(0)
        model = gcn.Net(x.shape[1], 64, 3, dropout=dropout).to(dev())
        return model, gcn.make_optimizer(model, capturable=True)

    m1, o1 = make(0.0)
    eager = [float(gcn.train_epoch(m1, o1, x, g, y, idx)) for _ in range(13)]
    m2, o2 = make(0.0)
    step = gcn.CapturedEpoch(m2, o2, x, g, y, train, warmup=3)
    replay = [float(step()) for _ in range(10)]
    assert np.allclose(replay, eager[3:], rtol=0, atol=1e-5), (replay, eager[3:])

    m3, o3 = make(0.5)
    step = gcn.CapturedEpoch(m3, o3, x, g, y, train, warmup=3)
    losses = [float(step()) for _ in range(30)]
    assert np.isfinite(losses).all() and losses[-1] < losses[0]
    with pytest.raises(ValueError):
        gcn.CapturedEpoch(m3, gcn.make_optimizer(m3), x, g, y, train)


def test_sparse_features_product(oracle):
    """X @ W with X held as CSR (SpMM forward, SpMM with X^T for dW) against the dense
    product in FP64, and a captured epoch that reads the sparse features."""
    x, g, y, train, _ = gcn.synthetic_task(seed=1)
    feats = gcn.SparseFeatures(x)
    torch.manual_seed(3)
    W = (torch.randn(500, 64, device=dev()) * 0.1).requires_grad_(True)
    G = torch.randn(x.shape[0], 64, device=dev())
    out = feats.matmul(W)
    (out * G).sum().backward()
    xd, Wd, Gd = x.double(), W.detach().double(), G.double()
    ref = xd @ Wd
    scale = xd.abs() @ Wd.abs()
    assert ((out.double() - ref).abs() / scale.clamp_min(1e-30)).max() < 1e-5
    dref = xd.t() @ Gd
    dscale = xd.abs().t() @ Gd.abs()
    assert ((W.grad.double() - dref).abs() / dscale.clamp_min(1e-30)).max() < 1e-5
    # a training epoch on sparse features tracks the dense one
    torch.manual_seed(0)
    m1 = gcn.Net(500, 64, 3, dropout=0.0).to(dev())
    torch.manual_seed(0)
    m2 = gcn.Net(500, 64, 3, dropout=0.0).to(dev())
    o1, o2 = gcn.make_optimizer(m1), gcn.make_optimizer(m2, capturable=True)
    dense = [float(gcn.train_epoch(m1, o1, x, g, y, train)) for _ in range(8)]
    step = gcn.CapturedEpoch(m2, o2, feats, g, y, train, warmup=3)
    sparse = [float(step()) for _ in range(5)]
    assert np.allclose(sparse, dense[3:], rtol=0, atol=1e-4), (sparse, dense[3:])


@pytest.mark.parametrize("n,width,C", [(5000, 48, 47), (3001, 47, 47), (1, 8, 3), (700, 64, 64)])
def test_softmax_xent_matches_torch(n, width, C):
    """The fused loss kernels against log_softmax + nll_loss in fp32 on the same bf16 scores:
    the loss to fp32 rounding, the gradient to bf16 rounding, zero padding columns, the
    upstream gradient applied on the device, deterministic."""
    gen = torch.Generator(device=dev()).manual_seed(n + width)
    s = (torch.randn(n, width, generator=gen, device=dev()) * 3).to(torch.bfloat16)
    y = torch.randint(0, C, (n,), generator=gen, device=dev())
    x = s.detach().clone().requires_grad_(True)
    ref = torch.nn.functional.nll_loss(torch.nn.functional.log_softmax(x[:, :C].float(), 1), y)
    (3.0 * ref).backward()
    si = s.detach().clone().requires_grad_(True)
    loss = gcn.SoftmaxXent.apply(si, y, C)
    (3.0 * loss).backward()
    assert abs(loss.item() - ref.item()) <= 2e-6 * max(1.0, abs(ref.item()))
    g, gr = si.grad.float(), x.grad.float()
    assert torch.allclose(g[:, :C], gr[:, :C], rtol=8e-3, atol=1e-9)
    assert (g[:, C:] == 0).all()
    assert torch.equal(gcn.SoftmaxXent.apply(s, y, C), gcn.SoftmaxXent.apply(s, y, C))
    A.sync_status()


def test_softmax_xent_bad_label_is_flagged():
    s = torch.zeros(4, 8, dtype=torch.bfloat16, device=dev())
    y = torch.tensor([0, 1, 9, 2], device=dev())
    gcn.SoftmaxXent.apply(s, y, 8)
    with pytest.raises(A.NativeError) as e:
        A.sync_status()
    assert e.value.status == 1
