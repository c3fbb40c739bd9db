"""The selector's network kernels (include/armsparse_mlp.h) against the float64 numpy oracle,
a finite-difference check of the whole network gradient, and the trained selector against the
autotuner and against the fixed width rule."""
import ctypes
import json
import os

import numpy as np
import pytest
import torch

from armsparse_gb300 import _native as N
from armsparse_gb300 import selector as SEL

pytestmark = pytest.mark.gpu


def _lib():
    return SEL._Lib(torch.device("cuda", 0))


def test_linear_forward_backward_against_oracle(oracle):
    rng = np.random.default_rng(0)
    B, I, O = 37, 23, 19
    X = rng.standard_normal((B, I)).astype(np.float32)
    W = rng.standard_normal((O, I)).astype(np.float32)
    b = rng.standard_normal(O).astype(np.float32)
    dY = rng.standard_normal((B, O)).astype(np.float32)
    relu_in = np.maximum(X, 0)
    d = torch.device("cuda", 0)
    t = lambda a: torch.from_numpy(a).to(d)
    Xd, Wd, bd, dYd, Rd = t(X), t(W), t(b), t(dY), t(relu_in)
    L = _lib()
    for relu in (0, 1):
        Y = torch.empty(B, O, device=d)
        L.call("as_mlp_linear_fwd", B, I, O, Xd.data_ptr(), Wd.data_ptr(), bd.data_ptr(), Y.data_ptr(), relu)
        assert np.allclose(Y.cpu().numpy(), oracle.mlp_linear_fwd(X, W, b, bool(relu)), rtol=1e-5, atol=1e-5)
    dX, dW, db = torch.empty(B, I, device=d), torch.empty(O, I, device=d), torch.empty(O, device=d)
    L.call("as_mlp_linear_bwd", B, I, O, dYd.data_ptr(), Rd.data_ptr(), Wd.data_ptr(), Rd.data_ptr(),
           dX.data_ptr(), dW.data_ptr(), db.data_ptr())
    rX, rW, rb = oracle.mlp_linear_bwd(dY, relu_in, W, relu_in=relu_in)
    assert np.allclose(dX.cpu().numpy(), rX, rtol=1e-5, atol=1e-5)
    assert np.allclose(dW.cpu().numpy(), rW, rtol=1e-5, atol=1e-4)
    assert np.allclose(db.cpu().numpy(), rb, rtol=1e-5, atol=1e-5)


def test_softmax_xent_and_adam_against_oracle(oracle):
    rng = np.random.default_rng(1)
    Z = rng.standard_normal((50, 20)).astype(np.float32) * 3
    T = rng.random((50, 20)).astype(np.float32)
    T /= T.sum(axis=1, keepdims=True)
    d = torch.device("cuda", 0)
    Zd, Td = torch.from_numpy(Z).to(d), torch.from_numpy(T).to(d)
    loss, dZ = torch.empty(50, device=d), torch.empty(50, 20, device=d)
    L = _lib()
    L.call("as_mlp_softmax_xent", 50, 20, Zd.data_ptr(), Td.data_ptr(), loss.data_ptr(), dZ.data_ptr(),
           ctypes.c_float(0.02))
    rl, rd = oracle.mlp_softmax_xent(Z, T, 0.02)
    assert np.allclose(loss.cpu().numpy(), rl, rtol=1e-5, atol=1e-5)
    assert np.allclose(dZ.cpu().numpy(), rd, rtol=1e-5, atol=1e-7)
    p = rng.standard_normal(100).astype(np.float32)
    g = rng.standard_normal(100).astype(np.float32)
    pd, gd = torch.from_numpy(p).to(d), torch.from_numpy(g).to(d)
    m, v = torch.zeros(100, device=d), torch.zeros(100, device=d)
    rp, rm, rv = p.astype(np.float64), np.zeros(100), np.zeros(100)
    for step in (1, 2, 3):
        L.call("as_mlp_adam", 100, pd.data_ptr(), gd.data_ptr(), m.data_ptr(), v.data_ptr(),
               ctypes.c_float(1e-2), ctypes.c_float(0.9), ctypes.c_float(0.999), ctypes.c_float(1e-8),
               ctypes.c_float(1e-3), step)
        rp, rm, rv = oracle.mlp_adam(rp, g.astype(np.float64), rm, rv, 1e-2, 0.9, 0.999, 1e-8, 1e-3, step)
    assert np.allclose(pd.cpu().numpy(), rp, rtol=1e-5, atol=1e-6)


def test_network_gradient_against_finite_differences(oracle):
    """Backward of the whole 3-layer network (GPU kernels) vs central differences of the loss
    computed by the float64 oracle."""
    rng = np.random.default_rng(2)
    net = SEL.MLP(11, 7, hidden=9, seed=3)
    X = rng.standard_normal((16, 11)).astype(np.float32)
    T = rng.random((16, 7)).astype(np.float32)
    T /= T.sum(axis=1, keepdims=True)
    d = net.device
    loss, grads = net.loss_and_grads(torch.from_numpy(X).to(d), torch.from_numpy(T).to(d))
    W = net.host_weights()

    def f(Ws):
        h = X.astype(np.float64)
        for i in range(3):
            h = oracle.mlp_linear_fwd(h, Ws[2 * i], Ws[2 * i + 1], relu=i < 2)
        return oracle.mlp_softmax_xent(h, T)[0].mean()

    assert abs(float(loss) - f(W)) < 1e-5
    for pi in range(6):
        g = grads[pi].cpu().numpy().astype(np.float64).ravel()
        flat = W[pi].ravel()
        for j in rng.choice(flat.size, min(6, flat.size), replace=False):
            Wp = [w.copy() for w in W]
            Wm = [w.copy() for w in W]
            Wp[pi].ravel()[j] += 1e-5
            Wm[pi].ravel()[j] -= 1e-5
            num = (f(Wp) - f(Wm)) / 2e-5
            assert abs(num - g[j]) < 1e-4 + 1e-3 * abs(num), (pi, j, num, g[j])


def test_trained_selector_beats_width_rule():
    """Train on a small sweep, evaluate on held-out matrices: the network's pick must be closer
    to the autotuner's best than the fixed width rule is (the gain the network brings)."""
    cfgs = SEL.sweep_configs(48, seed=11, max_nnz=1_500_000)
    for c in cfgs:
        c["n"] = min(c["n"], 200_000)
    recs = SEL.sweep(cfgs, reps=2)
    train, test = recs[:36], recs[36:]
    model = SEL.train(train, epochs=1500)
    ev = SEL.evaluate(model, test)
    assert ev["mlp_geomean"] <= ev["rule_geomean"], ev
    assert ev["mlp_geomean"] < 1.6, ev


def test_sddmm_path_choice_against_autotuner():
    """The learned SDDMM path choice (CUDA-core FP32 or a tcgen05 split-bf16 variant) on
    held-out seeded patterns the model was not trained on (another seed): its pick's time
    within 1.1x of the exhaustive autotuner's best (geometric mean), and at least as good as
    always taking the CUDA-core path -- the only kind the reference has, chosen by K % 4 and
    K % 2 alone (gcn/pytorch-custom/sddmm.cu:438-455). Every path agrees with FP64."""
    if not os.path.exists(SEL.DEFAULT_SDDMM_MODEL):
        pytest.skip("no SDDMM selector model file")
    from armsparse_gb300 import sparse as S
    from armsparse_gb300 import tuner
    sel = SEL.SddmmSelector.load()
    cfgs = SEL.sddmm_sweep_configs(16, seed=777, max_nnz=3_000_000,
                                   max_dense_bytes=256 << 20)
    recs = SEL.sddmm_sweep(cfgs, reps=3)
    ev = SEL.evaluate_sddmm(sel.model, recs)
    assert ev["mlp_geomean"] <= 1.1, ev
    assert ev["mlp_geomean"] <= ev["simt_geomean"] + 1e-9, ev
    # the API's "auto" takes the model's pick and stays within the accuracy of either path
    d = torch.device("cuda", 0)
    cfg = cfgs[0]
    rp, ci = SEL.make_sddmm_pattern(cfg, d)
    g = torch.Generator(device=d).manual_seed(5)
    X = torch.randn(cfg["M"], cfg["K"], generator=g, device=d)
    Y = torch.randn(cfg["N"], cfg["K"], generator=g, device=d)
    out = S.sddmm(rp, ci, X, Y, tensor_cores="auto")
    r64 = S.sddmm(rp, ci, X.double(), Y.double())
    s64 = S.sddmm(rp, ci, X.double().abs(), Y.double().abs())
    err = ((out.double() - r64).abs() / torch.maximum(r64.abs(), s64)).max().item()
    assert err < 3e-5
    assert S.sddmm_path(rp, ci, cfg["N"], cfg["K"]) in tuner.sddmm_paths()
