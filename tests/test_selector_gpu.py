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
