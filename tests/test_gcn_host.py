"""Host-side pieces of the GCN path that need no GPU."""
import torch
import torch.nn.functional as F

from armsparse_gb300 import gcn


def test_nll_mean_matches_nll_loss():
    g = torch.Generator().manual_seed(0)
    logits = torch.randn(5000, 47, generator=g, dtype=torch.float64)
    y = torch.randint(0, 47, (5000,), generator=g)
    a = F.log_softmax(logits.clone().requires_grad_(True), dim=1)
    b_in = logits.clone().requires_grad_(True)
    b = F.log_softmax(b_in, dim=1)
    ref = F.nll_loss(a, y)
    got = gcn.nll_mean(b, y)
    assert torch.allclose(got, ref, rtol=1e-12, atol=0)
    got.backward()
    la = logits.clone().requires_grad_(True)
    F.nll_loss(F.log_softmax(la, dim=1), y).backward()
    assert torch.allclose(b_in.grad, la.grad, rtol=1e-12, atol=1e-15)
