"""Helpers shared by the GPU tests (device copies of seeded CSR inputs)."""
import numpy as np
import torch


def dev():
    return torch.device("cuda", 0)


def to_dev(a, dtype=None):
    t = torch.from_numpy(np.ascontiguousarray(a))
    if dtype is not None:
        t = t.to(dtype)
    return t.to(dev())


def csr_dev(a):
    return to_dev(a.rowptr), to_dev(a.colind), to_dev(a.val)


def bits(t):
    a = t.detach().cpu().numpy() if isinstance(t, torch.Tensor) else np.asarray(t)
    return a.view(np.uint32) if a.dtype == np.float32 else a
