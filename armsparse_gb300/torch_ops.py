"""Loader of the in-tree PyTorch extension module ``spmm`` (armsparse_gb300/csrc/torch_spmm.cpp).

``from armsparse_gb300.torch_ops import spmm`` replaces the reference's
``spmm = load(name='spmm', sources=['spmm.cpp'], ...)`` (gcn/pytorch-custom/op.py:6): same
module name, same ``csr_spmm(rowptr, colind, values, dense)``, CUDA tensors. The module is
built by ``armsparse_gb300.build`` (``__graft_entry__.build()``); importing this file raises if
it is missing -- there is no CPU fallback.
"""
from __future__ import annotations

import glob
import importlib.util
import os

import torch  # noqa: F401  (the extension needs torch's libraries loaded first)

_PKG = os.path.dirname(os.path.abspath(__file__))


def _load():
    found = sorted(glob.glob(os.path.join(_PKG, "spmm*.so")))
    if not found:
        raise ImportError("the `spmm` torch extension is not built "
                          "(python -m armsparse_gb300.build)")
    spec = importlib.util.spec_from_file_location("spmm", found[0])
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


spmm = _load()
