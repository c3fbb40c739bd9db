"""The bounded-wait failure path on the GPU, taken without a fault or a hang: with the
context's spin limit at 0, the bulk-copy SpMM's wait for a gathered row (and the long-row
kernel's wait for a pipeline stage) gives up at once;
the call then reports AS_ERR_TIMEOUT through the status word, every copy it issued has landed
before its warps leave, and the same context computes the right result once the limit is
back to its default."""
import ctypes

import numpy as np
import pytest
import torch

import armsparse_gb300 as A
from armsparse_gb300 import _native as N
from armsparse_gb300 import synthetic as S
from gpu_util import bits, csr_dev, dev, to_dev

pytestmark = pytest.mark.gpu


def _bulk_variant():
    names = A.spmm_variants(torch.float32)
    return names.index("bulk_lb16_s8") + 1


def test_wait_timeout_reported_then_context_recovers(oracle):
    lib = N.load()
    ctx = N.Context(0)
    try:
        a = S.uniform_csr(2048, 1024, 40000, seed=81)
        B = S.dense_uniform((1024, 256), 82)
        rp, ci, v = csr_dev(a)
        Bd = to_dev(B)
        C = torch.full((2048, 256), 3.0, device=dev())
        var = _bulk_variant()
        stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

        def call():
            return lib.as_spmm_csr_f32(ctx.handle, 2048, 1024, 256, a.nnz, rp.data_ptr(),
                                       ci.data_ptr(), v.data_ptr(), Bd.data_ptr(), 256,
                                       C.data_ptr(), 256, ctypes.c_float(0.0), var, stream)

        assert lib.as_ctx_set_spin_limit(ctx.handle, 0) == 0
        assert call() == 0  # the launch itself succeeds
        st = lib.as_ctx_sync_status(ctx.handle, stream)
        assert st == 5  # AS_ERR_TIMEOUT
        # the warps that gave up left their rows unwritten
        assert (C == 3.0).any()

        assert lib.as_ctx_set_spin_limit(ctx.handle, 1 << 22) == 0
        assert call() == 0
        assert lib.as_ctx_sync_status(ctx.handle, stream) == 0
        ref = oracle.spmm_fma_chain_f32(a.rowptr, a.colind, a.val, B)
        assert np.array_equal(bits(C), bits(ref))
        assert lib.as_ctx_set_spin_limit(None, 0) == 1  # AS_ERR_INVALID_VALUE
    finally:
        ctx.close()


def test_long_row_wait_timeout_then_recovers(oracle):
    """The same for the long-row kernel's pipeline (a row of 20,000 entries): its consumer's
    wait for a stage gives up at once with the limit at 0, the producers see the abort and
    leave, the row stays unwritten and AS_ERR_TIMEOUT is reported; with the default limit the
    same context gives the bit-exact result."""
    lib = N.load()
    ctx = N.Context(0)
    try:
        rng = np.random.default_rng(83)
        lens = rng.integers(0, 30, 1000)
        lens[17] = 20000
        rp_h = np.zeros(1001, np.int32)
        np.cumsum(lens, out=rp_h[1:])
        ci_h = np.concatenate([np.sort(rng.choice(30000, l, replace=False)) for l in lens]).astype(np.int32)
        v_h = rng.uniform(-1, 1, ci_h.size).astype(np.float32)
        B = S.dense_uniform((30000, 64), 84)
        rp, ci, v, Bd = to_dev(rp_h), to_dev(ci_h), to_dev(v_h), to_dev(B)
        C = torch.full((1000, 64), 3.0, device=dev())
        stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)

        def call():
            return lib.as_spmm_csr_f32(ctx.handle, 1000, 30000, 64, ci_h.size, rp.data_ptr(),
                                       ci.data_ptr(), v.data_ptr(), Bd.data_ptr(), 64,
                                       C.data_ptr(), 64, ctypes.c_float(0.0), 0, stream)

        assert lib.as_ctx_set_spin_limit(ctx.handle, 0) == 0
        assert call() == 0
        assert lib.as_ctx_sync_status(ctx.handle, stream) == 5  # AS_ERR_TIMEOUT
        assert bool((C[17] == 3.0).all())  # the long row was left unwritten
        assert lib.as_ctx_set_spin_limit(ctx.handle, 1 << 22) == 0
        assert call() == 0
        assert lib.as_ctx_sync_status(ctx.handle, stream) == 0
        ref = oracle.spmm_fma_chain_f32(rp_h, ci_h, v_h, B)
        assert np.array_equal(bits(C), bits(ref))
    finally:
        ctx.close()
