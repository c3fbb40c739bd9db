"""ctypes binding of ``libarmsparse_gpu.so`` (the C ABI in ``include/armsparse_gpu.h``).

There is no fallback: if the library is missing or fails to load, importing the ops raises.
Build it with ``python -m armsparse_gb300.build`` (or ``__graft_entry__.build()``).
"""
from __future__ import annotations

import ctypes
import os
import threading

_PKG = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_PKG, "libarmsparse_gpu.so")

AS_OK = 0
STATUS_NAMES = {
    0: "AS_OK", 1: "AS_ERR_INVALID_VALUE", 2: "AS_ERR_INVALID_CSR", 3: "AS_ERR_UNSUPPORTED",
    4: "AS_ERR_CUDA", 5: "AS_ERR_TIMEOUT", 6: "AS_ERR_ALLOC",
}

# name -> (restype, argtypes) for every entry point of include/armsparse_gpu.h
_P, _I, _L, _F, _U64 = (ctypes.c_void_p, ctypes.c_int, ctypes.c_long, ctypes.c_float,
                        ctypes.c_uint64)
SIGNATURES = {
    "as_ctx_create": (_I, [ctypes.POINTER(_P), _I]),
    "as_ctx_destroy": (_I, [_P]),
    "as_ctx_sync_status": (_I, [_P, _P]),
    "as_last_error": (ctypes.c_char_p, []),
    "as_status_string": (ctypes.c_char_p, [_I]),
    "as_ctx_launch_count": (_U64, [_P]),
    "as_ctx_set_spin_limit": (_I, [_P, ctypes.c_uint]),
    "as_csr_validate": (_I, [_P, _I, _I, _I, _P, _P, _I, _P]),
    "as_spmm_csr_f32": (_I, [_P, _I, _I, _I, _I, _P, _P, _P, _P, _L, _P, _L, _F, _I, _P]),
    "as_spmm_csr_bf16": (_I, [_P, _I, _I, _I, _I, _P, _P, _P, _P, _L, _P, _L, _F, _I, _P]),
    "as_softmax_xent_bf16": (_I, [_P, _I, _I, _P, _L, _P, _P, _P, _P]),
    "as_softmax_xent_bwd_bf16": (_I, [_P, _I, _I, _P, _L, _P, _P, _P, _P, _L, _I, _P]),
    "as_spmm_csr_bf16_out16": (_I, [_P, _I, _I, _I, _I, _P, _P, _P, _P, _L, _P, _L, _I, _I, _P]),
    "as_spmm_sddmm_csr_bf16_out16": (_I, [_P, _I, _I, _I, _I, _P, _P, _P, _P, _L, _P, _L, _P,
                                         _L, _P, _P, _I, _P]),
    "as_spmm_sddmm_csr_f32": (_I, [_P, _I, _I, _I, _I, _P, _P, _P, _P, _L, _P, _L, _F, _P, _L,
                                  _P, _P, _I, _P]),
    "as_spmm_sddmm_csr_bf16": (_I, [_P, _I, _I, _I, _I, _P, _P, _P, _P, _L, _P, _L, _F, _P, _L,
                                   _P, _P, _I, _P]),
    "as_spmm_csr_reduce_f32": (_I, [_P, _I, _I, _I, _I, _P, _P, _P, _P, _L, _P, _L, _I, _P]),
    "as_spgemm_csr_dense_f32": (_I, [_P, _I, _I, _I, _I, _P, _P, _P, _I, _P, _P, _P, _P, _L, _F,
                                     _P]),
    "as_spmm_variant_count": (_I, [_I]),
    "as_spmm_variant_name": (ctypes.c_char_p, [_I, _I]),
    "as_spmm_variant_supported": (_I, [_I, _I, _I, _L, _L, _P, _P]),
    "as_spmm_default_variant": (_I, [_I, _I, _I, _I, _I, _L, _L, _P, _P]),
    "as_spmv_csr_f32": (_I, [_P, _I, _I, _I, _P, _P, _P, _P, _P, _F, _P]),
    "as_spmv_vcsr4_f32": (_I, [_P, _I, _I, _I, _P, _P, _P, _P, _P, _F, _P]),
    "as_sddmm_csr_f32": (_I, [_P, _I, _I, _I, _I, _P, _P, _P, _P, _L, _P, _L, _P, _P]),
    "as_sddmm_csr_bf16": (_I, [_P, _I, _I, _I, _I, _P, _P, _P, _P, _L, _P, _L, _P, _P]),
    "as_sddmm_csr_bf16x3": (_I, [_P, _I, _I, _I, _I, _P, _P, _P, _P, _L, _P, _L, _P, _P]),
    "as_csr2csc_static": (_I, [_I, _I, _I, _P, _P, _P, _P, _P, _P, _P]),
    "as_sddmm_csr_bf16x3_v": (_I, [_P, _I, _I, _I, _I, _P, _P, _P, _P, _L, _P, _L, _P, _I, _P]),
    "as_sddmm_bf16x3_variant_count": (_I, []),
    "as_sddmm_coo_f32": (_I, [_P, _I, _I, _I, _I, _P, _P, _P, _P, _L, _P, _L, _P, _P]),
    "as_csr2csc": (_I, [_P, _I, _I, _I, _P, _P, _P, _P, _P, _P, _P]),
    "as_gather_f32": (_I, [_P, _L, _L, _P, _P, _P, _P]),
    "as_csr2csc_perm": (_I, [_P, _I, _I, _I, _P, _P, _P, _P, _P, _P]),
    "as_spmm_csr_f64": (_I, [_P, _I, _I, _I, _I, _P, _P, _P, _P, _L, _P, _L, ctypes.c_double, _P]),
    "as_sddmm_csr_f64": (_I, [_P, _I, _I, _I, _I, _P, _P, _P, _P, _L, _P, _L, _P, _P]),
    "as_f32_to_bf16": (_I, [_P, _L, _P, _P, _P]),
    "as_dense_to_csr_count": (_I, [_P, _I, _I, _P, _L, _P, _P]),
    "as_dense_to_csr_fill": (_I, [_P, _I, _I, _P, _L, _P, _P, _P, _P]),
    "as_spmm_vcsr4_f32": (_I, [_P, _I, _I, _I, _I, _P, _P, _P, _P, _L, _P, _L, _F, _P]),
    "as_csr_to_rowpair_count": (_I, [_P, _I, _I, _P, _P, _P, _P]),
    "as_csr_to_rowpair_fill": (_I, [_P, _I, _I, _P, _P, _P, _P, _P, _P, _P, _P]),
    "as_spmm_rowpair_f32": (_I, [_P, _I, _I, _I, _I, _P, _P, _P, _P, _P, _L, _P, _L, _F, _P]),
    "as_csr_to_vcsr4_count": (_I, [_P, _I, _I, _P, _P, _P, _P]),
    "as_csr_to_vcsr4_fill": (_I, [_P, _I, _I, _P, _P, _P, _P, _P, _P, _P]),
    # include/armsparse_mlp.h
    "as_mlp_linear_fwd": (_I, [_P, _I, _I, _I, _P, _P, _P, _P, _I, _P]),
    "as_mlp_linear_bwd": (_I, [_P, _I, _I, _I, _P, _P, _P, _P, _P, _P, _P, _P]),
    "as_mlp_softmax_xent": (_I, [_P, _I, _I, _P, _P, _P, _P, _F, _P]),
    "as_mlp_adam": (_I, [_P, _L, _P, _P, _P, _P, _F, _F, _F, _F, _F, _I, _P]),
}

_lock = threading.Lock()
_lib = None


class NativeError(RuntimeError):
    def __init__(self, status: int, where: str, msg: str):
        self.status = status
        super().__init__(f"{where}: {STATUS_NAMES.get(status, status)}: {msg}")


def load(path: str | None = None) -> ctypes.CDLL:
    """Load the C-ABI library (raises if it is absent: there is no CPU fallback)."""
    global _lib
    with _lock:
        if _lib is None:
            p = path or LIB_PATH
            if not os.path.exists(p):
                raise ImportError(
                    f"{p} is missing: build the CUDA library first "
                    "(python -m armsparse_gb300.build)")
            lib = ctypes.CDLL(p)
            for name, (res, args) in SIGNATURES.items():
                fn = getattr(lib, name)
                fn.restype = res
                fn.argtypes = args
            _lib = lib
    return _lib


def check(status: int, where: str) -> None:
    if status != AS_OK:
        msg = load().as_last_error().decode(errors="replace")
        raise NativeError(status, where, msg)


class Context:
    """Owns an ``as_ctx`` (device status word + scratch arena) for one device."""

    def __init__(self, device: int = 0):
        self.device = device
        h = ctypes.c_void_p()
        check(load().as_ctx_create(ctypes.byref(h), device), "as_ctx_create")
        self.handle = h

    def sync_status(self, stream: int | None = None) -> None:
        check(load().as_ctx_sync_status(self.handle, stream), "as_ctx_sync_status")

    @property
    def launches(self) -> int:
        return int(load().as_ctx_launch_count(self.handle))

    def close(self) -> None:
        if self.handle:
            load().as_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


_tls = threading.local()


def context(device: int = 0) -> Context:
    """Per-thread, per-device default context."""
    ctxs = getattr(_tls, "ctxs", None)
    if ctxs is None:
        ctxs = _tls.ctxs = {}
    c = ctxs.get(device)
    if c is None:
        c = ctxs[device] = Context(device)
    return c


def total_launches() -> int:
    """Launches through every default context of this thread."""
    return sum(c.launches for c in getattr(_tls, "ctxs", {}).values())
