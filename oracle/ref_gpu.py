"""The reference's own CUDA kernels as a GPU comparator (TEST INFRASTRUCTURE).

``oracle/Makefile`` (target ``ref-cuda``) compiles gcn/pytorch-custom/spmm_kernel.cu and
sddmm.cu, unmodified, for sm_103a into device-only cubins under ``oracle/_ref/``. This module
loads them with the CUDA driver API (libcuda through ctypes, inside the CUDA context torch
made current) and launches them with the launch configurations of their host wrappers:

* ``spmm_cuda`` -- spmm_kernel.cu:425-458: spmm_test0 for k < 32 (block k x 128/k), spmm_test1
  for k < 64 (32 x 4, 1 KB shared), spmm_test2 otherwise (32 x 8, 2 KB shared, 64-column
  tiles); out = A * dense (overwrite);
* ``sddmm_cuda_csr`` -- sddmm.cu:459-483: sddmmCSR2Scale<float> for even K (16 x 4 blocks, four
  entries per block row), out[e] = <D1[row(e)], D2[col(e)]>.

Only tests and ``bench.py --impl reference`` use it, as the same-box GPU figure of the
reference; the product package never imports it. Inputs are restricted to what the kernels
handle in bounds, checked by reading them: sddmmCSR2Scale's blocks past nnz / 16 (used when
nnz is not a multiple of 16) start their second warp 32 columns into the row and read up to
32 floats past its end, so ``sddmm_cuda_csr`` refuses such an nnz; its int offsets need
rows * K < 2^31; odd K (sddmmCSR1Scale) is not wrapped.
"""
from __future__ import annotations

import ctypes
import os

_HERE = os.path.dirname(os.path.abspath(__file__))
CUBINS = {"spmm": os.path.join(_HERE, "_ref", "ref_spmm_kernel.cubin"),
          "sddmm": os.path.join(_HERE, "_ref", "ref_sddmm.cubin")}
# Itanium-mangled names of the kernels (the signatures of spmm_kernel.cu:210-309 and
# sddmm.cu:255-257, instantiated for float by sddmm_cuda_csr)
_NAMES = {"spmm_test0": "_Z10spmm_test0iiPiS_PfS0_S0_",
          "spmm_test1": "_Z10spmm_test1iiPiS_PfS0_S0_",
          "spmm_test2": "_Z10spmm_test2iiPiS_PfS0_S0_",
          "sddmmCSR2Scale": "_Z14sddmmCSR2ScaleIfEviimPiS0_PT_S2_S2_"}

_cuda = None
_funcs = {}


def available() -> bool:
    return all(os.path.exists(p) for p in CUBINS.values())


def _drv():
    global _cuda
    if _cuda is None:
        lib = ctypes.CDLL("libcuda.so.1")
        lib.cuModuleLoad.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_char_p]
        lib.cuModuleGetFunction.argtypes = [ctypes.POINTER(ctypes.c_void_p), ctypes.c_void_p,
                                            ctypes.c_char_p]
        lib.cuLaunchKernel.argtypes = [ctypes.c_void_p] + [ctypes.c_uint] * 7 + \
            [ctypes.c_void_p, ctypes.POINTER(ctypes.c_void_p), ctypes.c_void_p]
        lib.cuCtxGetCurrent.argtypes = [ctypes.POINTER(ctypes.c_void_p)]
        _cuda = lib
    return _cuda


def _check(rc, what):
    if rc != 0:
        raise RuntimeError(f"CUDA driver call {what} failed with {rc}")


def _func(kernel: str, device_index: int):
    key = (kernel, device_index)
    if key not in _funcs:
        import torch
        torch.cuda.set_device(device_index)
        torch.zeros(1, device=f"cuda:{device_index}")  # the runtime's context is current
        lib = _drv()
        ctx = ctypes.c_void_p()
        _check(lib.cuCtxGetCurrent(ctypes.byref(ctx)), "cuCtxGetCurrent")
        if not ctx.value:
            raise RuntimeError("no current CUDA context")
        mod = ctypes.c_void_p()
        path = CUBINS["sddmm" if kernel.startswith("sddmm") else "spmm"]
        _check(lib.cuModuleLoad(ctypes.byref(mod), path.encode()), "cuModuleLoad")
        f = ctypes.c_void_p()
        _check(lib.cuModuleGetFunction(ctypes.byref(f), mod, _NAMES[kernel].encode()),
               "cuModuleGetFunction")
        _funcs[key] = f
    return _funcs[key]


def _launch(kernel, device_index, grid, block, smem, stream, args):
    ptrs = (ctypes.c_void_p * len(args))(*[ctypes.cast(ctypes.byref(a), ctypes.c_void_p) for a in args])
    _check(_drv().cuLaunchKernel(_func(kernel, device_index), *grid, *block, smem,
                                 ctypes.c_void_p(stream), ptrs, None), f"cuLaunchKernel {kernel}")


def spmm_cuda(rowptr, colind, values, dense, out=None):
    """The reference's spmm_cuda (spmm_kernel.cu:425-458) on the current stream."""
    import torch
    m = rowptr.numel() - 1
    k = dense.shape[1]
    if out is None:
        out = torch.empty((m, k), dtype=torch.float32, device=dense.device)
    stream = torch.cuda.current_stream(dense.device).cuda_stream
    args = [ctypes.c_int(m), ctypes.c_int(k), ctypes.c_void_p(rowptr.data_ptr()),
            ctypes.c_void_p(colind.data_ptr()), ctypes.c_void_p(values.data_ptr()),
            ctypes.c_void_p(dense.data_ptr()), ctypes.c_void_p(out.data_ptr())]
    dev = dense.device.index
    if k < 32:
        rpb = 128 // k
        _launch("spmm_test0", dev, ((m + rpb - 1) // rpb, 1, 1), (k, rpb, 1), 0, stream, args)
    elif k < 64:
        _launch("spmm_test1", dev, ((m + 3) // 4, (k + 31) // 32, 1), (32, 4, 1), 32 * 4 * 8,
                stream, args)
    else:
        _launch("spmm_test2", dev, ((m + 7) // 8, (k + 63) // 64, 1), (32, 8, 1), 32 * 8 * 8,
                stream, args)
    return out


def sddmm_cuda_csr(rowptr, colind, D1, D2, out=None):
    """The reference's sddmm_cuda_csr (sddmm.cu:459-483, even K) on the current stream."""
    import torch
    m, k = D1.shape
    nnz = colind.numel()
    if k % 2:
        raise ValueError("odd K (sddmmCSR1Scale) is not wrapped")
    if nnz % 16:
        raise ValueError("nnz must be a multiple of 16: the kernel's blocks past nnz / 16 read "
                         "past the end of a row")
    if max(m, D2.shape[0]) * k >= 2 ** 31:
        raise ValueError("the kernel's int offsets need rows * K < 2^31")
    if out is None:
        out = torch.empty(nnz, dtype=torch.float32, device=D1.device)
    stream = torch.cuda.current_stream(D1.device).cuda_stream
    args = [ctypes.c_int(m), ctypes.c_int(k), ctypes.c_ulong(nnz),
            ctypes.c_void_p(rowptr.data_ptr()), ctypes.c_void_p(colind.data_ptr()),
            ctypes.c_void_p(D1.data_ptr()), ctypes.c_void_p(D2.data_ptr()),
            ctypes.c_void_p(out.data_ptr())]
    _launch("sddmmCSR2Scale", D1.device.index, (nnz // 16 + (nnz & 15), 1, 1), (16, 4, 1), 0,
            stream, args)
    return out
