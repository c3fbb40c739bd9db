"""Tensor-level API over the C ABI: CUDA tensors in, CUDA tensors out, on torch's current
stream. Every function checks dtypes, devices and contiguity and raises on anything else;
nothing here computes on the CPU.
"""
from __future__ import annotations

import torch

from . import _native as N


def _ptr(t: torch.Tensor | None):
    return None if t is None else t.data_ptr()


def _stream(device: torch.device) -> int:
    return torch.cuda.current_stream(device).cuda_stream


def _dev(*ts) -> torch.device:
    dev = None
    for t in ts:
        if t is None:
            continue
        if not t.is_cuda:
            raise ValueError("armsparse_gb300 works on CUDA tensors only (no CPU path)")
        if dev is None:
            dev = t.device
        elif t.device != dev:
            raise ValueError("all tensors must be on the same device")
    if dev is None:
        raise ValueError("no tensor given")
    return dev


def _need(t: torch.Tensor, dtype, name: str, ndim: int | None = None):
    if t.dtype != dtype:
        raise TypeError(f"{name} must be {dtype}, got {t.dtype}")
    if not t.is_contiguous():
        raise ValueError(f"{name} must be contiguous")
    if ndim is not None and t.dim() != ndim:
        raise ValueError(f"{name} must have {ndim} dims")


def _csr(rowptr, colind):
    _need(rowptr, torch.int32, "rowptr", 1)
    _need(colind, torch.int32, "colind", 1)
    return rowptr.numel() - 1, colind.numel()


def validate_csr(rowptr, colind, n_cols: int, require_sorted: bool = False) -> None:
    """Synchronous device-side CSR check; raises NativeError(AS_ERR_INVALID_CSR) if bad."""
    dev = _dev(rowptr, colind)
    M, nnz = _csr(rowptr, colind)
    ctx = N.context(dev.index)
    N.check(N.load().as_csr_validate(ctx.handle, M, n_cols, nnz, _ptr(rowptr), _ptr(colind),
                                     int(require_sorted), _stream(dev)), "as_csr_validate")


def sync_status(device=None) -> None:
    """Wait for the current stream and raise if a kernel saw malformed input since the last
    check."""
    dev = torch.device("cuda", torch.cuda.current_device()) if device is None else torch.device(device)
    N.context(dev.index).sync_status(_stream(dev))


def spmm(rowptr, colind, val, B, C=None, beta: float = 0.0, variant: int = 0,
         out_dtype: torch.dtype = torch.float32, relu: bool = False):
    """C = A*B + beta*C with A (M x K) in CSR. fp32 val/B -> fp32 path (bit-identical to the
    reference's rowBaseSpmm3 for row-split variants); bf16 val/B -> bf16 storage with fp32
    accumulation. C is fp32 (allocated when None); with bf16 val/B, out_dtype=torch.bfloat16
    gives C in bf16 (the fp32 result rounded to nearest even, beta 0) without a second pass,
    and relu=True (bf16 output only) stores max(C, 0) in the same pass."""
    dev = _dev(rowptr, colind, val, B, C)
    M, nnz = _csr(rowptr, colind)
    if B.dim() != 2:
        raise ValueError("B must be 2-D")
    if B.stride(1) != 1:
        raise ValueError("B must be row-major with unit column stride")
    K, Ncols = B.shape
    ldb = B.stride(0) if K > 1 else Ncols
    if out_dtype == torch.bfloat16:
        return _spmm_bf16_out16(rowptr, colind, val, B, C, beta, variant, dev, M, nnz, K, Ncols,
                                ldb, relu)
    if out_dtype != torch.float32:
        raise TypeError("out_dtype must be float32 or bfloat16")
    if relu:
        raise ValueError("relu is an epilogue of the bf16 output")
    if val.dtype == torch.float32 and B.dtype == torch.float32:
        fn, dname = N.load().as_spmm_csr_f32, "as_spmm_csr_f32"
    elif val.dtype == torch.bfloat16 and B.dtype == torch.bfloat16:
        fn, dname = N.load().as_spmm_csr_bf16, "as_spmm_csr_bf16"
    elif val.dtype == torch.float64 and B.dtype == torch.float64:
        return _spmm_f64(rowptr, colind, val, B, C, beta)
    else:
        raise TypeError("val and B must both be float32, both bfloat16 or both float64")
    _need(val, val.dtype, "val", 1)
    if val.numel() != nnz:
        raise ValueError("val and colind lengths differ")
    if C is None:
        if beta != 0.0:
            raise ValueError("beta != 0 needs C")
        C = torch.empty((M, Ncols), dtype=torch.float32, device=dev)
    else:
        if C.dtype != torch.float32 or C.dim() != 2 or C.shape != (M, Ncols) or C.stride(1) != 1:
            raise ValueError("C must be float32 (M, N) row-major")
    ldc = C.stride(0) if M > 1 else Ncols
    ctx = N.context(dev.index)
    N.check(fn(ctx.handle, M, K, Ncols, nnz, _ptr(rowptr), _ptr(colind), _ptr(val), _ptr(B),
               ldb, _ptr(C), ldc, float(beta), int(variant), _stream(dev)), dname)
    return C


def _spmm_bf16_out16(rowptr, colind, val, B, C, beta, variant, dev, M, nnz, K, Ncols, ldb,
                     relu=False):
    if val.dtype != torch.bfloat16 or B.dtype != torch.bfloat16:
        raise TypeError("a bf16 output needs bf16 val and B")
    if beta != 0.0:
        raise ValueError("a bf16 output is written with beta = 0")
    _need(val, torch.bfloat16, "val", 1)
    if val.numel() != nnz:
        raise ValueError("val and colind lengths differ")
    if C is None:
        C = torch.empty((M, Ncols), dtype=torch.bfloat16, device=dev)
    elif C.dtype != torch.bfloat16 or C.dim() != 2 or C.shape != (M, Ncols) or C.stride(1) != 1:
        raise ValueError("C must be bfloat16 (M, N) row-major")
    ldc = C.stride(0) if M > 1 else Ncols
    ctx = N.context(dev.index)
    N.check(N.load().as_spmm_csr_bf16_out16(ctx.handle, M, K, Ncols, nnz, _ptr(rowptr),
                                            _ptr(colind), _ptr(val), _ptr(B), ldb, _ptr(C), ldc,
                                            int(bool(relu)), int(variant), _stream(dev)),
            "as_spmm_csr_bf16_out16")
    return C


def _spmm_f64(rowptr, colind, val, B, C, beta):
    """float64 SpMM (gradient checks only)."""
    dev = B.device
    M, nnz = _csr(rowptr, colind)
    K, Ncols = B.shape
    _need(val, torch.float64, "val", 1)
    if C is None:
        C = torch.empty((M, Ncols), dtype=torch.float64, device=dev)
    ctx = N.context(dev.index)
    N.check(N.load().as_spmm_csr_f64(ctx.handle, M, K, Ncols, nnz, _ptr(rowptr), _ptr(colind),
                                     _ptr(val), _ptr(B), B.stride(0) if K > 1 else Ncols,
                                     _ptr(C), C.stride(0) if M > 1 else Ncols, float(beta),
                                     _stream(dev)), "as_spmm_csr_f64")
    return C


def spgemm_dense(a_rowptr, a_colind, a_val, b_rowptr, b_colind, b_val, n_cols: int, C=None,
                 beta: float = 0.0):
    """C = A*B + beta*C with A and B in CSR (fp32 values) and C a dense fp32 (M, n_cols)
    matrix: the reference's sparse_matrix_mul3 (SpMM.cpp:309-327), bit for bit."""
    dev = _dev(a_rowptr, a_colind, a_val, b_rowptr, b_colind, b_val, C)
    M, nnz_a = _csr(a_rowptr, a_colind)
    K, nnz_b = _csr(b_rowptr, b_colind)
    _need(a_val, torch.float32, "a_val", 1)
    _need(b_val, torch.float32, "b_val", 1)
    if a_val.numel() != nnz_a or b_val.numel() != nnz_b:
        raise ValueError("value and column-index lengths differ")
    if C is None:
        if beta != 0.0:
            raise ValueError("beta != 0 needs C")
        C = torch.empty((M, n_cols), dtype=torch.float32, device=dev)
    elif C.dtype != torch.float32 or C.shape != (M, n_cols) or C.stride(1) != 1:
        raise ValueError("C must be float32 (M, n_cols) row-major")
    ctx = N.context(dev.index)
    N.check(N.load().as_spgemm_csr_dense_f32(ctx.handle, M, K, n_cols, nnz_a, _ptr(a_rowptr),
                                             _ptr(a_colind), _ptr(a_val), nnz_b, _ptr(b_rowptr),
                                             _ptr(b_colind), _ptr(b_val), _ptr(C),
                                             C.stride(0) if M > 1 else n_cols, float(beta),
                                             _stream(dev)), "as_spgemm_csr_dense_f32")
    return C


def spmm_reduce(rowptr, colind, B, val=None, op: str = "sum", C=None):
    """C[i,:] = reduce over row i of w_e * B[col(e),:], reduce in {"sum", "max"}, w_e = val or 1
    (the unweighted copy-sum / copy-max aggregations); rows without entries give 0."""
    dev = _dev(rowptr, colind, val, B, C)
    M, nnz = _csr(rowptr, colind)
    if B.dtype != torch.float32 or B.dim() != 2 or B.stride(1) != 1:
        raise ValueError("B must be float32, 2-D, row-major")
    if val is not None:
        _need(val, torch.float32, "val", 1)
    K, Ncols = B.shape
    if C is None:
        C = torch.empty((M, Ncols), dtype=torch.float32, device=dev)
    ctx = N.context(dev.index)
    N.check(N.load().as_spmm_csr_reduce_f32(ctx.handle, M, K, Ncols, nnz, _ptr(rowptr),
                                            _ptr(colind), _ptr(val), _ptr(B),
                                            B.stride(0) if K > 1 else Ncols, _ptr(C),
                                            C.stride(0) if M > 1 else Ncols,
                                            {"sum": 0, "max": 1, "max_dgl": 2}[op], _stream(dev)),
            "as_spmm_csr_reduce_f32")
    return C


def spmm_variants(dtype: torch.dtype = torch.float32) -> list[str]:
    d = 0 if dtype == torch.float32 else 1
    L = N.load()
    return [L.as_spmm_variant_name(d, i).decode() for i in range(1, L.as_spmm_variant_count(d) + 1)]


def spmm_variant_supported(variant: int, width: int, dtype=torch.float32, ldb: int | None = None,
                           ldc: int | None = None, B_ptr: int = 256, C_ptr: int = 256) -> bool:
    """Whether a variant can run dense width `width` (contiguous, 256-byte aligned operands
    unless given otherwise)."""
    d = 0 if dtype == torch.float32 else 1
    return bool(N.load().as_spmm_variant_supported(d, int(variant), int(width), ldb or width,
                                                   ldc or width, B_ptr, C_ptr))


def spmm_default_variant(B: torch.Tensor, C: torch.Tensor | None, M: int, nnz: int) -> int:
    d = 0 if B.dtype == torch.float32 else 1
    K, Ncols = B.shape
    ldb = B.stride(0)
    ldc = C.stride(0) if C is not None else Ncols
    return int(N.load().as_spmm_default_variant(d, M, K, Ncols, nnz, ldb, ldc, _ptr(B),
                                                _ptr(C) if C is not None else 256))


def spmv(rowptr, colind, val, x, y=None, beta: float = 0.0):
    """y = A*x + beta*y, plain CSR, fp32."""
    dev = _dev(rowptr, colind, val, x, y)
    M, nnz = _csr(rowptr, colind)
    _need(val, torch.float32, "val", 1)
    _need(x, torch.float32, "x", 1)
    if y is None:
        if beta != 0.0:
            raise ValueError("beta != 0 needs y")
        y = torch.empty(M, dtype=torch.float32, device=dev)
    _need(y, torch.float32, "y", 1)
    ctx = N.context(dev.index)
    N.check(N.load().as_spmv_csr_f32(ctx.handle, M, x.numel(), nnz, _ptr(rowptr), _ptr(colind),
                                     _ptr(val), _ptr(x), _ptr(y), float(beta), _stream(dev)),
            "as_spmv_csr_f32")
    return y


def spmv_vcsr4(vrowptr, vcolind, vval, x, y=None, beta: float = 0.0):
    """y = A*x + beta*y over the reference's 1x4-blocked layout (SpMV.cpp:15-38)."""
    dev = _dev(vrowptr, vcolind, vval, x, y)
    M, nslots = _csr(vrowptr, vcolind)
    _need(vval, torch.float32, "val", 1)
    _need(x, torch.float32, "x", 1)
    if y is None:
        if beta != 0.0:
            raise ValueError("beta != 0 needs y")
        y = torch.empty(M, dtype=torch.float32, device=dev)
    _need(y, torch.float32, "y", 1)
    ctx = N.context(dev.index)
    N.check(N.load().as_spmv_vcsr4_f32(ctx.handle, M, x.numel(), nslots, _ptr(vrowptr),
                                       _ptr(vcolind), _ptr(vval), _ptr(x), _ptr(y), float(beta),
                                       _stream(dev)), "as_spmv_vcsr4_f32")
    return y


_SDDMM_SELECTOR = []


def sddmm_path(rowptr, colind, n_cols: int, K: int) -> str:
    """The learned choice of SDDMM path for this pattern and K ("simt" or "tc<variant>", see
    tuner.sddmm_paths), from armsparse_gb300/sddmm_selector_model.json; "simt" when no model
    file is present. Computes the pattern's features on the device (one pass over it): cache
    the answer when the same pattern is used again."""
    if not _SDDMM_SELECTOR:
        from . import selector
        try:
            _SDDMM_SELECTOR.append(selector.SddmmSelector.load())
        except (OSError, ValueError):
            _SDDMM_SELECTOR.append(None)
    sel = _SDDMM_SELECTOR[0]
    return "simt" if sel is None else sel.choose(rowptr, colind, n_cols, K)


def sddmm(rowptr, colind, X, Y, aval=None, out=None, tensor_cores=False, variant: int = 0):
    """out[e] = aval[e] * <X[row(e)], Y[col(e)]> (aval None -> unscaled, the reference's
    sddmm_cuda_csr). X: M x K, Y: N x K, fp32 -- or both bf16 (fp32 products and sums, fp32
    out). tensor_cores=True selects the tcgen05 split-bf16 path (fp32 inputs; ``variant`` its
    kernel; columns must ascend within each row), False the CUDA-core FP32 path, "auto" the
    learned choice between them (``sddmm_path``) for fp32 inputs -- which may be the
    tensor-core path, so it too needs ascending columns."""
    if tensor_cores == "auto":
        if X.dtype == torch.float32 and Y.dtype == torch.float32:
            path = sddmm_path(rowptr, colind, Y.shape[0], X.shape[1])
            tensor_cores = path != "simt"
            variant = int(path[2:]) if tensor_cores else 0
        else:
            tensor_cores = False
    dev = _dev(rowptr, colind, X, Y, aval, out)
    M, nnz = _csr(rowptr, colind)
    if X.dtype == torch.float64:
        return _sddmm_f64(rowptr, colind, X, Y, aval, out)
    bf16 = X.dtype == torch.bfloat16 and Y.dtype == torch.bfloat16 and not tensor_cores
    for t, n in ((X, "X"), (Y, "Y")):
        if (t.dtype != torch.float32 and not bf16) or t.dim() != 2 or t.stride(1) != 1:
            raise ValueError(f"{n} must be float32 (or both X and Y bfloat16), 2-D, row-major")
    if X.shape[0] != M:
        raise ValueError("X must have one row per pattern row")
    if X.shape[1] != Y.shape[1]:
        raise ValueError("X and Y need the same K")
    if aval is not None:
        _need(aval, torch.float32, "aval", 1)
    if out is None:
        out = torch.empty(nnz, dtype=torch.float32, device=dev)
    _need(out, torch.float32, "out", 1)
    K = X.shape[1]
    ldx = X.stride(0) if M > 1 else K
    ldy = Y.stride(0) if Y.shape[0] > 1 else K
    ctx = N.context(dev.index)
    if bf16:
        N.check(N.load().as_sddmm_csr_bf16(ctx.handle, M, Y.shape[0], K, nnz, _ptr(rowptr),
                                           _ptr(colind), _ptr(aval), _ptr(X), ldx, _ptr(Y), ldy,
                                           _ptr(out), _stream(dev)), "as_sddmm_csr_bf16")
    elif tensor_cores:
        N.check(N.load().as_sddmm_csr_bf16x3_v(ctx.handle, M, Y.shape[0], K, nnz, _ptr(rowptr),
                                               _ptr(colind), _ptr(aval), _ptr(X), ldx, _ptr(Y),
                                               ldy, _ptr(out), int(variant), _stream(dev)),
                "as_sddmm_csr_bf16x3_v")
    else:
        N.check(N.load().as_sddmm_csr_f32(ctx.handle, M, Y.shape[0], K, nnz, _ptr(rowptr),
                                          _ptr(colind), _ptr(aval), _ptr(X), ldx, _ptr(Y), ldy,
                                          _ptr(out), _stream(dev)), "as_sddmm_csr_f32")
    return out


def _sddmm_f64(rowptr, colind, X, Y, aval, out):
    """float64 SDDMM (gradient checks only)."""
    dev = X.device
    M, nnz = _csr(rowptr, colind)
    for t, n in ((X, "X"), (Y, "Y")):
        if t.dtype != torch.float64 or t.dim() != 2 or not t.is_contiguous():
            raise ValueError(f"{n} must be float64, 2-D, contiguous")
    if aval is not None:
        _need(aval, torch.float64, "aval", 1)
    if out is None:
        out = torch.empty(nnz, dtype=torch.float64, device=dev)
    K = X.shape[1]
    ctx = N.context(dev.index)
    N.check(N.load().as_sddmm_csr_f64(ctx.handle, M, Y.shape[0], K, nnz, _ptr(rowptr),
                                      _ptr(colind), _ptr(aval), _ptr(X), K, _ptr(Y), K, _ptr(out),
                                      _stream(dev)), "as_sddmm_csr_f64")
    return out


def sddmm_coo(rowind, colind, X, Y, aval=None, out=None):
    """out[e] = aval[e] * <X[rowind[e]], Y[colind[e]]>, entries in any order (FP32)."""
    dev = _dev(rowind, colind, X, Y, aval, out)
    _need(rowind, torch.int32, "rowind", 1)
    _need(colind, torch.int32, "colind", 1)
    nnz = colind.numel()
    if rowind.numel() != nnz:
        raise ValueError("rowind and colind lengths differ")
    for t, n in ((X, "X"), (Y, "Y")):
        if t.dtype != torch.float32 or t.dim() != 2 or t.stride(1) != 1:
            raise ValueError(f"{n} must be float32, 2-D, row-major")
    if X.shape[1] != Y.shape[1]:
        raise ValueError("X and Y need the same K")
    if aval is not None:
        _need(aval, torch.float32, "aval", 1)
    if out is None:
        out = torch.empty(nnz, dtype=torch.float32, device=dev)
    K = X.shape[1]
    ldx = X.stride(0) if X.shape[0] > 1 else K
    ldy = Y.stride(0) if Y.shape[0] > 1 else K
    ctx = N.context(dev.index)
    N.check(N.load().as_sddmm_coo_f32(ctx.handle, X.shape[0], Y.shape[0], K, nnz, _ptr(rowind),
                                      _ptr(colind), _ptr(aval), _ptr(X), ldx, _ptr(Y), ldy,
                                      _ptr(out), _stream(dev)), "as_sddmm_coo_f32")
    return out


def csr2csc(rowptr, colind, val, n_cols: int):
    """(colptr, rowind, cscval): rows ascending within each column (bit-exact, deterministic).
    val may be None for a pattern-only transpose (cscval is then None)."""
    dev = _dev(rowptr, colind, val)
    M, nnz = _csr(rowptr, colind)
    if val is not None:
        _need(val, torch.float32, "val", 1)
    colptr = torch.empty(n_cols + 1, dtype=torch.int32, device=dev)
    rowind = torch.empty(nnz, dtype=torch.int32, device=dev)
    cscval = torch.empty(nnz, dtype=torch.float32, device=dev) if val is not None else None
    ctx = N.context(dev.index)
    N.check(N.load().as_csr2csc(ctx.handle, M, n_cols, nnz, _ptr(rowptr), _ptr(colind), _ptr(val),
                                _ptr(colptr), _ptr(rowind), _ptr(cscval), _stream(dev)),
            "as_csr2csc")
    return colptr, rowind, cscval


def csr2csc_perm(rowptr, colind, n_cols: int):
    """(colptr, rowind, perm): the transpose's pattern and, for each CSC entry j, its CSR
    position perm[j] (so values in CSC order are ``val[perm]`` for any values)."""
    dev = _dev(rowptr, colind)
    M, nnz = _csr(rowptr, colind)
    colptr = torch.empty(n_cols + 1, dtype=torch.int32, device=dev)
    rowind = torch.empty(nnz, dtype=torch.int32, device=dev)
    perm = torch.empty(nnz, dtype=torch.int32, device=dev)
    ctx = N.context(dev.index)
    N.check(N.load().as_csr2csc_perm(ctx.handle, M, n_cols, nnz, _ptr(rowptr), _ptr(colind),
                                     _ptr(colptr), _ptr(rowind), _ptr(perm), _stream(dev)),
            "as_csr2csc_perm")
    return colptr, rowind, perm


def gather(src, idx, out=None):
    """out[i] = src[idx[i]] (fp32 values, int32 indices) with this library's kernel."""
    dev = _dev(src, idx, out)
    _need(src, torch.float32, "src", 1)
    _need(idx, torch.int32, "idx", 1)
    if out is None:
        out = torch.empty(idx.numel(), dtype=torch.float32, device=dev)
    else:
        _need(out, torch.float32, "out", 1)
        if out.numel() != idx.numel():
            raise ValueError("out and idx lengths differ")
    ctx = N.context(dev.index)
    N.check(N.load().as_gather_f32(ctx.handle, idx.numel(), src.numel(), _ptr(src), _ptr(idx),
                                   _ptr(out), _stream(dev)), "as_gather_f32")
    return out


def spmm_sddmm(rowptr, colind, val, B, F, perm=None, C=None, beta: float = 0.0,
               variant: int = 0, dA=None, out_dtype: torch.dtype = torch.float32):
    """(C, dA): C = A*B + beta*C as ``spmm`` and, in the same pass over A, the SDDMM
    dA[perm[e]] = <B[col(e), :], F[row(e), :]> (dA[e] when perm is None) in fp32. With A the
    CSC of a forward matrix, B = dOut, F = the forward's input and perm from
    ``csr2csc_perm``, this is the backward of out = A_fwd * F with trainable values.
    variant: 0 = library choice, else an nnz-split variant whose column tile covers N.
    out_dtype=torch.bfloat16 (bf16 inputs, beta 0): C in bf16, as ``spmm``."""
    dev = _dev(rowptr, colind, val, B, F, perm, C, dA)
    M, nnz = _csr(rowptr, colind)
    if B.dim() != 2 or F.dim() != 2 or B.stride(1) != 1 or F.stride(1) != 1:
        raise ValueError("B and F must be 2-D row-major with unit column stride")
    K, Ncols = B.shape
    if F.shape != (M, Ncols):
        raise ValueError("F must be (M, N)")
    if val.dtype == torch.float32 and B.dtype == torch.float32 and F.dtype == torch.float32:
        fn, dname = N.load().as_spmm_sddmm_csr_f32, "as_spmm_sddmm_csr_f32"
    elif val.dtype == torch.bfloat16 and B.dtype == torch.bfloat16 and F.dtype == torch.bfloat16:
        fn, dname = N.load().as_spmm_sddmm_csr_bf16, "as_spmm_sddmm_csr_bf16"
    else:
        raise TypeError("val, B and F must all be float32 or all bfloat16")
    _need(val, val.dtype, "val", 1)
    if val.numel() != nnz:
        raise ValueError("val and colind lengths differ")
    if perm is not None:
        _need(perm, torch.int32, "perm", 1)
        if perm.numel() != nnz:
            raise ValueError("perm and colind lengths differ")
    c16 = out_dtype == torch.bfloat16
    if c16 and (val.dtype != torch.bfloat16 or beta != 0.0):
        raise ValueError("a bf16 output needs bf16 inputs and beta = 0")
    cdt = torch.bfloat16 if c16 else torch.float32
    if C is None:
        if beta != 0.0:
            raise ValueError("beta != 0 needs C")
        C = torch.empty((M, Ncols), dtype=cdt, device=dev)
    elif C.dtype != cdt or C.dim() != 2 or C.shape != (M, Ncols) or C.stride(1) != 1:
        raise ValueError(f"C must be {cdt} (M, N) row-major")
    if dA is None:
        dA = torch.empty(nnz, dtype=torch.float32, device=dev)
    else:
        _need(dA, torch.float32, "dA", 1)
        if dA.numel() != nnz:
            raise ValueError("dA and colind lengths differ")
    ldb = B.stride(0) if K > 1 else Ncols
    ldc = C.stride(0) if M > 1 else Ncols
    ldf = F.stride(0) if M > 1 else Ncols
    ctx = N.context(dev.index)
    if c16:
        N.check(N.load().as_spmm_sddmm_csr_bf16_out16(
            ctx.handle, M, K, Ncols, nnz, _ptr(rowptr), _ptr(colind), _ptr(val), _ptr(B), ldb,
            _ptr(C), ldc, _ptr(F), ldf, _ptr(perm), _ptr(dA), int(variant), _stream(dev)),
            "as_spmm_sddmm_csr_bf16_out16")
        return C, dA
    N.check(fn(ctx.handle, M, K, Ncols, nnz, _ptr(rowptr), _ptr(colind), _ptr(val), _ptr(B), ldb,
               _ptr(C), ldc, float(beta), _ptr(F), ldf, _ptr(perm), _ptr(dA), int(variant),
               _stream(dev)), dname)
    return C, dA


def softmax_xent(scores, labels, n_classes: int):
    """(loss, lse): the mean softmax cross-entropy of bf16 class scores (the first n_classes
    columns of each row; further columns are padding) against int64 labels --
    F.nll_loss(F.log_softmax(x), y) in one pass, summed in a fixed order -- as a 0-dim fp32
    tensor, and each row's logsumexp (fp32, for ``softmax_xent_grad``)."""
    dev = _dev(scores, labels)
    if scores.dtype != torch.bfloat16 or scores.dim() != 2 or scores.stride(1) != 1:
        raise ValueError("scores must be bfloat16 (n, width) row-major")
    _need(labels, torch.int64, "labels", 1)
    n = scores.shape[0]
    if labels.numel() != n or not 1 <= n_classes <= scores.shape[1]:
        raise ValueError("labels must have one entry per row; 1 <= n_classes <= width")
    loss = torch.empty((), dtype=torch.float32, device=dev)
    lse = torch.empty(n, dtype=torch.float32, device=dev)
    ctx = N.context(dev.index)
    N.check(N.load().as_softmax_xent_bf16(ctx.handle, n, n_classes, _ptr(scores),
                                          scores.stride(0) if n > 1 else scores.shape[1],
                                          _ptr(labels), _ptr(lse), _ptr(loss), _stream(dev)),
            "as_softmax_xent_bf16")
    return loss, lse


def softmax_xent_grad(scores, labels, n_classes: int, lse, gscale):
    """d(softmax_xent)/d(scores) times the device scalar gscale, bf16, zero in the padding
    columns; lse from ``softmax_xent``."""
    dev = _dev(scores, labels, lse, gscale)
    n, width = scores.shape
    _need(lse, torch.float32, "lse", 1)
    _need(gscale, torch.float32, "gscale")
    G = torch.empty((n, width), dtype=torch.bfloat16, device=dev)
    ctx = N.context(dev.index)
    N.check(N.load().as_softmax_xent_bwd_bf16(ctx.handle, n, n_classes, _ptr(scores),
                                              scores.stride(0) if n > 1 else width,
                                              _ptr(labels), _ptr(lse), _ptr(gscale), _ptr(G),
                                              width, width, _stream(dev)),
            "as_softmax_xent_bwd_bf16")
    return G


def to_bf16(x: torch.Tensor) -> torch.Tensor:
    """fp32 -> bf16 (round to nearest even) with this library's kernel."""
    dev = _dev(x)
    _need(x, torch.float32, "x")
    out = torch.empty(x.shape, dtype=torch.bfloat16, device=dev)
    ctx = N.context(dev.index)
    N.check(N.load().as_f32_to_bf16(ctx.handle, x.numel(), _ptr(x), _ptr(out), _stream(dev)),
            "as_f32_to_bf16")
    return out


def dense_to_csr(D: torch.Tensor):
    """(rowptr, colind, val) of a dense fp32 matrix: entries != 0, row-major order (the
    reference's toCSR). Synchronises once to size the outputs."""
    dev = _dev(D)
    if D.dtype != torch.float32 or D.dim() != 2 or D.stride(1) != 1:
        raise ValueError("D must be float32, 2-D, row-major")
    M, K = D.shape
    ld = D.stride(0) if M > 1 else K
    rowptr = torch.empty(M + 1, dtype=torch.int32, device=dev)
    ctx = N.context(dev.index)
    N.check(N.load().as_dense_to_csr_count(ctx.handle, M, K, _ptr(D), ld, _ptr(rowptr),
                                           _stream(dev)), "as_dense_to_csr_count")
    nnz = int(rowptr[M])
    colind = torch.empty(nnz, dtype=torch.int32, device=dev)
    val = torch.empty(nnz, dtype=torch.float32, device=dev)
    N.check(N.load().as_dense_to_csr_fill(ctx.handle, M, K, _ptr(D), ld, _ptr(rowptr),
                                          _ptr(colind), _ptr(val), _stream(dev)),
            "as_dense_to_csr_fill")
    return rowptr, colind, val


def csr_to_vcsr4(rowptr, colind, val):
    """The reference's 1x4-blocked layout (toVectorAwareCSR) from CSR with ascending columns.
    Synchronises once to size the outputs."""
    dev = _dev(rowptr, colind, val)
    M, nnz = _csr(rowptr, colind)
    _need(val, torch.float32, "val", 1)
    vrowptr = torch.empty(M + 1, dtype=torch.int32, device=dev)
    ctx = N.context(dev.index)
    N.check(N.load().as_csr_to_vcsr4_count(ctx.handle, M, nnz, _ptr(rowptr), _ptr(colind),
                                           _ptr(vrowptr), _stream(dev)), "as_csr_to_vcsr4_count")
    ns = int(vrowptr[M])
    vcolind = torch.empty(ns, dtype=torch.int32, device=dev)
    vval = torch.empty(ns, dtype=torch.float32, device=dev)
    N.check(N.load().as_csr_to_vcsr4_fill(ctx.handle, M, nnz, _ptr(rowptr), _ptr(colind),
                                          _ptr(val), _ptr(vrowptr), _ptr(vcolind), _ptr(vval),
                                          _stream(dev)), "as_csr_to_vcsr4_fill")
    return vrowptr, vcolind, vval


def csr_to_rowpair(rowptr, colind, val):
    """The reference's row-pair reuse layout (toDataReuseFormat, suitesparse_sdmm.cpp:150-179)
    from CSR with ascending columns: (rowptr2, colind2, val2, flag2 as uint8). The entry count
    is unchanged, so nothing synchronises."""
    dev = _dev(rowptr, colind, val)
    M, nnz = _csr(rowptr, colind)
    _need(val, torch.float32, "val", 1)
    rowptr2 = torch.empty(M + 1, dtype=torch.int32, device=dev)
    colind2 = torch.empty(nnz, dtype=torch.int32, device=dev)
    val2 = torch.empty(nnz, dtype=torch.float32, device=dev)
    flag2 = torch.empty(nnz, dtype=torch.uint8, device=dev)
    ctx = N.context(dev.index)
    N.check(N.load().as_csr_to_rowpair_count(ctx.handle, M, nnz, _ptr(rowptr), _ptr(colind),
                                             _ptr(rowptr2), _stream(dev)),
            "as_csr_to_rowpair_count")
    N.check(N.load().as_csr_to_rowpair_fill(ctx.handle, M, nnz, _ptr(rowptr), _ptr(colind),
                                            _ptr(val), _ptr(rowptr2), _ptr(colind2), _ptr(val2),
                                            _ptr(flag2), _stream(dev)), "as_csr_to_rowpair_fill")
    return rowptr2, colind2, val2, flag2


def spmm_rowpair(rowptr2, colind2, val2, flag2, B, C=None, beta: float = 0.0):
    """C = A*B + beta*C over the row-pair layout, bit for bit the reference's DataReuseSpmm
    (suitesparse_sdmm.cpp:25-44): even rows are their CSR chains, odd rows chain over the
    columns they share with the row above first."""
    dev = _dev(rowptr2, colind2, val2, flag2, B, C)
    M, nnz = _csr(rowptr2, colind2)
    _need(val2, torch.float32, "val2", 1)
    if flag2.dtype != torch.uint8 or flag2.numel() != nnz:
        raise ValueError("flag2 must be uint8 with one byte per entry")
    if B.dtype != torch.float32 or B.dim() != 2 or B.stride(1) != 1:
        raise ValueError("B must be float32, 2-D, row-major")
    K, Ncols = B.shape
    if C is None:
        C = torch.empty((M, Ncols), dtype=torch.float32, device=dev)
    ctx = N.context(dev.index)
    N.check(N.load().as_spmm_rowpair_f32(ctx.handle, M, K, Ncols, nnz, _ptr(rowptr2),
                                         _ptr(colind2), _ptr(val2), _ptr(flag2), _ptr(B),
                                         B.stride(0) if K > 1 else Ncols, _ptr(C),
                                         C.stride(0) if M > 1 else Ncols, float(beta),
                                         _stream(dev)), "as_spmm_rowpair_f32")
    return C


def spmm_vcsr4(vrowptr, vcolind, vval, B, C=None, beta: float = 0.0):
    """C = A*B + beta*C with A in the reference's 1x4-blocked layout (``csr_to_vcsr4``); slots
    holding 0 are skipped, so the result is the CSR SpMM's, bit for bit."""
    dev = _dev(vrowptr, vcolind, vval, B, C)
    M, ns = _csr(vrowptr, vcolind)
    _need(vval, torch.float32, "vval", 1)
    if B.dtype != torch.float32 or B.dim() != 2 or B.stride(1) != 1:
        raise ValueError("B must be float32, 2-D, row-major")
    K, Ncols = B.shape
    if C is None:
        C = torch.empty((M, Ncols), dtype=torch.float32, device=dev)
    ctx = N.context(dev.index)
    N.check(N.load().as_spmm_vcsr4_f32(ctx.handle, M, K, Ncols, ns, _ptr(vrowptr), _ptr(vcolind),
                                       _ptr(vval), _ptr(B), B.stride(0) if K > 1 else Ncols,
                                       _ptr(C), C.stride(0) if M > 1 else Ncols, float(beta),
                                       _stream(dev)), "as_spmm_vcsr4_f32")
    return C
