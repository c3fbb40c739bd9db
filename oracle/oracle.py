"""CPU oracle for the sparse hot path (TEST INFRASTRUCTURE).

Only ``tests/``, ``__graft_entry__.smoke()`` and ``bench.py``'s CPU-baseline leg / reference
arm may import this module, and only as the checker or as the timed CPU baseline; the
product package ``armsparse_gb300`` never imports it.

It wraps two shared libraries:

* ``oracle/_build/liboracle.so`` -- ``oracle.c``, a plain-C restatement of the reference's
  kernels (each function there cites the reference file:line it follows);
* ``oracle/_ref/libref_*.so`` -- the reference's own kernels compiled from its sources by
  ``oracle/Makefile`` (only where the reference sources exist, i.e. not on a GPU host).

Pinning: ``tests/test_oracle_pins.py`` checks the restatement against the compiled reference
and against ``tests/golden/*.npz`` (made from the compiled reference by
``tests/golden/make_golden.py``).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import threading

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LOCK = threading.Lock()
_LIB = None
_REF = {}

_i32p = np.ctypeslib.ndpointer(dtype=np.int32, flags="C_CONTIGUOUS")
_f32p = np.ctypeslib.ndpointer(dtype=np.float32, flags="C_CONTIGUOUS")
_f64p = np.ctypeslib.ndpointer(dtype=np.float64, flags="C_CONTIGUOUS")
_c_int, _c_long = ctypes.c_int, ctypes.c_long


def build(quiet: bool = True) -> str:
    """Compile ``liboracle.so`` (fast; a single C file)."""
    out = subprocess.run(["make", "-C", _HERE, "oracle"], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    return os.path.join(_HERE, "_build", "liboracle.so")


def build_ref(ref_dir: str | None = None, gcn: bool = False, cuda: bool = False) -> bool:
    """Compile the reference's own kernels into ``oracle/_ref`` when its sources exist (with
    ``cuda``, also its CUDA kernels as sm_103a cubins for oracle/ref_gpu.py)."""
    args = ["make", "-C", _HERE, "ref"] + (["ref-gcn"] if gcn else []) + (["ref-cuda"] if cuda else [])
    if ref_dir:
        args.append(f"REF={ref_dir}")
    out = subprocess.run(args, capture_output=True, text=True)
    return out.returncode == 0


def lib():
    global _LIB
    with _LOCK:
        if _LIB is None:
            path = os.path.join(_HERE, "_build", "liboracle.so")
            if not os.path.exists(path):
                build()
            L = ctypes.CDLL(path)
            L.or_spmm_fma_chain_f32.argtypes = [_c_int, _c_int, _i32p, _i32p, _f32p, _f32p,
                                                _c_long, _f32p, _c_long, _c_int, _c_int]
            L.or_spmm_nnz_order_f32.argtypes = [_c_int, _c_int, _i32p, _i32p, _f32p, _f32p,
                                                _c_long, _f32p, _c_long, ctypes.c_float,
                                                _c_int, _c_int, _c_int]
            L.or_spmm_f64.argtypes = [_c_int, _c_int, _i32p, _i32p, _f64p, _f64p, _c_long,
                                      _f64p, _f64p, _c_int]
            L.or_spmv_vcsr4_f32.argtypes = [_c_int, _i32p, _i32p, _f32p, _f32p, _f32p, _c_int,
                                            _c_int]
            L.or_csr_to_vcsr4.argtypes = [_c_int, _i32p, _i32p, _f32p, ctypes.c_void_p,
                                          ctypes.c_void_p, ctypes.c_void_p]
            L.or_csr_to_vcsr4.restype = _c_long
            L.or_spmv_f64.argtypes = [_c_int, _i32p, _i32p, _f64p, _f64p, _f64p, _f64p]
            L.or_sddmm_csr_f64.argtypes = [_c_int, _c_int, _i32p, _i32p, ctypes.c_void_p, _f64p,
                                           _c_long, _f64p, _c_long, _f64p, _f64p, _c_int]
            L.or_sddmm_csr_f32_group.argtypes = [_c_int, _c_int, _i32p, _i32p, ctypes.c_void_p,
                                                 _f32p, _c_long, _f32p, _c_long, _f32p, _c_int]
            L.or_sddmm_csr_f32_lanes.argtypes = [_c_int, _c_int, _i32p, _i32p, ctypes.c_void_p,
                                                 _f32p, _c_long, _f32p, _c_long, _f32p, _c_int]
            L.or_sddmm_csr_f32_slices.argtypes = [_c_int, _c_int, _i32p, _i32p, _f32p, _c_long,
                                                  _f32p, _c_long, ctypes.c_void_p, _c_int,
                                                  _c_int, _c_int, _f32p, _c_int]
            L.or_csr2csc.argtypes = [_c_int, _c_int, _i32p, _i32p, _f32p, _i32p, _i32p, _f32p]
            L.or_max_threads.restype = _c_int
            L.or_spgemm_dense_f32.argtypes = [_c_int, _c_int, _i32p, _i32p, _f32p, _i32p, _i32p,
                                              _f32p, _f32p, _c_long, _c_int]
            L.or_spmm_reduce_f32.argtypes = [_c_int, _c_int, _i32p, _i32p, ctypes.c_void_p, _f32p,
                                             _c_long, _f32p, _c_int]
            L.or_csr_to_rowpair.argtypes = [_c_int, _i32p, _i32p, _f32p, _i32p, _i32p, _f32p,
                                            np.ctypeslib.ndpointer(dtype=np.uint8,
                                                                   flags="C_CONTIGUOUS")]
            L.or_spmm_rowpair_f32.argtypes = [_c_int, _c_int, _i32p, _i32p, _f32p,
                                              np.ctypeslib.ndpointer(dtype=np.uint8,
                                                                     flags="C_CONTIGUOUS"),
                                              _f32p, _c_long, _f32p, _c_long, _c_int]
            _LIB = L
    return _LIB


def ref_lib(name: str):
    """Load ``oracle/_ref/libref_<name>.so`` (the reference's own compiled code) or None."""
    with _LOCK:
        if name not in _REF:
            path = os.path.join(_HERE, "_ref", f"libref_{name}.so")
            _REF[name] = ctypes.CDLL(path) if os.path.exists(path) else None
    return _REF[name]


def max_threads() -> int:
    return int(lib().or_max_threads())


# ------------------------------------------------------------------------------------------
# Restatement wrappers
# ------------------------------------------------------------------------------------------
def _csr(rowptr, colind):
    return (np.ascontiguousarray(rowptr, dtype=np.int32),
            np.ascontiguousarray(colind, dtype=np.int32))


def spmm_fma_chain_f32(rowptr, colind, val, B, C=None, threads=None):
    """C (+)= A*B as the reference's rowBaseSpmm3 computes it (per-output fused-FMA chain in
    CSR order, SDMM.cpp:90-114). ``C`` None means a zero-initialised output."""
    rowptr, colind = _csr(rowptr, colind)
    M = rowptr.size - 1
    B = np.ascontiguousarray(B, dtype=np.float32)
    N = B.shape[1]
    acc = C is not None
    out = np.ascontiguousarray(C, dtype=np.float32).copy() if acc else np.empty((M, N), np.float32)
    lib().or_spmm_fma_chain_f32(M, N, rowptr, colind, np.ascontiguousarray(val, np.float32), B,
                                N, out, N, int(acc), threads or max_threads())
    return out


def spmm_nnz_order_f32(rowptr, colind, val, B, chunk, subchains=1, C=None, beta=0.0,
                       threads=None):
    """C = A*B + beta*C in the summation order of the GPU's entry-balanced SpMM kernels:
    chunks of `chunk` entries, `subchains` interleaved chains per chunk segment (1 for the
    one-entry-per-step kernels, 32 / group for the multi-entry ones) and the fix-up's order
    for rows over several chunks. Test infrastructure for bit-exact checks of those kernels."""
    rowptr, colind = _csr(rowptr, colind)
    M = rowptr.size - 1
    B = np.ascontiguousarray(B, dtype=np.float32)
    N = B.shape[1]
    if subchains < 1 or subchains > 32 or subchains & (subchains - 1):
        raise ValueError("subchains must be a power of two <= 32")
    out = (np.ascontiguousarray(C, dtype=np.float32).copy() if C is not None
           else np.zeros((M, N), np.float32))
    lib().or_spmm_nnz_order_f32(M, N, rowptr, colind, np.ascontiguousarray(val, np.float32), B,
                                N, out, N, float(beta), int(chunk), int(subchains),
                                threads or max_threads())
    return out


def spgemm_dense_f32(a_rowptr, a_colind, a_val, b_rowptr, b_colind, b_val, n_cols, C=None,
                     threads=None):
    """C (+)= A*B with A and B in CSR, C dense, as the reference's sparse_matrix_mul3
    (SpMM.cpp:309-327) computes it. ``C`` None means a zero-initialised output."""
    rp1, ci1 = _csr(a_rowptr, a_colind)
    rp2, ci2 = _csr(b_rowptr, b_colind)
    M = rp1.size - 1
    out = (np.zeros((M, n_cols), np.float32) if C is None
           else np.ascontiguousarray(C, dtype=np.float32).copy())
    lib().or_spgemm_dense_f32(M, n_cols, rp1, ci1, np.ascontiguousarray(a_val, np.float32), rp2,
                              ci2, np.ascontiguousarray(b_val, np.float32), out, n_cols,
                              threads or max_threads())
    return out


def spgemm_dense_f64(a_rowptr, a_colind, a_val, b_rowptr, b_colind, b_val, n_cols):
    """(A*B, |A|*|B|) in double precision for the sparse x sparse product (small cases)."""
    import scipy.sparse as sp
    M = len(a_rowptr) - 1
    K = len(b_rowptr) - 1
    A = sp.csr_matrix((np.asarray(a_val, np.float64), a_colind, a_rowptr), shape=(M, K))
    B = sp.csr_matrix((np.asarray(b_val, np.float64), b_colind, b_rowptr), shape=(K, n_cols))
    return (A @ B).toarray(), (abs(A) @ abs(B)).toarray()


def spmm_reduce_f32(rowptr, colind, B, val=None, op="sum"):
    """Sum / max aggregation in CSR order (w_e = val or 1); empty rows give 0."""
    rowptr, colind = _csr(rowptr, colind)
    M = rowptr.size - 1
    B = np.ascontiguousarray(B, np.float32)
    out = np.empty((M, B.shape[1]), np.float32)
    v = None if val is None else np.ascontiguousarray(val, np.float32)
    lib().or_spmm_reduce_f32(M, B.shape[1], rowptr, colind, None if v is None else v.ctypes.data,
                             B, B.shape[1], out, {"sum": 0, "max": 1, "max_dgl": 2}[op])
    return out


def spmm_f64(rowptr, colind, val, B, threads=None):
    """(A*B, |A|*|B|) in double precision."""
    rowptr, colind = _csr(rowptr, colind)
    M = rowptr.size - 1
    B = np.ascontiguousarray(B, dtype=np.float64)
    N = B.shape[1]
    C = np.empty((M, N), np.float64)
    A = np.empty((M, N), np.float64)
    lib().or_spmm_f64(M, N, rowptr, colind, np.ascontiguousarray(val, np.float64), B, N, C, A,
                      threads or max_threads())
    return C, A


def csr_to_vcsr4(rowptr, colind, val):
    """CSR -> the reference's 1x4-blocked layout (SpMV.cpp:15-38 semantics; K % 4 == 0)."""
    rowptr, colind = _csr(rowptr, colind)
    val = np.ascontiguousarray(val, np.float32)
    M = rowptr.size - 1
    size = lib().or_csr_to_vcsr4(M, rowptr, colind, val, None, None, None)
    vr = np.empty(M + 1, np.int32)
    vc = np.empty(max(size, 1), np.int32)
    vv = np.empty(max(size, 1), np.float32)
    lib().or_csr_to_vcsr4(M, rowptr, colind, val, vr.ctypes.data, vc.ctypes.data, vv.ctypes.data)
    return vr, vc[:size], vv[:size]


def spmv_vcsr4_f32(vrowptr, vcolind, vval, x, y=None, fused=True, threads=None):
    """y (+)= A*x over the 1x4-blocked layout (SpMV.cpp:155-179)."""
    vrowptr, vcolind = _csr(vrowptr, vcolind)
    M = vrowptr.size - 1
    out = (np.zeros(M, np.float32) if y is None
           else np.ascontiguousarray(y, np.float32).copy())
    lib().or_spmv_vcsr4_f32(M, vrowptr, vcolind, np.ascontiguousarray(vval, np.float32),
                            np.ascontiguousarray(x, np.float32), out, int(fused),
                            threads or max_threads())
    return out


def spmv_f64(rowptr, colind, val, x):
    rowptr, colind = _csr(rowptr, colind)
    M = rowptr.size - 1
    y = np.empty(M, np.float64)
    a = np.empty(M, np.float64)
    lib().or_spmv_f64(M, rowptr, colind, np.ascontiguousarray(val, np.float64),
                      np.ascontiguousarray(x, np.float64), y, a)
    return y, a


def sddmm_f64(rowptr, colind, X, Y, aval=None, threads=None):
    """(out, |out| scale) for out[e] = aval[e] * <X[row(e)], Y[col(e)]> in double."""
    rowptr, colind = _csr(rowptr, colind)
    M = rowptr.size - 1
    X = np.ascontiguousarray(X, np.float64)
    Y = np.ascontiguousarray(Y, np.float64)
    nnz = int(rowptr[-1])
    out = np.empty(nnz, np.float64)
    ab = np.empty(nnz, np.float64)
    av = None if aval is None else np.ascontiguousarray(aval, np.float64)
    lib().or_sddmm_csr_f64(M, X.shape[1], rowptr, colind,
                           None if av is None else av.ctypes.data, X, X.shape[1], Y, Y.shape[1],
                           out, ab, threads or max_threads())
    return out, ab


def sddmm_f32_lanes(rowptr, colind, X, Y, aval=None, threads=None):
    """FP32 SDDMM with 8 interleaved partial sums (the CPU baseline)."""
    rowptr, colind = _csr(rowptr, colind)
    M = rowptr.size - 1
    X = np.ascontiguousarray(X, np.float32)
    Y = np.ascontiguousarray(Y, np.float32)
    out = np.empty(int(rowptr[-1]), np.float32)
    av = None if aval is None else np.ascontiguousarray(aval, np.float32)
    lib().or_sddmm_csr_f32_lanes(M, X.shape[1], rowptr, colind,
                                 None if av is None else av.ctypes.data, X, X.shape[1], Y,
                                 Y.shape[1], out, threads or max_threads())
    return out


def sddmm_f32_group(rowptr, colind, X, Y, aval=None, threads=None):
    """FP32 SDDMM in the GPU kernel's order: per edge, G lanes (a power of two, about one per
    16 elements of K, up to 32) each run one fused-FMA chain over their 4-element blocks
    (blocks l, l + G, ...), then a butterfly sum across the lanes. The parity oracle of the
    GPU SIMT SDDMM."""
    rowptr, colind = _csr(rowptr, colind)
    M = rowptr.size - 1
    X = np.ascontiguousarray(X, np.float32)
    Y = np.ascontiguousarray(Y, np.float32)
    out = np.empty(int(rowptr[-1]), np.float32)
    av = None if aval is None else np.ascontiguousarray(aval, np.float32)
    lib().or_sddmm_csr_f32_group(M, X.shape[1], rowptr, colind,
                                 None if av is None else av.ctypes.data, X, X.shape[1], Y,
                                 Y.shape[1], out, threads or max_threads())
    return out


def sddmm_f32_slices(rowptr, colind, X, Y, group, elems, cpl, perm=None, threads=None):
    """FP32 SDDMM in the order of the SpMM pass with the SDDMM fused in: per entry, `group`
    lanes each chain over their `elems`-element slices (lane l: slices (j*group + l)*elems,
    j < cpl), then a butterfly across the lanes; written at perm[e] (e when perm is None).
    The parity oracle of as_spmm_sddmm_csr_*'s dot products."""
    rowptr, colind = _csr(rowptr, colind)
    M = rowptr.size - 1
    X = np.ascontiguousarray(X, np.float32)
    Y = np.ascontiguousarray(Y, np.float32)
    if group > 32 or group & (group - 1):
        raise ValueError("group must be a power of two <= 32")
    out = np.zeros(int(rowptr[-1]), np.float32)
    pp = None if perm is None else np.ascontiguousarray(perm, np.int32)
    lib().or_sddmm_csr_f32_slices(M, X.shape[1], rowptr, colind, X, X.shape[1], Y, Y.shape[1],
                                  None if pp is None else pp.ctypes.data, group, elems, cpl, out,
                                  threads or max_threads())
    return out


def csr2csc(rowptr, colind, val, n_cols):
    """Stable CSR -> CSC (rows ascending within each column)."""
    rowptr, colind = _csr(rowptr, colind)
    M = rowptr.size - 1
    nnz = int(rowptr[-1])
    colptr = np.empty(n_cols + 1, np.int32)
    rowind = np.empty(max(nnz, 1), np.int32)
    cval = np.empty(max(nnz, 1), np.float32)
    lib().or_csr2csc(M, n_cols, rowptr, colind, np.ascontiguousarray(val, np.float32), colptr,
                     rowind, cval)
    return colptr, rowind[:nnz], cval[:nnz]


# ------------------------------------------------------------------------------------------
# Error metric
# ------------------------------------------------------------------------------------------
def rel_err(got, ref, absref):
    """Per-output relative error |got - ref| / max(|ref|, absref * 2**-20), where absref is
    the sum of |products| behind each output (the definition the measurement plan quotes;
    reported, not used as a pass/fail bar, because an FP32 sum that cancels toward zero is
    legitimately far from its own tiny value)."""
    got = np.asarray(got, np.float64)
    ref = np.asarray(ref, np.float64)
    den = np.maximum(np.abs(ref), np.asarray(absref, np.float64) * 2.0 ** -20)
    den = np.where(den == 0, 1.0, den)
    return np.abs(got - ref) / den


def scaled_err(got, ref, absref):
    """Per-output error relative to the output's magnitude scale:
    |got - ref| / max(|ref|, absref), absref = sum of |products| behind the output.
    For an FP32 sum of n terms in any order this stays near sqrt(n) * 2**-24; it is the
    metric the 1e-5 (FP32 paths) and 1e-2 (bf16 storage) tolerances of the tests apply to."""
    got = np.asarray(got, np.float64)
    ref = np.asarray(ref, np.float64)
    den = np.maximum(np.abs(ref), np.asarray(absref, np.float64))
    den = np.where(den == 0, 1.0, den)
    return np.abs(got - ref) / den


def bf16_round(a) -> np.ndarray:
    """Round float32 values to bfloat16 (nearest even), returned as float32."""
    a = np.ascontiguousarray(a, np.float32)
    u = a.view(np.uint32).astype(np.uint64)
    nan = (u & 0x7FFFFFFF) > 0x7F800000
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    r = np.where(nan, (u | 0x400000) & 0xFFFF0000, r).astype(np.uint32)
    return r.view(np.float32).reshape(a.shape)


# ------------------------------------------------------------------------------------------
# Dense-network reference for the selector's kernels (float64 numpy)
# ------------------------------------------------------------------------------------------
def mlp_linear_fwd(X, W, b=None, relu=False):
    Y = np.asarray(X, np.float64) @ np.asarray(W, np.float64).T
    if b is not None:
        Y = Y + np.asarray(b, np.float64)
    return np.maximum(Y, 0.0) if relu else Y


def mlp_linear_bwd(dY, X, W, relu_in=None):
    dY = np.asarray(dY, np.float64)
    dX = dY @ np.asarray(W, np.float64)
    if relu_in is not None:
        dX = np.where(np.asarray(relu_in) > 0, dX, 0.0)
    return dX, dY.T @ np.asarray(X, np.float64), dY.sum(axis=0)


def mlp_softmax_xent(Z, T, scale=1.0):
    Z = np.asarray(Z, np.float64)
    T = np.asarray(T, np.float64)
    m = Z.max(axis=1, keepdims=True)
    lse = m + np.log(np.exp(Z - m).sum(axis=1, keepdims=True))
    P = np.exp(Z - lse)
    return -(T * (Z - lse)).sum(axis=1), (P - T) * scale


def mlp_adam(p, g, m, v, lr, b1, b2, eps, wd, step):
    g = g + wd * p
    m = b1 * m + (1 - b1) * g
    v = b2 * v + (1 - b2) * g * g
    mh = m / (1 - b1 ** step)
    vh = v / (1 - b2 ** step)
    return p - lr * mh / (np.sqrt(vh) + eps), m, v


def ref_read_mtx(path: str):
    """The reference's own readMtx<float> (gcn/util/util.hpp:286-333) run on ``path`` through
    ``oracle/_ref/libref_mtx.so``: (nrows, ncols, rows, cols, vals) as it leaves its vectors,
    or None when the library was not built (no reference sources)."""
    L = ref_lib("mtx")
    if L is None:
        return None
    ip = ctypes.POINTER(ctypes.c_int)
    fp = ctypes.POINTER(ctypes.c_float)
    L.ref_read_mtx.argtypes = [ctypes.c_char_p, ip, ip, ip, ctypes.POINTER(ip),
                               ctypes.POINTER(ip), ctypes.POINTER(fp)]
    L.ref_read_mtx.restype = ctypes.c_int
    L.ref_mtx_free.argtypes = [ctypes.c_void_p]
    m, n, nv = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    r, c, v = ip(), ip(), fp()
    L.ref_read_mtx(path.encode(), ctypes.byref(m), ctypes.byref(n), ctypes.byref(nv),
                   ctypes.byref(r), ctypes.byref(c), ctypes.byref(v))
    k = nv.value
    out = (np.ctypeslib.as_array(r, (max(k, 1),))[:k].copy(),
           np.ctypeslib.as_array(c, (max(k, 1),))[:k].copy(),
           np.ctypeslib.as_array(v, (max(k, 1),))[:k].copy())
    for p in (r, c, v):
        L.ref_mtx_free(ctypes.cast(p, ctypes.c_void_p))
    return (m.value, n.value) + out


def csr_to_rowpair(rowptr, colind, val):
    """The reference's row-pair reuse layout (suitesparse_sdmm.cpp:150-179) from CSR with
    ascending columns: (rowptr2, colind2, val2, flag2)."""
    rowptr, colind = _csr(rowptr, colind)
    M, nnz = rowptr.size - 1, colind.size
    val = np.ascontiguousarray(val, np.float32)
    rp2 = np.zeros(M + 1, np.int32)
    ci2 = np.zeros(max(nnz, 1), np.int32)
    v2 = np.zeros(max(nnz, 1), np.float32)
    f2 = np.zeros(max(nnz, 1), np.uint8)
    lib().or_csr_to_rowpair(M, rowptr, colind, val, rp2, ci2, v2, f2)
    return rp2, ci2[:nnz], v2[:nnz], f2[:nnz]


def spmm_rowpair_f32(rowptr2, colind2, val2, flag2, B, C=None, threads=None):
    """DataReuseSpmm (suitesparse_sdmm.cpp:25-44) over the row-pair layout: C += A*B."""
    rowptr2, colind2 = _csr(rowptr2, colind2)
    M = rowptr2.size - 1
    B = np.ascontiguousarray(B, np.float32)
    C = np.zeros((M, B.shape[1]), np.float32) if C is None else np.ascontiguousarray(C, np.float32).copy()
    lib().or_spmm_rowpair_f32(M, B.shape[1], rowptr2, colind2,
                              np.ascontiguousarray(val2, np.float32),
                              np.ascontiguousarray(flag2, np.uint8), B, B.shape[1], C,
                              B.shape[1], threads or 0)
    return C
