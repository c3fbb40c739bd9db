"""Generate the golden vectors in this folder from the reference's own kernels.

Run with the path of a reference checkout (REF, required):

    python tests/golden/make_golden.py REF [--only NAME]

It compiles the reference's SDMM.cpp, SpMV.cpp and sparseTranspose.cpp unmodified through
oracle/Makefile (target ``ref``; on x86_64 a scalar NEON shim stands in for <arm_neon.h>),
runs them on small seeded inputs and saves inputs and outputs as .npz files:

* spmm_rowbasespmm3.npz -- rowBaseSpmm3 (SDMM.cpp:90-114) from a zeroed C, and after a
  second call (the driver's accumulate pattern, SDMM.cpp:277-283), plus origin
  (SDMM.cpp:422-448) and rowBaseSpmm2 (SDMM.cpp:65-89, its cblas_saxpy restated as
  OpenBLAS's fused kernels compute it: oracle/ref_bridge/cblas_saxpy.c); A built by the reference's toCSR (SDMM.cpp:355-370) from a dense
  matrix;
* spmv_vcsr4.npz -- toVectorAwareCSR (SpMV.cpp:15-38) and sparse_dense_vector
  (SpMV.cpp:155-179);
* spgemm_dense.npz -- sparse_matrix_mul3 (SpMM.cpp:309-327): A and B in CSR (row-major
  scan, ascending columns, as toCSR writes them), C dense, accumulated over two calls;
* transpose_triplets.npz -- convert (sparseTranspose.cpp:71-92) and fast_transpose
  (sparseTranspose.cpp:95-142) run on one thread (stable order);
* rowpair_reuse.npz -- the row-pair reuse layout toDataReuseFormat (suitesparse_sdmm.cpp:
  150-179) and DataReuseSpmm (:25-44) over it, A built by that file's toCSR;
* mtx_reader.npz -- the reference's Matrix Market reader readMtx<float> (gcn/util/util.hpp:
  286-333, with makeSymmetric :218-284) on small seeded .mtx texts (stored in the file):
  symmetric real and pattern files with self-loops and duplicates, general real with
  duplicates, integer with upper-case qualifiers, skew-symmetric;
* gcn_op.npz -- the reference's own gcn/pytorch-custom/op.py imported as is: its
  SPMMFunction forward and backward and one GCNConv forward+backward on a small seeded graph.
  The module's ``spmm = load(name='spmm', ...)`` (op.py:6) is served by the reference's
  compiled csr_spmm_kernel (spmm.cpp:49-71, oracle target ``ref-gcn``) called with a zeroed
  output (spmm.cpp:41 leaves it uninitialised), and ``torch_geometric.nn.inits`` -- not
  installed -- by a stub whose glorot/zeros follow pytorch_geometric's inits.py:30-33, :58-59.

The fixtures are small (a few hundred KB in total) and the GPU tests read only them, never
the reference.
"""
from __future__ import annotations

import ctypes
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from oracle import oracle as O  # noqa: E402


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def dense_sparse(rng, rows, cols, density, kind="ref_int"):
    d = np.zeros((rows, cols), np.float32)
    nnz = int(density * rows * cols)
    pos = rng.choice(rows * cols, nnz, replace=False)
    if kind == "ref_int":
        v = ((rng.integers(0, 20000, nnz) - 10000) / 1000.0).astype(np.float32)
    else:
        v = rng.uniform(-1, 1, nnz).astype(np.float32)
    v[v == 0] = 0.5
    d.flat[pos] = v
    return d


def spmm_cases(ref):
    cases = [(64, 48, 32, 0.08, 1), (50, 40, 7, 0.2, 2), (33, 33, 3, 0.1, 3),
             (40, 64, 130, 0.15, 4), (16, 16, 1, 0.3, 5), (8, 7, 6, 0.45, 6)]
    out = {}
    for i, (M, K, N, dens, seed) in enumerate(cases):
        rng = np.random.default_rng(1000 + seed)
        dense = dense_sparse(rng, M, K, dens)
        if i == 0:
            dense[5, :] = 0  # an empty row
        nnz = int((dense != 0).sum())
        rowptr = np.zeros(M + 1, np.int32)
        colind = np.zeros(max(nnz, 1), np.int32)
        val = np.zeros(max(nnz, 1), np.float32)
        ref.ref_toCSR(_p(dense), M, K, _p(rowptr), _p(colind), _p(val))
        B = rng.uniform(-1, 1, (K, N)).astype(np.float32)
        C1 = np.zeros((M, N), np.float32)
        ref.ref_rowBaseSpmm3(_p(rowptr), _p(colind), _p(val), _p(B), _p(C1), M, K, N, 4)
        C2 = C1.copy()
        ref.ref_rowBaseSpmm3(_p(rowptr), _p(colind), _p(val), _p(B), _p(C2), M, K, N, 4)
        Co = np.zeros((M, N), np.float32)
        ref.ref_origin(_p(rowptr), _p(colind), _p(val), _p(B), _p(Co), M, K, N, 4)
        Cs = np.zeros((M, N), np.float32)
        ref.ref_rowBaseSpmm2(_p(rowptr), _p(colind), _p(val), _p(B), _p(Cs), M, K, N, 4)
        out.update({f"c{i}_shape": np.array([M, K, N], np.int32), f"c{i}_rowptr": rowptr,
                    f"c{i}_colind": colind[:nnz], f"c{i}_val": val[:nnz], f"c{i}_B": B,
                    f"c{i}_C": C1, f"c{i}_C_twice": C2, f"c{i}_C_origin": Co,
                    f"c{i}_C_saxpy": Cs})
    out["n_cases"] = np.array(len(cases), np.int32)
    np.savez_compressed(os.path.join(HERE, "spmm_rowbasespmm3.npz"), **out)


def spmv_cases(ref):
    cases = [(37, 64, 0.1, 11), (64, 128, 0.03, 12), (5, 8, 0.5, 13)]
    out = {}
    for i, (M, K, dens, seed) in enumerate(cases):
        rng = np.random.default_rng(2000 + seed)
        dense = dense_sparse(rng, M, K, dens, kind="u11")
        cap = 4 * M * K
        rowptr = np.zeros(M + 1, np.int32)
        colind = np.zeros(cap, np.int32)
        val = np.zeros(cap, np.float32)
        ref.ref_toVectorAwareCSR(_p(dense), M, K, _p(rowptr), _p(colind), _p(val))
        n = int(rowptr[M])
        x = rng.uniform(-1, 1, K).astype(np.float32)
        y = np.zeros(M, np.float32)
        ref.ref_sparse_dense_vector(_p(x), _p(y), _p(rowptr), _p(colind), _p(val), M, 1)
        # the same matrix in plain CSR, for the layout converter
        rows, cols = np.nonzero(dense)
        crow = np.zeros(M + 1, np.int32)
        np.cumsum(np.bincount(rows, minlength=M), out=crow[1:])
        out.update({f"c{i}_shape": np.array([M, K], np.int32), f"c{i}_vrowptr": rowptr,
                    f"c{i}_vcolind": colind[:n], f"c{i}_vval": val[:n], f"c{i}_x": x,
                    f"c{i}_y": y, f"c{i}_rowptr": crow, f"c{i}_colind": cols.astype(np.int32),
                    f"c{i}_val": dense[rows, cols].astype(np.float32)})
    out["n_cases"] = np.array(len(cases), np.int32)
    np.savez_compressed(os.path.join(HERE, "spmv_vcsr4.npz"), **out)


def _csr_of(dense):
    rows, cols = np.nonzero(dense)
    rp = np.zeros(dense.shape[0] + 1, np.int32)
    np.cumsum(np.bincount(rows, minlength=dense.shape[0]), out=rp[1:])
    return rp, cols.astype(np.int32), dense[rows, cols].astype(np.float32)


def spgemm_cases(ref):
    cases = [(64, 48, 40, 0.1, 0.1, 31), (30, 50, 7, 0.2, 0.3, 32), (16, 16, 16, 0.3, 0.3, 33),
             (100, 80, 130, 0.05, 0.08, 34)]
    out = {}
    for i, (M, K, N, da, db, seed) in enumerate(cases):
        rng = np.random.default_rng(4000 + seed)
        A = dense_sparse(rng, M, K, da, kind="u11")
        B = dense_sparse(rng, K, N, db, kind="u11")
        if i == 0:
            A[3, :] = 0  # an empty row of A
            B[7, :] = 0  # an empty row of B
        rp1, ci1, v1 = _csr_of(A)
        rp2, ci2, v2 = _csr_of(B)
        C1 = np.zeros((M, N), np.float32)
        ref.ref_sparse_matrix_mul3(_p(rp1), _p(ci1), _p(v1), _p(rp2), _p(ci2), _p(v2), _p(C1),
                                   M, K, N, 4)
        C2 = C1.copy()
        ref.ref_sparse_matrix_mul3(_p(rp1), _p(ci1), _p(v1), _p(rp2), _p(ci2), _p(v2), _p(C2),
                                   M, K, N, 4)
        out.update({f"c{i}_shape": np.array([M, K, N], np.int32), f"c{i}_a_rowptr": rp1,
                    f"c{i}_a_colind": ci1, f"c{i}_a_val": v1, f"c{i}_b_rowptr": rp2,
                    f"c{i}_b_colind": ci2, f"c{i}_b_val": v2, f"c{i}_C": C1,
                    f"c{i}_C_twice": C2})
    out["n_cases"] = np.array(len(cases), np.int32)
    np.savez_compressed(os.path.join(HERE, "spgemm_dense.npz"), **out)


def transpose_cases(ref):
    cases = [(30, 20, 0.1, 21), (7, 40, 0.3, 22), (64, 64, 0.05, 23)]
    out = {}
    for i, (M, N, dens, seed) in enumerate(cases):
        rng = np.random.default_rng(3000 + seed)
        A = np.zeros((M, N), np.int32)
        nnz = int(dens * M * N)
        A.flat[rng.choice(M * N, nnz, replace=False)] = rng.integers(1, 100, nnz)
        sm = np.zeros(((nnz + 1) * 3,), np.int32)
        ref.ref_convert(_p(A), _p(sm), M, N)
        res = np.zeros_like(sm)
        ref.ref_fast_transpose(_p(sm), _p(res), 1)
        out.update({f"c{i}_dense": A, f"c{i}_triplets": sm, f"c{i}_transposed": res})
    out["n_cases"] = np.array(len(cases), np.int32)
    np.savez_compressed(os.path.join(HERE, "transpose_triplets.npz"), **out)


def rowpair_cases(ref):
    """The reference's row-pair reuse layout (toDataReuseFormat) and DataReuseSpmm on small
    seeded matrices whose paired rows share columns (half of each odd row's columns copied from
    the even row above it), an odd row count included."""
    cases = [(64, 80, 32, 0.1, 41), (33, 40, 7, 0.2, 42), (50, 64, 130, 0.15, 43),
             (16, 16, 1, 0.3, 44)]
    out = {}
    for i, (M, K, N, dens, seed) in enumerate(cases):
        rng = np.random.default_rng(6000 + seed)
        dense = dense_sparse(rng, M, K, dens)
        for r in range(1, M, 2):  # let pairs share columns
            share = (dense[r - 1] != 0) & (rng.random(K) < 0.5)
            dense[r, share] = rng.uniform(-1, 1, int(share.sum())).astype(np.float32) + 2.0
        nnz = int((dense != 0).sum())
        rowptr = np.zeros(M + 1, np.int32)
        colind = np.zeros(max(nnz, 1), np.int32)
        val = np.zeros(max(nnz, 1), np.float32)
        ref.ref_toCSR_rp(_p(dense), M, K, _p(rowptr), _p(colind), _p(val))
        work = dense.copy()
        rp2 = np.zeros(M + 1, np.int32)
        ci2 = np.zeros(max(nnz, 1), np.int32)
        v2 = np.zeros(max(nnz, 1), np.float32)
        f2 = np.zeros(max(nnz, 1), np.uint8)
        ref.ref_toDataReuseFormat(_p(work), M, K, _p(rp2), _p(ci2), _p(v2), _p(f2))
        B = rng.uniform(-1, 1, (K, N)).astype(np.float32)
        C = np.zeros((M, N), np.float32)
        ref.ref_DataReuseSpmm(_p(rp2), _p(ci2), _p(v2), _p(B), _p(C), M, K, N, 4, _p(f2))
        out.update({f"c{i}_shape": np.array([M, K, N], np.int32), f"c{i}_rowptr": rowptr,
                    f"c{i}_colind": colind[:nnz], f"c{i}_val": val[:nnz], f"c{i}_B": B,
                    f"c{i}_rowptr2": rp2, f"c{i}_colind2": ci2[:nnz], f"c{i}_val2": v2[:nnz],
                    f"c{i}_flag2": f2[:nnz], f"c{i}_C": C})
    out["n_cases"] = np.array(len(cases), np.int32)
    np.savez_compressed(os.path.join(HERE, "rowpair_reuse.npz"), **out)


def mtx_texts():
    """Small seeded Matrix Market files covering what the reference's reader distinguishes:
    symmetric (mirrors, self-loops, duplicates, real values that the compaction misaligns),
    symmetric pattern, general with duplicates kept, integer, skew-symmetric (read as stored),
    upper-case qualifiers and comment lines."""
    rng = np.random.default_rng(4242)
    texts = {}

    def body(n, m, entries, field):
        lines = [f"{n} {m} {len(entries)}"]
        for r, c, v in entries:
            lines.append(f"{r + 1} {c + 1}" + ("" if field == "pattern" else f" {v}"))
        return "\n".join(lines) + "\n"

    def entries(n, m, k, field, diag=0, dups=0, lower=False):
        # symmetric (lower) files get distinct keys plus exact duplicate lines: the value that
        # survives a run of equal keys follows std::sort's unspecified order of equal elements,
        # so only same-valued duplicates give a result that does not depend on it
        out, seen = [], set()
        for _ in range(k):
            r, c = int(rng.integers(0, n)), int(rng.integers(0, m))
            if lower and c > r:
                r, c = c, r
            if lower and ((r, c) in seen or r == c):
                continue
            seen.add((r, c))
            v = int(rng.integers(-9, 10)) if field == "integer" else float(np.float32(rng.normal()))
            out.append((r, c, v))
        for i in rng.choice(min(n, m), diag, replace=False):
            out.append((int(i), int(i), 1.5))
        for _ in range(dups):
            out.append(out[int(rng.integers(0, len(out)))])
        order = rng.permutation(len(out))
        return [out[i] for i in order]

    texts["sym_real"] = ("%%MatrixMarket matrix coordinate real symmetric\n% seeded\n" +
                         body(40, 40, entries(40, 40, 120, "real", diag=6, dups=5, lower=True), "real"))
    texts["sym_pattern"] = ("%%MatrixMarket matrix coordinate pattern symmetric\n" +
                            body(60, 60, entries(60, 60, 200, "pattern", diag=4, dups=7, lower=True), "pattern"))
    texts["general_real"] = ("%%MatrixMarket matrix coordinate real general\n%\n% two comments\n" +
                             body(30, 45, entries(30, 45, 150, "real", diag=3, dups=6), "real"))
    texts["general_int"] = ("%%MatrixMarket MATRIX Coordinate INTEGER General\n" +
                            body(25, 25, entries(25, 25, 90, "integer"), "integer"))
    texts["skew_real"] = ("%%MatrixMarket matrix coordinate real skew-symmetric\n" +
                          body(20, 20, entries(20, 20, 50, "real", lower=True), "real"))
    return texts


def mtx_cases():
    import tempfile
    out = {}
    names = sorted(mtx_texts().items())
    with tempfile.TemporaryDirectory() as td:
        for i, (name, text) in enumerate(names):
            path = os.path.join(td, name + ".mtx")
            with open(path, "w") as f:
                f.write(text)
            m, n, r, c, v = O.ref_read_mtx(path)
            out.update({f"c{i}_name": np.array(name), f"c{i}_text": np.array(text),
                        f"c{i}_shape": np.array([m, n], np.int32), f"c{i}_rows": r,
                        f"c{i}_cols": c, f"c{i}_vals": v})
    out["n_cases"] = np.array(len(names), np.int32)
    np.savez_compressed(os.path.join(HERE, "mtx_reader.npz"), **out)


def gcn_cases(ref_dir):
    import types

    import torch
    import torch.utils.cpp_extension as ce

    lib = O.ref_lib("gcnspmm")
    if lib is None:
        raise SystemExit("oracle/_ref/libref_gcnspmm.so missing (make -C oracle ref-gcn)")

    def csr_spmm(rowptr, colind, values, dense):
        rp = np.ascontiguousarray(rowptr.numpy().astype(np.int32))
        ci = np.ascontiguousarray(colind.numpy().astype(np.int32))
        v = np.ascontiguousarray(values.detach().numpy().astype(np.float32))
        B = np.ascontiguousarray(dense.detach().numpy().astype(np.float32))
        C = np.zeros((rp.size - 1, B.shape[1]), np.float32)
        lib.ref_csr_spmm_kernel(rp.size - 1, B.shape[1], _p(rp), _p(ci), _p(v), _p(B), _p(C))
        return torch.from_numpy(C)

    fake = types.SimpleNamespace(csr_spmm=csr_spmm)
    saved_load = ce.load
    ce.load = lambda *a, **k: fake
    inits = types.ModuleType("torch_geometric.nn.inits")

    def glorot(t):
        a = (6.0 / (t.size(-2) + t.size(-1))) ** 0.5
        t.data.uniform_(-a, a)

    inits.glorot = glorot
    inits.zeros = lambda t: t.data.fill_(0.0) if t is not None else None
    for name in ["torch_geometric", "torch_geometric.nn"]:
        sys.modules.setdefault(name, types.ModuleType(name))
    sys.modules["torch_geometric.nn.inits"] = inits
    sys.path.insert(0, os.path.join(ref_dir, "gcn", "pytorch-custom"))
    try:
        import op  # the reference's module, unmodified
    finally:
        ce.load = saved_load
        sys.path.pop(0)

    from armsparse_gb300 import synthetic as syn
    a = syn.powerlaw_graph(300, 1600, seed=5)
    n = a.n_rows
    rng = np.random.default_rng(6)
    w = rng.uniform(0.5, 1.5, a.nnz).astype(np.float32)  # weighted edges
    cp, ri, cw = O.csr2csc(a.rowptr, a.colind, w, n)
    t = lambda x: torch.from_numpy(np.ascontiguousarray(x))
    feat = rng.standard_normal((n, 16)).astype(np.float32)
    gout = rng.standard_normal((n, 16)).astype(np.float32)
    f = t(feat).requires_grad_(True)
    out = op.SPMMFunction.apply(t(a.rowptr), t(a.colind), t(cp), t(ri), f, t(w), t(cw))
    out.backward(t(gout))
    # GCNConv with fixed weights: forward and input gradient
    conv = op.GCNConv(16, 8, cached=True, normalize=True)
    W = rng.standard_normal((16, 8)).astype(np.float32) * 0.3
    bvec = rng.standard_normal(8).astype(np.float32) * 0.1
    with torch.no_grad():
        conv.weight.copy_(t(W))
        conv.bias.copy_(t(bvec))
    x = t(feat).requires_grad_(True)
    y = conv(x, t(a.rowptr), t(a.colind), t(cp), t(ri), t(w), t(cw))
    gy = rng.standard_normal((n, 8)).astype(np.float32)
    y.backward(t(gy))
    np.savez_compressed(os.path.join(HERE, "gcn_op.npz"), rowptr=a.rowptr, colind=a.colind,
                        val=w, colptr=cp, rowind=ri, val_csc=cw, feat=feat, grad_out=gout,
                        out=out.detach().numpy(), grad_feat=f.grad.numpy(), W=W, b=bvec,
                        conv_out=y.detach().numpy(), conv_grad_out=gy,
                        conv_grad_x=x.grad.numpy(), conv_grad_W=conv.weight.grad.numpy(),
                        conv_grad_b=conv.bias.grad.numpy())


def main():
    args = [a for a in sys.argv[1:] if not a.startswith("--")]
    only = sys.argv[sys.argv.index("--only") + 1] if "--only" in sys.argv else None
    if only:
        args = [a for a in args if a != only]
    if not args:
        raise SystemExit("usage: make_golden.py REF [--only NAME] (REF: the reference checkout)")
    ref_dir = args[0]
    if not O.build_ref(ref_dir):
        raise SystemExit("could not build the reference kernels from " + ref_dir)
    makers = {"spmm": lambda: spmm_cases(O.ref_lib("sdmm")),
              "spmv": lambda: spmv_cases(O.ref_lib("spmv")),
              "transpose": lambda: transpose_cases(O.ref_lib("transpose")),
              "spgemm": lambda: spgemm_cases(O.ref_lib("spgemm")),
              "mtx": mtx_cases,
              "rowpair": lambda: rowpair_cases(O.ref_lib("rowpair"))}
    for name, make in makers.items():
        if only in (None, name):
            make()
    if only in (None, "gcn") and O.build_ref(ref_dir, gcn=True):
        gcn_cases(ref_dir)
    print("golden vectors written to", HERE)


if __name__ == "__main__":
    main()
