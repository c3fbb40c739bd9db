"""The C-ABI library loads and exports every entry point include/*.h declares; host-side
argument checks work without a GPU (no compute calls here)."""
import ctypes
import os
import re

import pytest
import torch

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols(header="armsparse_gpu.h"):
    syms = set()
    inc = os.path.join(ROOT, "include")
    for name in [header]:
        text = open(os.path.join(inc, name)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"\b(as_[A-Za-z0-9_]+)\s*\(", text):
            syms.add(m.group(1))
    return sorted(syms)


def test_header_declares_entry_points():
    syms = declared_symbols()
    for s in ["as_spmm_csr_f32", "as_spmm_csr_bf16", "as_spmv_csr_f32", "as_spmv_vcsr4_f32",
              "as_sddmm_csr_f32", "as_sddmm_csr_bf16x3", "as_csr2csc", "as_ctx_create"]:
        assert s in syms


def test_library_exports_every_declared_symbol(native_lib):
    missing = [s for s in declared_symbols() if not hasattr(native_lib, s)]
    assert not missing, missing


def test_every_header_is_checked():
    assert sorted(f for f in os.listdir(os.path.join(ROOT, "include")) if f.endswith(".h")) == \
        ["armsparse_drivers.h", "armsparse_gpu.h", "armsparse_mlp.h"]


def test_mlp_header_symbols_exported(native_lib):
    from armsparse_gb300 import _native
    syms = declared_symbols("armsparse_mlp.h")
    assert len(syms) == 4
    assert all(hasattr(native_lib, s) for s in syms) and set(syms) <= set(_native.SIGNATURES)


def test_drivers_library_exports_reference_signatures():
    from armsparse_gb300 import build
    lib = ctypes.CDLL(build.build_drivers())
    missing = [s for s in declared_symbols("armsparse_drivers.h") if not hasattr(lib, s)]
    assert not missing, missing
    # the C++ entry points keep the reference's exact (mangled) signatures
    out = os.popen("nm -D --defined-only " + build.os.path.join(build.PKG, build.DRIVERS_NAME)).read()
    for mangled in ["_Z12rowBaseSpmm3PiS_PfS0_S0_iiii", "_Z12rowBaseSpmm2PiS_PfS0_S0_iiii",
                    "_Z6originPiS_PfS0_S0_iiii", "_Z19sparse_dense_vectorPfS_PiS0_S_ii",
                    "_Z15csr_spmm_kerneliiPiS_PfS0_S0_", "_Z14fast_transposePiS_PSt5mutex",
                    "_Z13DataReuseSpmmPiS_PfS0_S0_iiiiPb", "_Z17toDataReuseFormatPfiiPiS0_S_Pb"]:
        assert mangled in out, mangled


def test_binding_covers_every_declared_symbol():
    from armsparse_gb300 import _native
    assert set(declared_symbols()) <= set(_native.SIGNATURES)


def test_null_context_is_rejected_on_the_host(native_lib):
    from armsparse_gb300 import _native as N
    st = native_lib.as_spmm_csr_f32(None, 4, 4, 4, 0, None, None, None, None, 4, None, 4,
                                    0.0, 0, None)
    assert st == 1  # AS_ERR_INVALID_VALUE
    assert b"ctx is NULL" in native_lib.as_last_error()
    assert native_lib.as_status_string(2) == b"AS_ERR_INVALID_CSR"
    for name in ["as_spmv_csr_f32", "as_spmv_vcsr4_f32"]:
        assert getattr(native_lib, name)(None, 1, 1, 0, None, None, None, None, None, 0.0,
                                         None) == 1
    assert native_lib.as_csr2csc(None, 1, 1, 0, None, None, None, None, None, None, None) == 1


def test_variant_table(native_lib):
    n32, n16 = native_lib.as_spmm_variant_count(0), native_lib.as_spmm_variant_count(1)
    assert n32 >= 90 and n16 >= 120
    names = [native_lib.as_spmm_variant_name(0, i).decode() for i in range(1, n32 + 1)]
    assert len(set(names)) == n32
    assert native_lib.as_spmm_variant_name(0, 0) == b"unknown"
    # the default pick for the 4096-wide fp32 case: full warps, 128-bit loads, the next index
    # batch prefetched; with B only 8-byte aligned, 64-bit loads
    v = native_lib.as_spmm_default_variant(0, 4096, 4096, 4096, 167772, 4096, 4096, 256, 256)
    assert native_lib.as_spmm_variant_name(0, v).decode() == "rowsplit_v16_g32_c2_u4_pf"
    v = native_lib.as_spmm_default_variant(0, 4096, 4096, 4096, 167772, 4096, 4096, 264, 256)
    assert native_lib.as_spmm_variant_name(0, v).decode() == "rowsplit_v8_g32_c4_u4"
    # narrower B: the column tile matched to the width (16-byte vectors where the layout
    # allows them, scalar lanes for N = 3)
    for n_, name in ((3, "rowsplit_v4_g8_c2_u4"), (16, "rowsplit_v16_g2_c2_u4"),
                     (64, "rowsplit_v8_g16_c2_u4"), (128, "rowsplit_v8_g32_c2_u4"),
                     (256, "rowsplit_v16_g32_c2_u4_pf"), (384, "rowsplit_v8_g32_c2_u4")):
        v = native_lib.as_spmm_default_variant(0, 100, 100, n_, 500, n_, n_, 256, 256)
        assert native_lib.as_spmm_variant_name(0, v).decode() == name, n_
    for n_, name in ((128, "rowsplit_v16_g8_c2_u4"), (768, "rowsplit_v16_g32_c1_u4"),
                     (1024, "rowsplit_v16_g32_c2_u4")):
        v = native_lib.as_spmm_default_variant(1, 100, 100, n_, 500, n_, n_, 256, 256)
        assert native_lib.as_spmm_variant_name(1, v).decode() == name, n_


@pytest.mark.skipif(torch.cuda.is_available(), reason="checks the no-GPU error path")
def test_context_creation_fails_loudly_without_gpu(native_lib):
    from armsparse_gb300 import _native as N
    with pytest.raises(N.NativeError):
        N.Context(0)


def test_ops_refuse_cpu_tensors(native_lib):
    import armsparse_gb300 as A
    rp = torch.tensor([0, 1], dtype=torch.int32)
    ci = torch.tensor([0], dtype=torch.int32)
    v = torch.ones(1)
    with pytest.raises(ValueError, match="CUDA"):
        A.spmm(rp, ci, v, torch.ones(1, 4))
    with pytest.raises(ValueError, match="CUDA"):
        A.csr2csc(rp, ci, v, 1)


def test_torch_extension_loads_and_refuses_cpu_tensors():
    from armsparse_gb300 import build
    build.build_torch_extension()
    from armsparse_gb300.torch_ops import spmm
    for name in ["csr_spmm", "csr_sddmm", "coo_sddmm", "csr2csc"]:
        assert hasattr(spmm, name)
    rp = torch.tensor([0, 1], dtype=torch.int32)
    with pytest.raises(RuntimeError, match="CUDA"):
        spmm.csr_spmm(rp, torch.tensor([0], dtype=torch.int32), torch.ones(1), torch.ones(1, 4))


def test_variant_feasibility_query(native_lib):
    import armsparse_gb300 as A
    names = A.spmm_variants()
    idx = {n: i + 1 for i, n in enumerate(names)}
    assert A.spmm_variant_supported(idx["nnzsplit_v16_g32_c1_ch128"], 64)
    assert not A.spmm_variant_supported(idx["nnzsplit_v16_g32_c1_ch128"], 3)
    assert A.spmm_variant_supported(idx["rowsplit_v4_g32_c2_u8"], 3)
    assert not A.spmm_variant_supported(idx["rowsplit_v16_g32_c2_u4"], 6)
    assert not A.spmm_variant_supported(idx["bulk_lb16_s8"], 6)
    # every default pick is feasible
    for N_ in (1, 3, 47, 64, 4096):
        v = native_lib.as_spmm_default_variant(0, 100, 100, N_, 500, N_, N_, 256, 256)
        assert A.spmm_variant_supported(v, N_)


def test_selector_model_names_known_variants(native_lib):
    """Every candidate of the shipped selector model (and of the sweep list) is a kernel of
    both variant tables, and the multi-entry family is in the tables."""
    import json
    import armsparse_gb300 as A
    from armsparse_gb300 import selector as SEL
    with open(SEL.DEFAULT_MODEL) as f:
        model = json.load(f)
    for dt in (torch.float32, torch.bfloat16):
        names = set(A.spmm_variants(dt))
        assert set(model["candidates"]) <= names
        assert set(SEL.CANDIDATES) <= names
        assert {n for n in names if n.startswith("nnzme_")}
    assert len(model["weights"][-1]) == len(model["candidates"])  # one score per candidate


def test_multi_entry_and_fused_feasibility(native_lib):
    import armsparse_gb300 as A
    from armsparse_gb300 import gcn
    names = A.spmm_variants(torch.bfloat16)
    idx = {n: i + 1 for i, n in enumerate(names)}
    assert A.spmm_variant_supported(idx["nnzme_v8_g16_ch1024"], 48, torch.bfloat16)
    assert not A.spmm_variant_supported(idx["nnzme_v8_g16_ch1024"], 46, torch.bfloat16)  # 4 | N
    assert gcn._nnz_tile("nnzme_v8_g16_ch1024", 2) == 64
    assert gcn._nnz_tile("nnzsplit_v16_g32_c2_ch1024_u8", 2) == 512
    assert gcn._nnz_tile("nnzsplit_v4_g32_c1_ch128", 4) == 32


def test_new_ops_validate_on_the_host():
    """Argument errors of the fused, gather and loss wrappers are raised before any device
    work (here, on CPU tensors)."""
    import armsparse_gb300 as A
    rp = torch.tensor([0, 1], dtype=torch.int32)
    ci = torch.tensor([0], dtype=torch.int32)
    with pytest.raises(ValueError, match="CUDA"):
        A.spmm_sddmm(rp, ci, torch.ones(1), torch.ones(1, 4), torch.ones(1, 4))
    with pytest.raises(ValueError, match="CUDA"):
        A.gather(torch.ones(4), torch.zeros(2, dtype=torch.int32))
    with pytest.raises(ValueError, match="CUDA"):
        A.softmax_xent(torch.zeros(2, 8, dtype=torch.bfloat16), torch.zeros(2, dtype=torch.long), 8)
    with pytest.raises(ValueError, match="CUDA"):
        A.csr2csc_perm(rp, ci, 1)
