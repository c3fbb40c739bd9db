"""Build recipe for the native parts of armsparse_gb300 (in-tree, sm_103a only).

Products (all git-ignored, rebuilt on every machine that runs them):

* ``armsparse_gb300/libarmsparse_gpu.so`` -- the CUDA kernels behind the C ABI declared in
  ``include/armsparse_gpu.h`` (nvcc, ``-gencode arch=compute_103a,code=sm_103a``);
* ``armsparse_gb300/libarmsparse_drivers.so`` -- C++ host shims with the reference drivers'
  exact signatures (rowBaseSpmm3, sparse_dense_vector, ...), linked to the library above;
* ``armsparse_gb300/spmm*.so`` -- the PyTorch C++ extension named ``spmm`` (the GCN op).

Translation units compile in parallel; an object is rebuilt only when its source, a header
or the flags changed.
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys
import sysconfig

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(ROOT, "_build")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                     "-I" + INCLUDE, "-I" + CSRC]
CU_SOURCES = ["api.cu", "spmm.cu", "spmm_bulk.cu", "spmm_nnz.cu", "spmm_long.cu", "spmv.cu", "sddmm_simt.cu", "sddmm_tc.cu", "transpose.cu",
              "fp64.cu", "mlp.cu", "formats.cu", "spmm_reduce.cu", "spgemm_dense.cu", "spmm_rowpair.cu",
              "spmm_vcsr4.cu",
              "xent.cu"]
LIB_NAME = "libarmsparse_gpu.so"
DRIVERS_NAME = "libarmsparse_drivers.so"


def nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build armsparse_gb300")
    return cand


def _headers() -> list[str]:
    hs = [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    hs += [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    return hs


def _stamp(src: str, flags: list[str]) -> str:
    h = hashlib.sha1()
    for p in [src] + _headers():
        with open(p, "rb") as f:
            h.update(f.read())
    h.update(" ".join(flags).encode())
    return h.hexdigest()


def _compile(src: str, obj: str, cmd: list[str]) -> str:
    stamp_file = obj + ".stamp"
    stamp = _stamp(src, cmd)
    if os.path.exists(obj) and os.path.exists(stamp_file):
        with open(stamp_file) as f:
            if f.read() == stamp:
                return obj
    out = subprocess.run(cmd, capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{out.stdout}\n{out.stderr}")
    with open(stamp_file, "w") as f:
        f.write(stamp)
    return obj


def _link(out_path: str, objs: list[str], cmd_tail: list[str], head: list[str]) -> None:
    cmd = head + objs + cmd_tail + ["-o", out_path + ".tmp"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    os.replace(out_path + ".tmp", out_path)


def build_library(jobs: int | None = None, verbose: bool = False) -> str:
    """Compile the CUDA sources and link ``libarmsparse_gpu.so``; returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    tasks = []
    for name in CU_SOURCES:
        src = os.path.join(CSRC, name)
        obj = os.path.join(BUILD, name.replace(".cu", ".o"))
        tasks.append((src, obj, [cc] + NVCC_FLAGS + ["-c", src, "-o", obj]))
    jobs = jobs or min(len(tasks), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(jobs) as ex:
        objs = list(ex.map(lambda t: _compile(*t), tasks))
    lib = os.path.join(PKG, LIB_NAME)
    newest = max(os.path.getmtime(o) for o in objs)
    if not os.path.exists(lib) or os.path.getmtime(lib) < newest:
        _link(lib, objs, ["-lcudart_static"], [cc] + ARCH + ["-shared", "-Xcompiler", "-fPIC"])
    if verbose:
        print("built", lib)
    return lib


def build_drivers(verbose: bool = False) -> str:
    """Host shims with the reference drivers' signatures, linked against the C-ABI library."""
    lib = build_library()
    src = os.path.join(CSRC, "drivers.cu")
    out = os.path.join(PKG, DRIVERS_NAME)
    cmd = ([nvcc()] + NVCC_FLAGS + ["-shared", src, "-L" + PKG, "-larmsparse_gpu",
                                    "-lcudart_static", "-lpthread", "-Xlinker", "-rpath,$ORIGIN",
                                    "-o", out + ".tmp"])
    stamp = _stamp(src, cmd)
    sf = os.path.join(BUILD, "drivers.stamp")
    if os.path.exists(out) and os.path.exists(sf) and open(sf).read() == stamp \
            and os.path.getmtime(out) >= os.path.getmtime(lib):
        return out
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"drivers build failed:\n{res.stdout}\n{res.stderr}")
    os.replace(out + ".tmp", out)
    with open(sf, "w") as f:
        f.write(stamp)
    if verbose:
        print("built", out)
    return out


def build_torch_extension(verbose: bool = False) -> str:
    """The ``spmm`` PyTorch C++ extension (csr_spmm and friends), built with g++ against
    torch's headers and linked to the C-ABI library; returns the module path."""
    import torch  # noqa: F401  (only for its include/library paths)
    from torch.utils import cpp_extension as ce

    lib = build_library()
    src = os.path.join(CSRC, "torch_spmm.cpp")
    suffix = sysconfig.get_config_var("EXT_SUFFIX") or ".so"
    out = os.path.join(PKG, "spmm" + suffix)
    cuda_inc = os.path.join(os.path.dirname(os.path.dirname(nvcc())), "include")
    incs = ["-I" + p for p in ce.include_paths()] + ["-I" + sysconfig.get_paths()["include"],
                                                     "-I" + INCLUDE, "-I" + cuda_inc]
    torch_lib = os.path.join(os.path.dirname(torch.__file__), "lib")
    abi = int(torch._C._GLIBCXX_USE_CXX11_ABI)
    cmd = (["g++", "-O2", "-std=c++17", "-fPIC", "-shared", f"-D_GLIBCXX_USE_CXX11_ABI={abi}",
            "-DTORCH_EXTENSION_NAME=spmm", "-DTORCH_API_INCLUDE_EXTENSION_H"] + incs +
           [src, "-L" + PKG, "-larmsparse_gpu", "-L" + torch_lib, "-lc10", "-ltorch",
            "-ltorch_cpu", "-ltorch_python", "-Wl,-rpath,$ORIGIN", "-Wl,-rpath," + torch_lib,
            "-o", out + ".tmp"])
    stamp = _stamp(src, cmd)
    sf = os.path.join(BUILD, "torch_spmm.stamp")
    if os.path.exists(out) and os.path.exists(sf) and open(sf).read() == stamp \
            and os.path.getmtime(out) >= os.path.getmtime(lib):
        return out
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"torch extension build failed:\n{res.stdout}\n{res.stderr}")
    os.replace(out + ".tmp", out)
    with open(sf, "w") as f:
        f.write(stamp)
    if verbose:
        print("built", out)
    return out


def build_all(verbose: bool = False) -> None:
    build_library(verbose=verbose)
    with cf.ThreadPoolExecutor(2) as ex:
        futs = []
        if os.path.exists(os.path.join(CSRC, "drivers.cu")):
            futs.append(ex.submit(build_drivers, verbose))
        if os.path.exists(os.path.join(CSRC, "torch_spmm.cpp")):
            futs.append(ex.submit(build_torch_extension, verbose))
        for f in futs:
            f.result()


if __name__ == "__main__":
    build_all(verbose=True)
    sys.exit(0)
