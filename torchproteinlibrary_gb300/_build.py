"""In-tree build of the native parts.

* ``lib/libtpl_gb300.so``: the CUDA kernels and the C ABI (include/tpl_gb300.h),
  compiled by nvcc for sm_103a only.
* ``_ReducedModel*.so`` / ``_FullAtomModel*.so``: the torch extension modules that
  keep the reference's entry-point names, compiled by g++ against torch's headers
  and linked to libtpl_gb300.so.

Everything is written inside the package directory (git-ignored), so the
interpreter that runs the tests loads the freshly built in-tree files.
"""
from __future__ import annotations

import os
import subprocess
import sys
import sysconfig
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
LIBDIR = os.path.join(PKG, "lib")
OBJDIR = os.path.join(PKG, "_objs")
INCLUDE = os.path.join(ROOT, "include")
LIBNAME = "libtpl_gb300.so"

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

CU_SOURCES = ["tpl_a2b.cu", "tpl_a2b_chain.cu", "tpl_a2c.cu", "tpl_rmsd.cu", "tpl_transform.cu", "tpl_typed.cu", "tpl_pdb.cpp", "tpl_capi.cu", "tpl_noalloc.cu"]
EXTENSIONS = {"_ReducedModel": "ext/reduced_model.cpp", "_FullAtomModel": "ext/full_atom_model.cpp",
              "_RMSD": "ext/rmsd.cpp"}


def _ext_suffix() -> str:
    return sysconfig.get_config_var("EXT_SUFFIX") or ".so"


def lib_path() -> str:
    return os.path.join(LIBDIR, LIBNAME)


def ext_path(name: str) -> str:
    return os.path.join(PKG, name + _ext_suffix())


def _headers() -> list[str]:
    hs = [os.path.join(INCLUDE, "tpl_gb300.h")]
    for f in os.listdir(CSRC):
        if f.endswith((".h", ".cuh")):
            hs.append(os.path.join(CSRC, f))
    return hs


def _stale(out: str, deps: list[str]) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout)


def _nvcc_obj(src: str) -> str:
    obj = os.path.join(OBJDIR, os.path.splitext(src)[0] + ".o")
    deps = [os.path.join(CSRC, src)] + _headers()
    if _stale(obj, deps):
        _run([NVCC, *ARCH, "-lineinfo", "-O3", "-std=c++17", "--expt-relaxed-constexpr", "-Xcompiler", "-fPIC",
              "-I", INCLUDE, "-c",
              os.path.join(CSRC, src), "-o", obj])
    return obj


def build_native(verbose: bool = False) -> str:
    """Compile libtpl_gb300.so (sm_103a).  Returns its path."""
    os.makedirs(LIBDIR, exist_ok=True)
    os.makedirs(OBJDIR, exist_ok=True)
    srcs = [s for s in CU_SOURCES if os.path.exists(os.path.join(CSRC, s))]
    with ThreadPoolExecutor(max_workers=len(srcs)) as ex:
        objs = list(ex.map(_nvcc_obj, srcs))
    out = lib_path()
    if _stale(out, objs):
        _run([NVCC, *ARCH, "-shared", "-o", out, *objs, "-lcudart"])
        if verbose:
            print("built", out)
    return out


def _torch_flags():
    import torch
    from torch.utils import cpp_extension as ce

    inc = ce.include_paths(device_type="cuda") if "device_type" in ce.include_paths.__code__.co_varnames else \
        ce.include_paths(cuda=True)
    libdirs = ce.library_paths(device_type="cuda") if "device_type" in ce.library_paths.__code__.co_varnames else \
        ce.library_paths(cuda=True)
    abi = int(torch._C._GLIBCXX_USE_CXX11_ABI)
    return inc, libdirs, abi


def _build_ext(name: str) -> str:
    src = os.path.join(CSRC, EXTENSIONS[name])
    out = ext_path(name)
    if not os.path.exists(src):
        return ""
    if not _stale(out, [src, lib_path()] + _headers()):
        return out
    inc, libdirs, abi = _torch_flags()
    py_inc = sysconfig.get_paths()["include"]
    cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-shared", f"-D_GLIBCXX_USE_CXX11_ABI={abi}",
           f"-DTORCH_EXTENSION_NAME={name}", "-DTORCH_API_INCLUDE_EXTENSION_H", "-w"]
    cmd += [f"-I{p}" for p in inc] + [f"-I{py_inc}", f"-I{os.path.join(CUDA_HOME, 'include')}", f"-I{INCLUDE}"]
    cmd += [src, "-o", out]
    cmd += [f"-L{p}" for p in libdirs] + [f"-L{LIBDIR}", "-ltpl_gb300", "-lc10", "-lc10_cuda", "-ltorch",
                                          "-ltorch_cpu", "-ltorch_python",
                                          f"-L{os.path.join(CUDA_HOME, 'lib64')}", "-lcudart",
                                          "-Wl,-rpath,$ORIGIN/lib"]
    cmd += [f"-Wl,-rpath,{p}" for p in libdirs]
    _run(cmd)
    return out


def build_extensions() -> list[str]:
    names = [n for n in EXTENSIONS if os.path.exists(os.path.join(CSRC, EXTENSIONS[n]))]
    with ThreadPoolExecutor(max_workers=max(1, len(names))) as ex:
        return list(ex.map(_build_ext, names))


def build_all(verbose: bool = False) -> None:
    build_native(verbose)
    build_extensions()


if __name__ == "__main__":
    build_all(verbose=True)
    sys.exit(0)
