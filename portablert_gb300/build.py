"""Builds the CUDA shared library libprt_b200.so (sm_103a) in-tree.

Every .cu file under csrc/ is compiled to an object in parallel, then linked with
nvcc into ``portablert_gb300/_build/libprt_b200.so``.  The host-side C++ backend test
program (portableRT API + B200Backend) is built beside it when a C++ compiler is
present.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_build")
LIB = os.path.join(OUT, "libprt_b200.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
              "--expt-relaxed-constexpr", f"-I{os.path.join(ROOT, 'include')}"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    hs.append(os.path.join(ROOT, "include", "prt_b200.h"))
    return hs


def _stale(target, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps if os.path.exists(d))


def _compile(src, extra=()):
    obj = os.path.join(OUT, os.path.basename(src)[:-3] + ".o")
    if not _stale(obj, [src] + _headers()):
        return obj
    cmd = [nvcc()] + ARCH + NVCC_FLAGS + list(extra) + ["-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build_library(verbose: bool = False, extra=()) -> str:
    os.makedirs(OUT, exist_ok=True)
    srcs = _sources()
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), srcs))
    if _stale(LIB, objs):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    if verbose:
        print(f"built {LIB}", file=sys.stderr)
    return LIB


CPP_TEST = os.path.join(OUT, "b200_api_test")


def build_cpp_test(verbose: bool = False) -> str:
    """Compiles the portableRT C++ API (compat headers + B200Backend) into a test
    program linked against libprt_b200.so."""
    lib = build_library()
    srcs = [os.path.join(ROOT, "tests", "cpp", "b200_api_test.cpp"),
            os.path.join(PKG, "src", "intersect_b200.cpp"),
            os.path.join(PKG, "compat", "backend.cpp")]
    deps = srcs + [lib, os.path.join(ROOT, "include", "portableRT", "intersect_b200.hpp")]
    deps += [os.path.join(PKG, "compat", "portableRT", f)
             for f in os.listdir(os.path.join(PKG, "compat", "portableRT"))]
    if _stale(CPP_TEST, deps):
        cxx = shutil.which(os.environ.get("CXX", "g++")) or "g++"
        cmd = [cxx, "-O2", "-std=c++17", "-Wall",
               f"-I{os.path.join(PKG, 'compat', 'portableRT')}",
               f"-I{os.path.join(PKG, 'compat')}", f"-I{os.path.join(ROOT, 'include')}"]
        cmd += srcs + ["-o", CPP_TEST, f"-L{OUT}", "-lprt_b200", f"-Wl,-rpath,{OUT}"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"C++ API test build failed:\n{r.stdout}\n{r.stderr}")
    if verbose:
        print(f"built {CPP_TEST}", file=sys.stderr)
    return CPP_TEST


if __name__ == "__main__":
    build_library(verbose=True)
    build_cpp_test(verbose=True)
