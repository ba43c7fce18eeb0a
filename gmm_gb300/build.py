"""Builds the sm_103a shared library ``gmm_gb300/_build/libgmm_gb300.so`` with nvcc.

Each CUDA translation unit compiles in parallel with
``-gencode arch=compute_103a,code=sm_103a -O3 -lineinfo``; the objects link into one shared
library with the C ABI of include/gmm_gb300.h. No torch extension machinery is involved: the
library is plain C ABI, loaded with ctypes.

The C++ host layer (``host/gmm_host.cpp``: the GMModel / estimator / ModelAdapt classes) and the
two command lines ``gmm_adapt`` and ``gmm_loglike`` compile with g++ against that library
(run path ``$ORIGIN``) into the same folder.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
HOST = os.path.join(HERE, "host")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(OUT_DIR, "libgmm_gb300.so")
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
CXX = os.environ.get("CXX", "g++")
CLIS = {"gmm_adapt": "gmm_adapt_main.cpp", "gmm_loglike": "gmm_loglike_main.cpp"}
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
         "-I" + os.path.join(ROOT, "include"), "-I" + CSRC]


def _compile(src: str, extra: list[str]) -> str:
    obj = os.path.join(OUT_DIR, os.path.basename(src) + ".o")
    deps = [src] + glob.glob(os.path.join(CSRC, "*.cuh")) + [os.path.join(ROOT, "include", "gmm_gb300.h")]
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(d) for d in deps):
        return obj
    cmd = [NVCC, *ARCH, *FLAGS, *extra, "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose: bool = False, extra: list[str] | None = None) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    extra = list(extra or [])
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), srcs))
    if not os.path.exists(LIB) or os.path.getmtime(LIB) < max(os.path.getmtime(o) for o in objs):
        cmd = [NVCC, *ARCH, "-shared", "-o", LIB, *objs]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    _build_host()
    if verbose:
        print(LIB)
    return LIB


def _build_host() -> None:
    """g++ builds of the host layer and the command lines, linked against the library."""
    hdrs = glob.glob(os.path.join(HOST, "*.hpp")) + [os.path.join(ROOT, "include", "gmm_gb300.h"), __file__]
    host_src = os.path.join(HOST, "gmm_host.cpp")
    flags = ["-O2", "-std=c++17", "-Wall", "-I" + os.path.join(ROOT, "include"), "-I" + HOST]

    def one(name: str) -> None:
        out = os.path.join(OUT_DIR, name)
        main = os.path.join(HOST, CLIS[name])
        deps = [main, host_src, LIB] + hdrs
        if os.path.exists(out) and os.path.getmtime(out) >= max(os.path.getmtime(d) for d in deps):
            return
        cmd = [CXX, *flags, main, host_src, "-o", out, "-L" + OUT_DIR, "-lgmm_gb300",
               "-Wl,-rpath,$ORIGIN"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"g++ failed for {name}:\n{r.stdout}\n{r.stderr}")

    with cf.ThreadPoolExecutor(max_workers=len(CLIS)) as ex:
        list(ex.map(one, CLIS))


if __name__ == "__main__":
    build(verbose=True, extra=sys.argv[1:])
