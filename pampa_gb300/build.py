"""Build libpampa_gb300.so in-tree: host C++ with g++, CUDA with nvcc for sm_103a.

Translation units compile in parallel; objects go to pampa_gb300/_build/ and the shared
library to pampa_gb300/libpampa_gb300.so.  Nothing is installed outside the package.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import platform
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
# objects are kept per machine architecture so an x86 build tree never links on aarch64
BUILD = os.path.join(PKG, "_build", platform.machine())
LIB = os.path.join(PKG, "libpampa_gb300.so")
INCLUDE = os.path.join(ROOT, "include")

NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
CXX = os.environ.get("CXX", "g++")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CUDA_HOME = os.path.dirname(os.path.dirname(NVCC))


def _sources():
    host = sorted(os.path.join(CSRC, "host", f) for f in os.listdir(os.path.join(CSRC, "host"))
                  if f.endswith(".cpp"))
    gpu = sorted(os.path.join(CSRC, "gpu", f) for f in os.listdir(os.path.join(CSRC, "gpu"))
                 if f.endswith(".cu"))
    return host, gpu


def _compile(src: str) -> str:
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    deps = [src] + [os.path.join(d, f) for d in (os.path.join(CSRC, "host"), os.path.join(CSRC, "gpu"), INCLUDE)
                    for f in os.listdir(d) if f.endswith((".hpp", ".cuh", ".h"))]
    if os.path.exists(obj) and os.path.getmtime(obj) >= max(os.path.getmtime(p) for p in deps):
        return obj
    if src.endswith(".cu"):
        cmd = [NVCC, *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
               "-Xptxas", "-O3", "-I", INCLUDE, "-I", os.path.join(CSRC, "gpu"), "-c", src, "-o", obj]
    else:
        cmd = [CXX, "-O2", "-std=c++17", "-fPIC", "-Wall", "-I", INCLUDE, "-I", os.path.join(CSRC, "host"),
               "-I", os.path.join(CUDA_HOME, "include"), "-c", src, "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    return obj


def build(verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    host, gpu = _sources()
    srcs = gpu + host
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(_compile, srcs))
    stamp = os.path.join(BUILD, "lib.stamp")
    if (os.path.exists(LIB) and os.path.exists(stamp)
            and os.path.getmtime(stamp) >= max(os.path.getmtime(o) for o in objs)):
        return LIB
    cmd = [NVCC, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed: {' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
    with open(stamp, "w") as fh:
        fh.write(platform.machine() + "\n")
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
