"""Build libtentaco_gb300.so (and the tensor-eval-gpu driver) in-tree for sm_103a.

Every translation unit under csrc/ is compiled in parallel: CUDA sources with
``nvcc -gencode arch=compute_103a,code=sm_103a``, host C++ with g++.  Objects
are cached under _build/ by a hash of the source and every header it can see,
so an unchanged tree relinks in seconds.  Output: tentaco_gb300/libtentaco_gb300.so
and tentaco_gb300/bin/tensor-eval-gpu.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import hashlib
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
INCLUDE = os.path.join(ROOT, "include")
LIB = os.path.join(PKG, "libtentaco_gb300.so")
BIN = os.path.join(PKG, "bin")
CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "--expt-relaxed-constexpr",
                     "-Xcompiler", "-fPIC,-fopenmp,-fvisibility=hidden", "-I" + INCLUDE]
CXX_FLAGS = ["-O3", "-std=c++17", "-fPIC", "-fopenmp", "-fvisibility=hidden", "-Wall",
             "-Wno-unused-function", "-I" + INCLUDE, "-I" + os.path.join(CUDA_HOME, "include")]


def _headers() -> bytes:
    h = hashlib.sha1()
    for pat in ("*.h", "*.cuh", "*.def"):
        for f in sorted(glob.glob(os.path.join(CSRC, pat)) + glob.glob(os.path.join(INCLUDE, "tentaco", pat))):
            with open(f, "rb") as fh:
                h.update(f.encode() + fh.read())
    return h.digest()


def _obj(src: str, hdr: bytes, flags: list) -> str:
    h = hashlib.sha1(hdr)
    with open(src, "rb") as fh:
        h.update(fh.read())
    h.update(" ".join(flags).encode())
    base = os.path.basename(src).replace(".", "_")
    return os.path.join(BUILD, f"{base}.{h.hexdigest()[:12]}.o")


def _compile(src: str, obj: str, verbose: bool) -> str:
    if os.path.exists(obj):
        return obj
    if src.endswith(".cu"):
        cmd = [NVCC] + NVCC_FLAGS + ["-c", src, "-o", obj + ".tmp"]
    else:
        cmd = ["g++"] + CXX_FLAGS + ["-c", src, "-o", obj + ".tmp"]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"compile failed: {src}\n{r.stdout}\n{r.stderr}")
    os.replace(obj + ".tmp", obj)
    return obj


def build(verbose: bool = False, jobs: int | None = None) -> str:
    """Compile every CUDA/C++ source and link the shared library; returns its path."""
    if not os.path.exists(NVCC):
        raise RuntimeError(f"nvcc not found at {NVCC}")
    os.makedirs(BUILD, exist_ok=True)
    hdr = _headers()
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))
    # the walk-kernel units take longest: start them first
    srcs.sort(key=lambda f: 0 if os.path.basename(f).startswith("tt_walk_o") else 1)
    jobs = jobs or max(2, os.cpu_count() or 2)
    with cf.ThreadPoolExecutor(jobs) as ex:
        futs = [ex.submit(_compile, s, _obj(s, hdr, NVCC_FLAGS if s.endswith(".cu") else CXX_FLAGS), verbose)
                for s in srcs]
        objs = [f.result() for f in futs]
    for stale in glob.glob(os.path.join(BUILD, "*.o")):
        if stale not in objs:
            os.remove(stale)
    tmp = LIB + ".tmp"
    cmd = [NVCC] + ARCH + ["-shared", "-o", tmp] + objs + ["-Xcompiler", "-fopenmp", "-lgomp", "-ldl"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    _build_driver(verbose)
    return LIB


def _build_driver(verbose: bool) -> None:
    src = os.path.join(PKG, "driver", "tensor_main.cpp")
    if not os.path.exists(src):
        return
    os.makedirs(BIN, exist_ok=True)
    out = os.path.join(BIN, "tensor-eval-gpu")
    cmd = ["g++", "-O2", "-std=c++17", "-I" + INCLUDE, src, "-o", out + ".tmp",
           "-L" + PKG, "-ltentaco_gb300", "-Wl,-rpath,$ORIGIN/.."]
    if verbose:
        print(" ".join(cmd), flush=True)
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"driver build failed\n{r.stdout}\n{r.stderr}")
    os.replace(out + ".tmp", out)


def clean() -> None:
    shutil.rmtree(BUILD, ignore_errors=True)


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
