"""Build the sm_103a shared library librisa_gb300.so in-tree (risa_gb300/_build/).

Every .cu is compiled by nvcc for sm_103a only, host .cpp files by g++ with
FMA contraction off (the table builders must round each operation on its own),
in parallel, then linked with nvcc. Rebuilds only what changed.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
INCLUDE = os.path.join(ROOT, "include")
LIB = os.path.join(BUILD, "librisa_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def _nvcc() -> str:
    cand = os.path.join(os.environ.get("CUDA_HOME", "/usr/local/cuda"), "bin", "nvcc")
    return cand if os.path.exists(cand) else "nvcc"


def _headers():
    return (glob.glob(os.path.join(CSRC, "*.h")) + glob.glob(os.path.join(CSRC, "*.cuh")) +
            glob.glob(os.path.join(INCLUDE, "*.h")) + glob.glob(os.path.join(PKG, "cpp", "*", "*.h")))


def _stale(obj: str, src: str) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(f) > t for f in [src] + _headers())


def _compile(src: str, verbose: bool) -> str:
    base = os.path.splitext(os.path.basename(src))[0]
    obj = os.path.join(BUILD, base + (".cu.o" if src.endswith(".cu") else ".cpp.o"))
    if not _stale(obj, src):
        return obj
    tmp = obj + f".tmp{os.getpid()}"
    if src.endswith(".cu"):
        cmd = [_nvcc(), *ARCH, "-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
               "-Xcompiler", "-ffp-contract=off", "-I", INCLUDE, "-I", CSRC, "-c", src, "-o", tmp]
        if verbose:
            cmd.insert(1, "-Xptxas=-v")
    else:
        cmd = ["g++", "-O2", "-std=c++17", "-fPIC", "-ffp-contract=off", "-fno-fast-math",
               "-Wall", "-I", INCLUDE, "-I", CSRC, "-c", src, "-o", tmp]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"compile failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    if verbose and res.stderr:
        sys.stderr.write(res.stderr)
    os.replace(tmp, obj)
    return obj


def build(verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    srcs = sorted(glob.glob(os.path.join(CSRC, "*.cu")) + glob.glob(os.path.join(CSRC, "*.cpp")))
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(srcs), os.cpu_count() or 4))) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
    if not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        tmp = LIB + f".tmp{os.getpid()}"
        cmd = [_nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError(f"link failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
        os.replace(tmp, LIB)
    _build_pipeline()
    return LIB


PIPELINE = os.path.join(BUILD, "risa_gb_pipeline")


def _build_pipeline():
    """The configuration-driven pipeline example (C++ stages over the C ABI)."""
    src = os.path.join(PKG, "cpp", "examples", "risa_gb_pipeline.cpp")
    deps = [src, LIB] + glob.glob(os.path.join(PKG, "cpp", "*", "*.h"))
    if os.path.exists(PIPELINE) and all(os.path.getmtime(d) <= os.path.getmtime(PIPELINE) for d in deps):
        return PIPELINE
    tmp = PIPELINE + f".tmp{os.getpid()}"
    cuda = os.environ.get("CUDA_HOME", "/usr/local/cuda")
    cmd = ["g++", "-std=c++17", "-O2", "-pthread", "-I", INCLUDE, "-I", os.path.join(cuda, "include"), src,
           "-o", tmp, "-L", BUILD, "-lrisa_gb300", "-L", os.path.join(cuda, "lib64"), "-lcudart",
           "-Wl,-rpath,$ORIGIN", "-Wl,-rpath," + os.path.join(cuda, "lib64")]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError(f"pipeline build failed: {' '.join(cmd)}\n{res.stdout}\n{res.stderr}")
    os.replace(tmp, PIPELINE)
    return PIPELINE


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
