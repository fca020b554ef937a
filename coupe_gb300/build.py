"""Builds libcoupe_gpu.so (sm_103a) in-tree with nvcc, and the oracle.

The library is the product: the C ABI of include/coupe.h and
include/coupe_gpu.h over the CUDA engine in csrc/.  Translation units compile
in parallel; objects go to coupe_gb300/_build/, the library to
coupe_gb300/libcoupe_gpu.so.  The CUDA runtime is linked statically so that
the library loads on a machine without a GPU (symbol checks) and needs no
LD_LIBRARY_PATH on the GPU host.
"""
import concurrent.futures
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libcoupe_gpu.so")
NVCC = os.environ.get("NVCC", "nvcc")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# -fmad=false: coupe's arithmetic has separate multiplies and adds (the Rib
# basis change, the imbalance test); FMA contraction would change results.
NVFLAGS = ARCH + [
    "-O3", "-lineinfo", "-std=c++17", "-fmad=false",
    "-Xcompiler", "-fPIC,-O2,-ffp-contract=off,-fno-fast-math",
    "-I" + os.path.join(ROOT, "include"),
]

SOURCES = ["engine_core.cu", "inst_ref32.cu", "inst_f64.cu", "inst_band.cu", "split_noalloc.cu", "imbalance.cu",
           "mesh.cu", "grid.cu", "multi_jagged.cu", "ffi.cpp"]


def _deps_mtime():
    latest = 0.0
    for d in (CSRC, os.path.join(ROOT, "include")):
        for f in os.listdir(d):
            latest = max(latest, os.path.getmtime(os.path.join(d, f)))
    return latest


def _compile(src):
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    if os.path.exists(obj) and os.path.getmtime(obj) >= _deps_mtime():
        return obj
    lang = ["-x", "cu"] if src.endswith(".cu") else ["-x", "c++"]
    cmd = [NVCC] + NVFLAGS + lang + ["-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed on %s:\n%s\n%s" % (src, " ".join(cmd), r.stderr))
    return obj


def build_library(verbose=False):
    os.makedirs(BUILD, exist_ok=True)
    with concurrent.futures.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(_compile, SOURCES))
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(o) for o in objs):
        return LIB
    cmd = [NVCC] + ARCH + ["-shared", "-cudart", "static", "-o", LIB] + objs + ["-lpthread", "-ldl", "-lrt"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
    if verbose:
        print("built", LIB)
    return LIB


def build_oracle(verbose=False):
    """Test infrastructure: the CPU oracle (oracle/Makefile)."""
    r = subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle")], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n%s\n%s" % (r.stdout, r.stderr))
    path = os.path.join(ROOT, "oracle", "build", "liboracle_rcb.so")
    if verbose:
        print("built", path)
    return path


if __name__ == "__main__":
    build_library(verbose=True)
    if "--oracle" in sys.argv:
        build_oracle(verbose=True)
