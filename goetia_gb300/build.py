"""Builds libgoetia_gb300.so in-tree with nvcc for sm_103a.

Each translation unit compiles in its own process (in parallel), then one
link step produces ``goetia_gb300/libgoetia_gb300.so``.  Objects go to
``goetia_gb300/_build/``.  A unit is rebuilt when it or any header is newer
than its object.
"""
import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libgoetia_gb300.so")
INCLUDE = os.path.join(ROOT, "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
              "-I", CSRC, "-I", INCLUDE] + ARCH


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cc")))


def _headers_mtime():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return max(os.path.getmtime(h) for h in hs)


def _compile(src, verbose):
    obj = os.path.join(BUILD, os.path.basename(src) + ".o")
    newest = max(os.path.getmtime(src), _headers_mtime())
    if os.path.exists(obj) and os.path.getmtime(obj) >= newest:
        return obj
    cmd = [_nvcc(), "-c", src, "-o", obj + ".tmp"] + NVCC_FLAGS
    if src.endswith(".cc"):
        cmd = [_nvcc(), "-x", "cu", "-c", src, "-o", obj + ".tmp"] + NVCC_FLAGS
    if verbose:
        print(" ".join(cmd), flush=True)
    subprocess.check_call(cmd)
    os.replace(obj + ".tmp", obj)
    return obj


WORKLOAD_SRC = os.path.join(HERE, "workload", "gen_reads.cc")
WORKLOAD_LIB = os.path.join(HERE, "libgoetia_workload.so")


def build_workload(verbose=False):
    """The host-only synthetic read generator the benchmark and tests use
    (g++, no CUDA): goetia_gb300/libgoetia_workload.so."""
    if os.path.exists(WORKLOAD_LIB) and os.path.getmtime(WORKLOAD_LIB) >= os.path.getmtime(WORKLOAD_SRC):
        return WORKLOAD_LIB
    cmd = [os.environ.get("CXX", "g++"), "-std=c++17", "-O3", "-fPIC", "-shared", "-pthread",
           "-o", WORKLOAD_LIB + ".tmp", WORKLOAD_SRC]
    if verbose:
        print(" ".join(cmd), flush=True)
    subprocess.check_call(cmd)
    os.replace(WORKLOAD_LIB + ".tmp", WORKLOAD_LIB)
    return WORKLOAD_LIB


def build(verbose=False, jobs=None):
    """Compile every CUDA/C++ unit for sm_103a and link the shared library
    (and the host-only workload generator)."""
    build_workload(verbose)
    os.makedirs(BUILD, exist_ok=True)
    srcs = sources()
    with ThreadPoolExecutor(max_workers=jobs or min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
    if os.path.exists(LIB) and os.path.getmtime(LIB) >= max(os.path.getmtime(o) for o in objs):
        return LIB
    cmd = [_nvcc(), "-shared", "-o", LIB + ".tmp"] + objs + ARCH + ["-lcudart"]
    if verbose:
        print(" ".join(cmd), flush=True)
    subprocess.check_call(cmd)
    os.replace(LIB + ".tmp", LIB)
    return LIB


if __name__ == "__main__":
    build(verbose="-v" in sys.argv)
    print(LIB)
