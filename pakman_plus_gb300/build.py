"""Build the C-ABI shared library libpakman_gb300.so in-tree with nvcc (sm_103a).

    python -m pakman_plus_gb300.build            # build if sources changed
    python -m pakman_plus_gb300.build --force

Translation units are compiled in parallel, then linked with -shared.  The result
sits next to this file so the package loads it from the tree.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
ROOT = os.path.dirname(HERE)
INCLUDE = os.path.join(ROOT, "include")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libpakman_gb300.so")
HOST = os.path.join(HERE, "host")
BIN = os.path.join(HERE, "bin")
PKMER = os.path.join(BIN, "pkmer")
SOURCES = ["pk_kernels.cu", "pk_capi.cu", "pk_noalloc.cu", "pk_server.cu", "pk_batch.cu", "pk_ingest.cu",
           "pk_compact.cu", "pk_chunked.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libpakman_gb300.so")


def _deps():
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)]
    deps += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    deps.append(os.path.abspath(__file__))
    return deps


def up_to_date() -> bool:
    if not os.path.exists(LIB):
        return False
    t = os.path.getmtime(LIB)
    return all(os.path.getmtime(d) <= t for d in _deps())


def _compile(src: str) -> str:
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), *ARCH, "-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC",
           "-I", INCLUDE, "-c", os.path.join(CSRC, src), "-o", obj]
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{p.stdout}")
    return obj


def cxx() -> str:
    for cand in (os.environ.get("CXX"), shutil.which("g++")):
        if cand:
            return cand
    raise RuntimeError("g++ not found")


def build_pkmer(force: bool = False) -> str:
    """The pkmer command-line driver, linked against the in-tree library."""
    src = os.path.join(HOST, "pkmer.cpp")
    if (not force and os.path.exists(PKMER) and os.path.getmtime(PKMER) >= os.path.getmtime(src)
            and os.path.getmtime(PKMER) >= os.path.getmtime(LIB)):
        return PKMER
    os.makedirs(BIN, exist_ok=True)
    cmd = [cxx(), "-O2", "-std=c++17", "-I", INCLUDE, src, "-o", PKMER + ".tmp", "-L", HERE,
           "-lpakman_gb300", "-Wl,-rpath,$ORIGIN/.."]
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError(f"g++ failed on pkmer.cpp:\n{p.stdout}")
    os.replace(PKMER + ".tmp", PKMER)
    return PKMER


def build(force: bool = False, verbose: bool = False) -> str:
    if not force and up_to_date():
        build_pkmer()
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(len(SOURCES)) as ex:
        objs = list(ex.map(_compile, SOURCES))
    tmp = LIB + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-cudart", "static", "-o", tmp, *objs]
    p = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if p.returncode != 0:
        raise RuntimeError(f"link failed:\n{p.stdout}")
    os.replace(tmp, LIB)
    build_pkmer(force=True)
    if verbose:
        print(f"built {LIB} and {PKMER}")
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
