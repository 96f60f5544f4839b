"""Build recipe of the native library ``nanopyx_gb300/_lib/libnanopyx_gb300.so``.

Every ``csrc/*.cu`` translation unit is compiled by ``nvcc`` for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``), in parallel, and linked into one
shared library with a static CUDA runtime.  The library exports the C ABI of
``include/nanopyx_gb300.h`` and nothing that depends on PyTorch.

Rebuilds are incremental: an object is recompiled when its source, any header
or the flags changed (content hash stamped next to the object).
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
INCLUDE = os.path.join(ROOT, "include")
OBJ = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "_lib")
LIB = os.path.join(LIBDIR, "libnanopyx_gb300.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC",
                     "-Xcompiler", "-O2", "-I", INCLUDE, "-I", CSRC]


def nvcc_path() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build nanopyx_gb300")


def _headers_digest() -> str:
    h = hashlib.sha256()
    for d in (CSRC, INCLUDE):
        for name in sorted(os.listdir(d)):
            if name.endswith((".h", ".cuh")):
                with open(os.path.join(d, name), "rb") as f:
                    h.update(name.encode() + f.read())
    return h.hexdigest()


def _sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def build(jobs: int | None = None, verbose: bool = False) -> str:
    """Compile (incrementally) and link the library; returns its path."""
    nvcc = nvcc_path()
    os.makedirs(OBJ, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    hdr = _headers_digest()
    flags_key = " ".join(NVCC_FLAGS)

    def compile_one(src):
        obj = os.path.join(OBJ, os.path.basename(src)[:-3] + ".o")
        with open(src, "rb") as f:
            key = hashlib.sha256(f.read() + hdr.encode() + flags_key.encode()).hexdigest()
        stamp = obj + ".key"
        if os.path.exists(obj) and os.path.exists(stamp) and open(stamp).read() == key:
            return obj, False
        cmd = [nvcc] + NVCC_FLAGS + ["-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {os.path.basename(src)}:\n{r.stderr[-4000:]}")
        if verbose and r.stderr:
            print(r.stderr)
        with open(stamp, "w") as f:
            f.write(key)
        return obj, True

    srcs = _sources()
    n = jobs or max(1, min(len(srcs), os.cpu_count() or 1))
    with cf.ThreadPoolExecutor(n) as ex:
        results = list(ex.map(compile_one, srcs))
    objs = [o for o, _ in results]
    relink = any(c for _, c in results) or not os.path.exists(LIB) or any(
        os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs)
    if relink:
        tmp = LIB + ".tmp"
        cmd = [nvcc] + ARCH + ["-shared", "-cudart", "static", "-o", tmp] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stderr[-4000:]}")
        os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
