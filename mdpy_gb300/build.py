"""Build libmdg.so (in-tree) from mdpy_gb300/csrc with nvcc for sm_103a.

Each translation unit is compiled in parallel, then linked against cudart
and cuFFT.  No cmake, no torch extension machinery: the product is a plain
C-ABI shared library that ctypes (or any FFI) loads.

    python -m mdpy_gb300.build            # build if sources changed
    python -m mdpy_gb300.build --force    # rebuild
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")
OBJ = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libmdg.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-ftz=true", "-Xcompiler", "-fPIC,-fvisibility=hidden",
              "-I" + INCLUDE, "--expt-relaxed-constexpr"]


def _nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found; libmdg needs the CUDA toolkit to build")
    return cand


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith(".cu"))


def _digest():
    h = hashlib.sha256()
    files = sources() + [os.path.join(CSRC, f) for f in sorted(os.listdir(CSRC))
                         if f.endswith((".cuh", ".h"))] + [os.path.join(INCLUDE, "mdg.h")]
    for p in files:
        with open(p, "rb") as fh:
            h.update(p.encode() + b"\0" + fh.read())
    h.update(" ".join(ARCH + NVCC_FLAGS).encode())
    return h.hexdigest()


def build(force=False, verbose=False, extra_flags=()):
    """Compile every .cu under csrc and link libmdg.so; returns its path."""
    stamp = os.path.join(OBJ, "stamp")
    digest = _digest() + "|" + " ".join(extra_flags)
    if not force and os.path.exists(LIB) and os.path.exists(stamp):
        with open(stamp) as fh:
            if fh.read() == digest:
                return LIB
    os.makedirs(OBJ, exist_ok=True)
    nvcc = _nvcc()

    def compile_one(src):
        obj = os.path.join(OBJ, os.path.basename(src)[:-3] + ".o")
        cmd = [nvcc] + ARCH + NVCC_FLAGS + list(extra_flags) + ["-c", src, "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed on %s:\n%s%s" % (src, r.stdout, r.stderr))
        if verbose and (r.stdout or r.stderr):
            sys.stderr.write(r.stdout + r.stderr)
        return obj

    srcs = sources()
    with cf.ThreadPoolExecutor(max_workers=min(len(srcs), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB + ".%d.tmp" % os.getpid()
    cmd = [nvcc] + ARCH + ["-shared", "-o", tmp] + objs + ["-lcufft", "-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    with open(stamp, "w") as fh:
        fh.write(digest)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True,
                extra_flags=["-Xptxas", "-v"] if "--ptxas-v" in sys.argv else []))
