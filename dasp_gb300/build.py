"""Build the in-tree CUDA library ``dasp_gb300/_build/libshwfs.so``.

Every ``dasp_gb300/csrc/*.cu`` translation unit is compiled for sm_103a in
parallel (one ``-gencode``), then linked into one shared library with the
shared CUDA runtime.  ``wfs_refnoise.cu`` is compiled without FMA contraction
so the reference-stream noise rounds where the reference's C code rounds.
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
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(BUILD, "libshwfs.so")
INCLUDE = os.path.join(os.path.dirname(HERE), "include")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-I" + INCLUDE]
NO_FMA = {"wfs_refnoise.cu"}


def nvcc() -> str:
    cand = [os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"]
    for c in cand:
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found")


def _sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith(".cu"))


def _digest() -> str:
    h = hashlib.sha256()
    for f in sorted(os.listdir(CSRC)) + [os.path.join("..", "..", "include", "shwfs.h")]:
        p = os.path.join(CSRC, f)
        if os.path.isfile(p):
            h.update(f.encode())
            with open(p, "rb") as fh:
                h.update(fh.read())
    h.update(" ".join(ARCH + COMMON).encode())
    return h.hexdigest()


def _compile(src: str, obj: str) -> None:
    flags = list(COMMON) + (["-fmad=false"] if src in NO_FMA else [])
    cmd = [nvcc()] + ARCH + flags + ["-c", os.path.join(CSRC, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))


def build(force: bool = False, jobs: int | None = None, verbose: bool = False) -> str:
    """Compile and link libshwfs.so (skipped when sources are unchanged)."""
    os.makedirs(BUILD, exist_ok=True)
    stamp = os.path.join(BUILD, "libshwfs.sha256")
    digest = _digest()
    if not force and os.path.exists(LIB) and os.path.exists(stamp):
        with open(stamp) as fh:
            if fh.read().strip() == digest:
                return LIB
    srcs = _sources()
    objs = [os.path.join(BUILD, s[:-3] + ".o") for s in srcs]
    jobs = jobs or min(len(srcs), os.cpu_count() or 4)
    with cf.ThreadPoolExecutor(max_workers=jobs) as ex:
        futs = [ex.submit(_compile, s, o) for s, o in zip(srcs, objs)]
        for f in futs:
            f.result()
    tmp = LIB + ".%d.tmp" % os.getpid()
    cudalib = os.path.join(os.path.dirname(os.path.dirname(nvcc())), "lib64")
    cmd = [nvcc()] + ARCH + ["-shared", "-cudart", "shared", "-o", tmp] + objs + [
        "-Xlinker", "-rpath=" + cudalib]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s\n%s" % (r.stdout, r.stderr))
    os.replace(tmp, LIB)
    with open(stamp, "w") as fh:
        fh.write(digest)
    if verbose:
        print("built", LIB)
    return LIB


if __name__ == "__main__":
    build(force="--force" in sys.argv, verbose=True)
