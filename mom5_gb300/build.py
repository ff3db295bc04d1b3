"""Build recipe for libmom5gpu.so (sm_103a) with nvcc, no CMake.

Each translation unit is compiled in parallel; the FP64 drop-in units are
built with ``--fmad=false`` so no product is fused into a multiply-add (the
reference's FP64 arithmetic rounds every product and sum), and host code with
``-ffp-contract=off`` for the same reason on aarch64 hosts, where GCC
contracts by default.  The precision-form unit keeps contraction on.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libmom5gpu.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]

# (source, exact FP64)
UNITS = [("capi.cu", True), ("k_fp64.cu", True), ("k_mixed.cu", False), ("k_batch.cu", False), ("k_batch64.cu", True),
         ("batch.cu", True), ("k_noalloc.cu", True), ("k_psom.cu", True), ("restart.cu", True), ("decomp.cu", True),
         ("k_mixed_tma.cu", False)]


def _nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libmom5gpu.so")


def _flags(exact: bool):
    f = ["-O3", "-std=c++17", "-lineinfo", *ARCH, "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
         "-I", os.path.join(HERE, "..", "include")]
    if exact:
        f += ["--fmad=false"]
    return f


def _sources():
    return [(s, e) for s, e in UNITS if os.path.exists(os.path.join(CSRC, s))]


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    """Compile the CUDA sources into mom5_gb300/libmom5gpu.so; returns its path."""
    os.makedirs(OUT_DIR, exist_ok=True)
    nvcc = _nvcc()
    headers = [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".h", ".cuh"))]
    headers.append(os.path.join(HERE, "..", "include", "mom5gpu.h"))
    objs = []
    jobs = []
    for src, exact in _sources():
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT_DIR, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, [s, *headers, __file__]):
            jobs.append([nvcc, *_flags(exact), "-c", s, "-o", o])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed:\n{' '.join(cmd)}\n{r.stdout}\n{r.stderr}")
        return r.stderr

    with ThreadPoolExecutor(max_workers=max(1, min(8, len(jobs)))) as ex:
        for msg in ex.map(run, jobs):
            if verbose and msg:
                print(msg, file=sys.stderr)
    if force or jobs or _stale(LIB, objs):
        run([nvcc, *ARCH, "-shared", "-o", LIB, *objs, "-lcudart"])
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
