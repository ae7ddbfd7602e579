"""Builds libgbturbo.so (the GPU path and its C-ABI) in-tree for sm_103a.

Every CUDA translation unit is compiled in parallel with nvcc, the host case reader with the same
compiler driver, and the objects are linked into ``libgbturbo.so`` next to this file. No cmake,
no torch extension machinery: a plain shared library with an ``extern "C"`` interface
(include/gbturbo.h).
"""
from __future__ import annotations

import concurrent.futures
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libgbturbo.so")
SOURCES = ["geometry.cu", "bc.cu", "resflux_cell.cu", "resflux_face.cu", "lusgs.cu", "mg.cu", "solver.cu",
           "capi.cu", "case_io.cpp", "noalloc.cu", "restart_io.cpp", "sa.cu", "warmstart.cu", "peak.cu", "face_tma.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _flags(extra_ptxas: bool) -> list:
    f = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2",
         "--expt-relaxed-constexpr", "-I", CSRC, "-I", os.path.join(HERE, "..", "include")] + ARCH
    if extra_ptxas:
        f += ["-Xptxas", "-v"]
    return f


def _compile(src: str, verbose: bool) -> str:
    obj = os.path.join(OUT_DIR, os.path.splitext(src)[0] + ".o")
    path = os.path.join(CSRC, src)
    deps = [path] + [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith((".cuh", ".hpp"))]
    if os.path.exists(obj) and all(os.path.getmtime(obj) >= os.path.getmtime(d) for d in deps):
        return obj
    cmd = [nvcc()] + _flags(verbose) + ["-c", path, "-o", obj]
    if src.endswith(".cpp"):
        cmd = [nvcc(), "-x", "c++"] + _flags(False)[:] + ["-Xcompiler", "-ffp-contract=off", "-c", path, "-o", obj]
        cmd = [c for c in cmd if c not in ARCH]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc failed on {src}:\n{r.stdout}\n{r.stderr}")
    if verbose and r.stderr:
        sys.stderr.write(r.stderr)
    return obj


def build(verbose: bool = False) -> str:
    os.makedirs(OUT_DIR, exist_ok=True)
    with concurrent.futures.ThreadPoolExecutor(max_workers=min(len(SOURCES), os.cpu_count() or 4)) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), SOURCES))
    if not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        cmd = [nvcc(), "-shared"] + ARCH + objs + ["-o", LIB, "-lcudart", "-lpthread"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv))
