"""Build the GB300 engine (csrc/*.cu, csrc/*.cpp) into lf_dem_gb300/_lib/liblfdem_gb300.so.

nvcc compiles every translation unit for sm_103a only, in parallel, in-tree.
The physics kernels (lfg_physics.cu) are compiled with --fmad=false so that
pair geometry rounds exactly like LF_DEM's scalar C++ (contact states flip at
a reduced gap of exactly 0).
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "_lib")
LIB = os.path.join(LIBDIR, "liblfdem_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NO_FMAD = {"lfg_physics.cu"}


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", shutil.which("nvcc")):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources():
    return sorted(f for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _compile(src: str, verbose: bool) -> str:
    obj = os.path.join(BUILD, src + ".o")
    cmd = [_nvcc(), "-c", os.path.join(CSRC, src), "-o", obj, "-O3", "-std=c++17", "-lineinfo",
           "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall", *ARCH, "-I", os.path.join(HERE, "..", "include")]
    if src.endswith(".cu"):
        cmd += ["-Xptxas", "-O3"]
        if src in NO_FMAD:
            cmd += ["--fmad=false"]
        if verbose:
            cmd += ["-Xptxas", "-v"]
    out = subprocess.run(cmd, capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{out.stderr}")
    if verbose and out.stderr:
        sys.stderr.write(out.stderr)
    return obj


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    srcs = sources()
    newest_src = max(os.path.getmtime(os.path.join(CSRC, s)) for s in os.listdir(CSRC))
    newest_src = max(newest_src, os.path.getmtime(os.path.join(HERE, "..", "include", "lfdem_gb300.h")))
    if not force and os.path.exists(LIB) and os.path.getmtime(LIB) > newest_src:
        return LIB
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
    tmp = LIB + ".tmp"
    cmd = [_nvcc(), "-shared", "-o", tmp, *objs, *ARCH, "-lcudart"]
    out = subprocess.run(cmd, capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("link failed:\n" + out.stderr)
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
