"""Build the GB300 engine (csrc/*.cu, csrc/*.cpp) into lf_dem_gb300/_lib/liblfdem_gb300.so.

nvcc compiles every translation unit for sm_103a only, in parallel, in-tree.
The physics kernels (lfg_physics.cu) are compiled with --fmad=false so that
pair geometry rounds exactly like LF_DEM's scalar C++ (contact states flip at
a reduced gap of exactly 0).
"""
from __future__ import annotations

import concurrent.futures as cf
import hashlib
import os
import platform
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIBDIR = os.path.join(HERE, "_lib")
LIB = os.path.join(LIBDIR, "liblfdem_gb300.so")
STAMP = os.path.join(LIBDIR, "liblfdem_gb300.fingerprint")
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


def _fingerprint(srcs) -> str:
    """Hash of everything the library is built from: the sources, the public
    header, this recipe, the compiler's version and the host architecture.  A
    library is reused only when its recorded fingerprint equals this one, so a
    copy built elsewhere (another machine, older sources) is always rebuilt."""
    h = hashlib.sha256()
    files = [os.path.join(CSRC, f) for f in sorted(os.listdir(CSRC))]
    files += [os.path.join(HERE, "..", "include", "lfdem_gb300.h"), os.path.abspath(__file__)]
    for f in files:
        h.update(os.path.basename(f).encode())
        with open(f, "rb") as fh:
            h.update(fh.read())
    ver = subprocess.run([_nvcc(), "--version"], capture_output=True, text=True).stdout
    h.update(ver.encode())
    h.update(platform.machine().encode())
    h.update(" ".join(ARCH).encode())
    return h.hexdigest()


def build(verbose: bool = False, force: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    srcs = sources()
    fp = _fingerprint(srcs)
    if not force and os.path.exists(LIB) and os.path.exists(STAMP):
        with open(STAMP) as f:
            if f.read().strip() == fp:
                return LIB
    with cf.ThreadPoolExecutor(max_workers=min(8, len(srcs))) as ex:
        objs = list(ex.map(lambda s: _compile(s, verbose), srcs))
    tmp = LIB + ".tmp"
    cmd = [_nvcc(), "-shared", "-o", tmp, *objs, *ARCH, "-lcudart"]
    out = subprocess.run(cmd, capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("link failed:\n" + out.stderr)
    os.replace(tmp, LIB)
    with open(STAMP, "w") as f:
        f.write(fp + "\n")
    sys.stderr.write(f"lf_dem_gb300: built {LIB} ({platform.machine()}, {len(srcs)} sources)\n")
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force="-f" in sys.argv))
