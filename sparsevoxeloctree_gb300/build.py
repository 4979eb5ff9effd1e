"""Build libsvo.so (the engine's CUDA kernels + C ABI) in-tree for sm_103a with nvcc.

The translation units listed in UNITS compile in parallel (seconds each) and link into
sparsevoxeloctree_gb300/libsvo.so; objects go to sparsevoxeloctree_gb300/_build/.  The march and texture
units are compiled with -fmad=false so their float arithmetic is rounded exactly like the reference's
scalar code.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libsvo.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall",
          "-I", os.path.join(ROOT, "include")]
UNITS = {
    "abi.cu": [],
    "voxelize.cu": [],
    "build.cu": [],
    "march.cu": ["-fmad=false", "-prec-div=true", "-prec-sqrt=true"],
    "noalloc.cu": [],
    "batch.cu": [],
    "serve.cu": [],
    "io.cu": [],
    "pt.cu": ["-Xcompiler", "-ffp-contract=off"],
    "texture.cu": ["-fmad=false", "-prec-div=true", "-prec-sqrt=true", "-Xcompiler", "-ffp-contract=off"],
}
HEADERS = ["common.cuh", "svo_internal.h"]


def nvcc() -> str:
    for c in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if c and os.path.exists(c):
            return c
    raise RuntimeError("nvcc not found: the engine needs the CUDA toolkit to build")


def _newest_input() -> float:
    paths = [os.path.join(CSRC, f) for f in list(UNITS) + HEADERS] + [os.path.join(ROOT, "include", "svo.h"),
                                                                      os.path.abspath(__file__)]
    return max(os.path.getmtime(p) for p in paths)


def needs_build() -> bool:
    return not os.path.exists(LIB) or os.path.getmtime(LIB) < _newest_input()


def build(force: bool = False, verbose: bool = False, extra: list[str] | None = None) -> str:
    if not force and not needs_build():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    extra = list(extra or [])
    if os.environ.get("SVO_CHECKED"):  # internal bounds checks (debug builds)
        extra.append("-DSVO_CHECKED")

    def compile_unit(name: str) -> str:
        obj = os.path.join(BUILD, name.replace(".cu", ".o"))
        cmd = [cc, *ARCH, *COMMON, *UNITS[name], *extra, "-c", os.path.join(CSRC, name), "-o", obj]
        if verbose:
            print(" ".join(cmd), flush=True)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {name}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr, flush=True)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(UNITS)) as ex:
        objs = list(ex.map(compile_unit, list(UNITS)))
    tmp = LIB + ".tmp"
    cmd = [cc, *ARCH, "-shared", "-o", tmp, *objs]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"nvcc link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv,
                extra=["-Xptxas", "-v"] if "--ptxas" in sys.argv else None))
