"""Builds the CUDA library in-tree: tweakseq_gb300/lib/libtsq_gb300.so.

Every translation unit under csrc/ is compiled by nvcc for sm_103a only
(``-gencode arch=compute_103a,code=sm_103a``), in parallel, and linked into
one shared library with the C ABI of include/tweakseq_gb300.h.  Plain nvcc, no
cmake, no torch: the library does not depend on PyTorch.
"""
from __future__ import annotations

import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIBDIR = os.path.join(PKG, "lib")
LIB = os.path.join(LIBDIR, "libtsq_gb300.so")
CLI_SRC = os.path.join(PKG, "cli", "tsq_align.cpp")
CLI = os.path.join(LIBDIR, "tsq_align")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CFLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-Wall", "-I", os.path.join(ROOT, "include")]


def nvcc() -> str:
    for cand in (shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def sources() -> list[str]:
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cu", ".cpp")))


def _deps() -> list[str]:
    return [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(ROOT, "include", "tweakseq_gb300.h"),
                                                                 os.path.join(ROOT, "include", "tweakseq_gb300_tool.hpp")]


def up_to_date() -> bool:
    if not os.path.exists(LIB) or not os.path.exists(CLI):
        return False
    t = min(os.path.getmtime(LIB), os.path.getmtime(CLI))
    return all(os.path.getmtime(d) <= t for d in _deps() + [CLI_SRC])


def build_cli() -> str:
    """The tsq_align command-line tool (host C++ linked to the library)."""
    cxx = shutil.which("g++") or "g++"
    tmp = CLI + ".tmp"
    r = subprocess.run([cxx, "-O2", "-std=c++17", "-I", os.path.join(ROOT, "include"), CLI_SRC, "-o", tmp,
                        "-L", LIBDIR, "-ltsq_gb300", "-Wl,-rpath,$ORIGIN"], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"tsq_align build failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, CLI)
    return CLI


def build(force: bool = False, verbose: bool = False, jobs: int | None = None) -> str:
    if not force and up_to_date():
        return LIB
    os.makedirs(BUILD, exist_ok=True)
    os.makedirs(LIBDIR, exist_ok=True)
    cc = nvcc()
    srcs = sources()

    def compile_one(src: str) -> str:
        obj = os.path.join(BUILD, os.path.basename(src) + ".o")
        cmd = [cc, *ARCH, *CFLAGS, "-c", src, "-o", obj]
        if src.endswith(".cu"):
            cmd += ["-Xptxas", "-v"] if verbose else []
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed on {os.path.basename(src)}:\n{r.stdout}\n{r.stderr}")
        if verbose and r.stderr:
            sys.stderr.write(r.stderr)
        return obj

    with ThreadPoolExecutor(max_workers=jobs or min(16, os.cpu_count() or 4)) as ex:
        objs = list(ex.map(compile_one, srcs))
    tmp = LIB + ".tmp"
    r = subprocess.run([cc, *ARCH, "-shared", "-o", tmp, *objs], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB)
    build_cli()
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
