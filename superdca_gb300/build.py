"""Build the engine's shared library in-tree: superdca_gb300/libsuperdca_gb300.so.

nvcc compiles each translation unit for sm_103a (GB300) in parallel, then
links them into one shared library that exports the C ABI declared in
include/superdca_gb300.h.  No CPU fallback is built.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libsuperdca_gb300.so")
CLI = os.path.join(HERE, "superdca-gb300")
CLI_SOURCES = [os.path.join(HERE, "cli", "superdca_gb300_cli.cpp")]

SOURCES = ["engine.cu", "kernels_gather.cu", "kernels_solver.cu", "kernels_tc.cu", "kernels_weights.cu",
           "noalloc.cu", "mlp.cu", "warmstart.cu", "kernels_dual.cu", "autotune.cpp"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O3", "--expt-relaxed-constexpr",
         "-I" + os.path.join(ROOT, "include")]


def nvcc() -> str:
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found")
    return path


def _compile(src: str, extra: list[str]) -> str:
    obj = os.path.join(BUILD, os.path.splitext(src)[0] + ".o")
    cmd = [nvcc(), *ARCH, *FLAGS, *extra, "-c", os.path.join(CSRC, src), "-o", obj]
    out = subprocess.run(cmd, capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError(f"nvcc failed for {src}:\n{' '.join(cmd)}\n{out.stdout}{out.stderr}")
    return obj


def build(verbose: bool = False, extra: list[str] | None = None) -> str:
    extra = list(extra or [])
    os.makedirs(BUILD, exist_ok=True)
    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(lambda s: _compile(s, extra), SOURCES))
    tmp = LIB + ".tmp"
    cmd = [nvcc(), *ARCH, "-shared", "-o", tmp, *objs, "-lcudart"]
    out = subprocess.run(cmd, capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError(f"link failed:\n{' '.join(cmd)}\n{out.stdout}{out.stderr}")
    os.replace(tmp, LIB)
    build_cli()
    if verbose:
        print("built", LIB, "and", CLI)
    return LIB


def build_cli() -> str:
    """The command-line front end: host C++ linked against the engine library."""
    cxx = shutil.which("g++") or "g++"
    tmp = CLI + ".tmp"
    cmd = [cxx, "-O2", "-std=c++17", "-Wall", "-I" + os.path.join(ROOT, "include"), *CLI_SOURCES,
           "-L" + HERE, "-lsuperdca_gb300", "-Wl,-rpath,$ORIGIN", "-pthread", "-o", tmp]
    out = subprocess.run(cmd, capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError(f"CLI build failed:\n{' '.join(cmd)}\n{out.stdout}{out.stderr}")
    os.replace(tmp, CLI)
    return CLI


if __name__ == "__main__":
    build(verbose=True, extra=sys.argv[1:])
