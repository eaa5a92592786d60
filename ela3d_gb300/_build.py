"""Build recipe for the CUDA library and its command-line runner.

``build_library()`` compiles every CUDA translation unit under ``csrc/`` for
sm_103a in parallel and links ``_build/libela3d.so`` (in-tree, git-ignored).
``build_runner()`` compiles the C++ runner ``csrc/ela3d_run.cpp`` (host code
on the C ABI) into ``_build/ela3d_run``, linked to that library.  Both
rebuild only when a source is newer than the output.
"""
from __future__ import annotations

import glob
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_build")
LIB = os.path.join(OUT, "libela3d.so")

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVCC_FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-O2"]


def _nvcc() -> str:
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.isabs(cand) and os.path.exists(cand) or not os.path.isabs(cand)):
            return cand
    return "nvcc"


def _newer(srcs: list[str], out: str) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(s) > t for s in srcs)


def build_library(verbose: bool = False) -> str:
    os.makedirs(OUT, exist_ok=True)
    units = sorted(glob.glob(os.path.join(CSRC, "*.cu")))
    headers = sorted(glob.glob(os.path.join(CSRC, "*.cuh")) + glob.glob(os.path.join(CSRC, "*.h")) +
                     glob.glob(os.path.join(ROOT, "include", "*.h")))
    objs = []
    procs = []
    for u in units:
        obj = os.path.join(OUT, os.path.basename(u)[:-3] + ".o")
        objs.append(obj)
        if _newer([u] + headers, obj):
            cmd = [_nvcc()] + ARCH + NVCC_FLAGS + ["-I", os.path.join(ROOT, "include"), "-c", u, "-o", obj]
            if verbose:
                print(" ".join(cmd), file=sys.stderr)
            procs.append((u, subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)))
    failed = []
    for u, p in procs:
        out, _ = p.communicate()
        if p.returncode != 0:
            failed.append((u, out.decode(errors="replace")))
    if failed:
        raise RuntimeError("nvcc failed:\n" + "\n".join(f"{u}:\n{o}" for u, o in failed))
    if _newer(objs, LIB):
        cmd = [_nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
        subprocess.run(cmd, check=True)
    return LIB


RUNNER = os.path.join(OUT, "ela3d_run")


def build_runner() -> str:
    """The C++ runner; the library is found next to it at run time."""
    src = os.path.join(CSRC, "ela3d_run.cpp")
    header = os.path.join(ROOT, "include", "ela3d.h")
    if _newer([src, header, LIB], RUNNER):
        subprocess.run(["g++", "-O2", "-std=c++17", src, "-I", os.path.join(ROOT, "include"), "-L", OUT, "-lela3d",
                        "-Wl,-rpath,$ORIGIN", "-o", RUNNER], check=True)
    return RUNNER


if __name__ == "__main__":
    print(build_library(verbose=True))
    print(build_runner())
