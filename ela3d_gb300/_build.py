"""Build recipe: nvcc for the CUDA library, gcc for the oracle.

``build_library()`` compiles every translation unit under ``csrc/`` for
sm_103a in parallel and links ``_build/libela3d.so`` (in-tree, git-ignored).
``build_oracle()`` compiles the CPU restatement under ``oracle/`` and, when
the patched reference source is present (generated by oracle/make_ref.py),
the reference program itself.  Rebuilds only when a source is newer than the
output.
"""
from __future__ import annotations

import glob
import shutil
import os
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT = os.path.join(PKG, "_build")
LIB = os.path.join(OUT, "libela3d.so")
ORACLE_DIR = os.path.join(ROOT, "oracle")
ORACLE_OUT = os.path.join(ORACLE_DIR, "_build")
ORACLE_LIB = os.path.join(ORACLE_OUT, "libela3d_oracle.so")

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


def build_oracle() -> str:
    os.makedirs(ORACLE_OUT, exist_ok=True)
    srcs = [os.path.join(ORACLE_DIR, f) for f in ("ela3d_oracle.c", "ela3d_oracle_impl.h", "ela3d_oracle.h")]
    if _newer(srcs, ORACLE_LIB):
        subprocess.run(["gcc", "-O2", "-ffp-contract=off", "-shared", "-fPIC", srcs[0], "-o", ORACLE_LIB, "-lm"],
                       check=True)
    return ORACLE_LIB


def build_reference() -> list[str]:
    """Patched reference program (oracle/_ref); empty list when unavailable."""
    sys.path.insert(0, ORACLE_DIR)
    try:
        import make_ref  # type: ignore
    finally:
        sys.path.pop(0)
    ref_src = os.path.join(make_ref.DEFAULT_REF_DIR, make_ref.REF_NAME)
    if os.path.exists(ref_src):
        make_ref.generate(make_ref.DEFAULT_REF_DIR)
    outs, procs = [], []
    jobs = [(os.path.join(make_ref.OUT, f"ref_{v}.cpp"), os.path.join(make_ref.OUT, f"ref_{v}"),
             make_ref.compiler_cmd) for v in ("f32", "f64")]
    if shutil.which("nvcc"):   # the reference's FP32 GPU program, a timing baseline
        jobs.append((os.path.join(make_ref.OUT, "ref_gpu_f32.cu"), os.path.join(make_ref.OUT, "ref_gpu_f32"),
                     make_ref.gpu_compiler_cmd))
    for src, exe, cmd in jobs:
        if os.path.exists(src):
            if _newer([src, os.path.join(ORACLE_DIR, "ref_harness.h")], exe):
                procs.append((exe, subprocess.Popen(cmd(src, exe))))
            outs.append(exe)
    for exe, p in procs:
        if p.wait() != 0:
            raise RuntimeError(f"building {exe} failed")
    return outs


if __name__ == "__main__":
    print(build_library(verbose=True))
    print(build_oracle())
    print(build_reference())
