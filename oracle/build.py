"""Build recipe for the checkers.  TEST INFRASTRUCTURE.

``build_oracle()`` compiles the C restatement (ela3d_oracle.c) into
``oracle/_build/libela3d_oracle.so``.  ``build_reference()`` writes the
patched reference program (make_ref.py) when the reference checkout is
readable, and compiles whatever patched sources exist under ``oracle/_ref/``
(on a machine without the checkout, the ones generated earlier travel with
the tree).  Both rebuild only when a source is newer than the output.
Called by ``__graft_entry__.build()``; the library package never imports
this file.
"""
from __future__ import annotations

import os
import shutil
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
ORACLE_OUT = os.path.join(HERE, "_build")
ORACLE_LIB = os.path.join(ORACLE_OUT, "libela3d_oracle.so")


def _newer(srcs: list[str], out: str) -> bool:
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(s) > t for s in srcs)


def build_oracle() -> str:
    os.makedirs(ORACLE_OUT, exist_ok=True)
    srcs = [os.path.join(HERE, f) for f in ("ela3d_oracle.c", "ela3d_oracle_impl.h", "ela3d_oracle.h")]
    if _newer(srcs, ORACLE_LIB):
        tmp = ORACLE_LIB + f".{os.getpid()}.tmp"
        subprocess.run(["gcc", "-O2", "-ffp-contract=off", "-shared", "-fPIC", srcs[0], "-o", tmp, "-lm"],
                       check=True)
        os.replace(tmp, ORACLE_LIB)
    return ORACLE_LIB


def build_reference() -> list[str]:
    """Patched reference program (oracle/_ref); empty list when unavailable."""
    from . import make_ref

    ref_dir = make_ref.reference_dir()
    if ref_dir and os.path.exists(os.path.join(ref_dir, make_ref.REF_NAME)):
        make_ref.generate(ref_dir)
    outs, procs = [], []
    jobs = [(os.path.join(make_ref.OUT, f"ref_{v}.cpp"), os.path.join(make_ref.OUT, f"ref_{v}"),
             make_ref.compiler_cmd) for v in ("f32", "f64")]
    if shutil.which("nvcc"):   # the reference's GPU programs, timing baselines
        for name in ("ref_gpu_f32", "ref_gpu_f64"):
            jobs.append((os.path.join(make_ref.OUT, name + ".cu"), os.path.join(make_ref.OUT, name),
                         make_ref.gpu_compiler_cmd))
    for src, exe, cmd in jobs:
        if os.path.exists(src):
            if _newer([src, os.path.join(HERE, "ref_harness.h")], exe):
                procs.append((exe, subprocess.Popen(cmd(src, exe))))
            outs.append(exe)
    for exe, p in procs:
        if p.wait() != 0:
            raise RuntimeError(f"building {exe} failed")
    return outs


if __name__ == "__main__":
    print(build_oracle())
    print(build_reference())
