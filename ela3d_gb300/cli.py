"""Command line: run one shot on the GPU from a parameter file and write the
reference program's output files.

    python -m ela3d_gb300 run params.txt [--outdir DIR] [--fp64]

params.txt holds "key value" lines with the reference's parameter names
(the locals of seismicCPML_3d_isotropic_simpelmodel.cpp:19-78): nx ny nz,
dx (one spacing, the reference's DELTAX), dt, nstep, sampgat, it_output,
ngatx ngaty (the receiver text layout), npml, npower, k_max, alpha_max,
rcoef, vpml, f0, t0, factor, angle, "src i j k" (0-based), src_kind
(0 force, 1 explosive), stf (0 Ricker, 1 Gaussian derivative, 2 Gaussian),
"w wx wy wz", clean (0/1 profile variant), model PREFIX (PREFIXcp.bin,
PREFIXcs.bin, PREFIXrh.bin; without it the reference's constant medium
cp 3300, cs 3300/1.732, rho 3000), and optional "rec i j k" lines (extra
receivers written to seis.npy as [nrec, 3, nsamp]).

Outputs (in --outdir): rechorvx.txt rechorvy.txt rechorvz.txt when ngatx
and ngaty are given (:625-671), vz%05i.bin vy%05i.bin vx%05i.bin every
it_output steps (:673-725), recsrcx.txt recsrcy.txt recsrcz.txt (the
source-point trace of elatic_3d_unified_cuda_memory.cu:1202-1223), seis.npy
for the rec lines.
"""
from __future__ import annotations

import argparse
import os
import sys

import numpy as np

from . import refio
from ._abi import Plan
from .params import FP32, FP64, ShotParams


# the keys of a parameter file (the C++ runner, ela3d_run.cpp, reads the same)
KEYS = ("nx", "ny", "nz", "dx", "dt", "nstep", "sampgat", "it_output", "ngatx", "ngaty", "npml", "npower", "k_max",
        "alpha_max", "rcoef", "vpml", "f0", "t0", "factor", "angle", "src", "src_kind", "stf", "w", "clean",
        "energy_every", "model", "rec")


def parse_params(path: str) -> tuple[ShotParams, dict]:
    kv = {}
    rec = []
    for line in open(path):
        parts = line.split()
        if not parts or parts[0].startswith("#"):
            continue
        k, v = parts[0], parts[1:]
        if k not in KEYS:
            raise ValueError(f"{path}: unknown key {k!r} (known: {' '.join(KEYS)})")
        if k == "rec":
            rec.append([int(x) for x in v[:3]])
        else:
            kv[k] = v
    g = lambda k, d, t=float: t(kv[k][0]) if k in kv else d  # noqa: E731
    dx = g("dx", 10.0)
    p = ShotParams(nx=g("nx", 32, int), ny=g("ny", 32, int), nz=g("nz", 32, int), nstep=g("nstep", 10, int),
                   dx=dx, dy=dx, dz=dx, dt=g("dt", 1e-3), npml=g("npml", 10, int), pml_mode=g("clean", 0, int),
                   npower=g("npower", 2.0), k_max=g("k_max", 1.0), alpha_max=g("alpha_max", -1.0),
                   rcoef=g("rcoef", 1e-3), vpml=g("vpml", 3000.0), f0=g("f0", 7.0), t0=g("t0", 1.2 / 7.0),
                   factor=g("factor", 1e7), stf=g("stf", 0, int), src_kind=g("src_kind", 0, int),
                   src=tuple(int(x) for x in kv.get("src", ["16", "16", "16"])), sampgat=g("sampgat", 1, int),
                   src_w=tuple(float(x) for x in kv.get("w", ["0", "0", "1"])), angle_force=g("angle", 0.0),
                   rec=np.array(rec, np.int32).reshape(-1, 3), it_output=g("it_output", 0, int),
                   energy_every=g("energy_every", 0, int))
    extra = {"ngatx": g("ngatx", 0, int), "ngaty": g("ngaty", 0, int),
             "model": kv["model"][0] if "model" in kv else None}
    return p, extra


def run(params_path: str, outdir: str, fp64: bool = False) -> dict:
    p, extra = parse_params(params_path)
    p = p.with_(precision=FP64 if fp64 else FP32)
    if extra["model"]:
        cp, cs, rho = refio.read_model(extra["model"], p.nx, p.ny, p.nz)
    else:
        shape = (p.nz, p.ny, p.nx)
        cp = np.full(shape, 3300.0, np.float32)
        cs = np.full(shape, np.float32(3300 / 1.732), np.float32)
        rho = np.full(shape, 3000.0, np.float32)
    user_rec = p.rec_array()
    slots = None
    if extra["ngatx"] > 0 and extra["ngaty"] > 0:
        cells, slots = refio.gather_layout(p.nx, p.ny, p.npml, extra["ngatx"], extra["ngaty"], int(p.src[2]))
        rec = np.concatenate([cells, user_rec]) if user_rec.size else cells
    else:
        cells = np.zeros((0, 3), np.int32)
        rec = user_rec
    os.makedirs(outdir, exist_ok=True)
    dt = np.float64 if fp64 else np.float32
    with Plan(p.with_(rec=rec), cp, cs, rho) as plan:
        done = 0
        chunk = p.it_output if p.it_output > 0 else p.nstep
        while done < p.nstep:
            n = min(chunk, p.nstep - done)
            plan.run(n)
            done += n
            if p.it_output > 0 and done % p.it_output == 0:
                fields = [plan.field(c, fp64=fp64) for c in range(3)]
                refio.write_snapshots(outdir, done, fields[0], fields[1], fields[2], dtype=dt)
        seis = plan.seismograms()
        trace = plan.source_trace(fp64=fp64)
    written = {"recsrc": refio.write_recsrc(outdir, trace)}
    if slots is not None:
        written["rechor"] = refio.write_rechor(outdir, seis[: len(cells)], slots)
    if user_rec.size:
        np.save(os.path.join(outdir, "seis.npy"), seis[len(cells):])
        written["seis"] = os.path.join(outdir, "seis.npy")
    return written


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(prog="python -m ela3d_gb300")
    sub = ap.add_subparsers(dest="cmd", required=True)
    r = sub.add_parser("run", help="run one shot from a parameter file")
    r.add_argument("params")
    r.add_argument("--outdir", default=".")
    r.add_argument("--fp64", action="store_true")
    a = ap.parse_args(argv)
    if a.cmd == "run":
        print(run(a.params, a.outdir, a.fp64))
    return 0


if __name__ == "__main__":
    sys.exit(main())
