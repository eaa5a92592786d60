"""Generates the golden fixtures in this directory from the reference program.

The reference repository has no tests, fixtures or known-answer vectors, so
the goldens are outputs of its own CPU program
(seismicCPML_3d_isotropic_simpelmodel.cpp), built unmodified except for the
parameter patch of oracle/make_ref.py, on small seeded inputs.  Each
``ref_<case>.npz`` holds the case parameters, the receiver traces
[nrec, 3, nsamp], per-field sums and sums of squares (float64), and two
slices of every final field (the x-y plane through the source depth and the
y-z plane through the source x).

Run from the repository root:  python tests/golden/make_golden.py
The full-size workloads (``ref_homogeneous_101_full.npz``,
``ref_anticline_256_full.npz``) take about half an hour of CPU and are made
separately:  python tests/golden/make_golden.py --full [name ...]
"""
from __future__ import annotations

import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from ela3d_gb300 import PML_CLEAN, SRC_EXPLOSIVE, STF_GAUSS_DERIV, ShotParams, configs, media  # noqa: E402


def small(shape=(24, 22, 28), **kw):
    nx, ny, nz = shape
    rec = np.array([[i, ny // 2, nz // 2 - 2] for i in range(2, nx - 1, 3)] + [[nx // 2, ny // 2, nz // 2]],
                   np.int32)
    p = ShotParams(nx=nx, ny=ny, nz=nz, nstep=80, dt=1e-3, npml=5, f0=25.0, t0=1.2 / 25.0,
                   src=(nx // 2, ny // 2, nz // 2), rec=rec, sampgat=2)
    p = p.with_(**kw)
    cp, cs, rho = media.anticline_layers(nx, ny, nz, depths=(nz * 0.25, nz * 0.5, nz * 0.75, nz * 2),
                                         amp=3.0, sigma=6.0, seed=3)
    return p, cp, cs, rho


def cases():
    out = {
        "ricker_vz_compat": small(),
        "ricker_vz_clean": small(pml_mode=PML_CLEAN),
        "explosive_gauss_deriv": small(stf=STF_GAUSS_DERIV, src_kind=SRC_EXPLOSIVE),
        "explosive_angle30": small(stf=STF_GAUSS_DERIV, src_kind=SRC_EXPLOSIVE, angle_force=30.0),
        "force_xyz": small(src_w=(1.0, 1.0, 1.0), shape=(26, 20, 24)),
    }
    # the reference program's own source settings (f0 = 35 Hz Gaussian
    # derivative, explosive, angle 0) on a 40^3 homogeneous cube
    n = 40
    rec = np.array([[i, 19, 11] for i in range(0, n, 4)], np.int32)
    p = ShotParams(nx=n, ny=n, nz=n, nstep=60, dt=1e-3, npml=10, f0=35.0, t0=1.2 / 35.0, factor=1e7,
                   stf=STF_GAUSS_DERIV, src_kind=SRC_EXPLOSIVE, src=(19, 19, 10), rec=rec, sampgat=2)
    out["reference_settings_40"] = (p,) + media.homogeneous(n, n, n, 3300.0, 3300.0 / 1.732, 3000.0)
    # the first 100 steps of the 101^3 homogeneous cube workload
    p, cp, cs, rho = configs.homogeneous_101(nstep=100)
    out["homogeneous_101_first100"] = (p, cp, cs, rho)
    return out


def slice_stride(p) -> int:
    """Slices of grids wider than 64 cells keep every third cell."""
    return 3 if max(p.nx, p.ny, p.nz) > 64 else 1


def summarize(p, fields):
    sx, sz = int(p.src[0]), int(p.src[2])
    s = slice_stride(p)
    return {
        "sum": fields.astype(np.float64).sum(axis=(1, 2, 3)),
        "sumsq": (fields.astype(np.float64) ** 2).sum(axis=(1, 2, 3)),
        "slice_xy": fields[:, sz, ::s, ::s].copy(),
        "slice_yz": fields[:, ::s, ::s, sx].copy(),
    }


def params_json(p) -> str:
    d = {k: getattr(p, k) for k in p.__dataclass_fields__ if k != "rec"}
    d["src"] = [int(v) for v in p.src]
    d["src_w"] = [float(v) for v in p.src_w]
    d["rec"] = p.rec_array().tolist()
    return json.dumps(d)


def full_cases():
    """The two benchmark workloads at their full sizes: the 101^3 homogeneous
    cube for its 1000 steps, and the 256^3 anticline shot for its 2000 steps
    with its 201-receiver line (a quarter of an hour of CPU per precision)."""
    return {
        "homogeneous_101_full": configs.homogeneous_101(),
        "anticline_256_full": configs.anticline_256(),
    }


def main_full(names=None):
    """Runs the reference program on the full-size workloads, both precisions
    in parallel.  The float32 seismograms are kept whole; the float64 ones,
    which check the FP64 build, are kept for every fourth receiver of lines
    longer than 64 receivers (the file stays a few MB)."""
    from concurrent.futures import ThreadPoolExecutor

    import oracle

    if oracle.reference_binary(False) is None or oracle.reference_binary(True) is None:
        raise SystemExit("build the reference program first: python oracle/make_ref.py")
    todo = {k: v for k, v in full_cases().items() if names is None or k in names}

    def one(job):
        name, fp64 = job
        p, cp, cs, rho = todo[name]
        seis, fields, secs, _ = oracle.run_reference(p, cp, cs, rho, fp64=fp64)
        return name, fp64, seis, summarize(p, fields), secs

    jobs = [(n, f) for n in todo for f in (False, True)]
    results = {}
    with ThreadPoolExecutor(len(jobs)) as ex:
        for name, fp64, seis, summ, secs in ex.map(one, jobs):
            results[(name, fp64)] = (seis, summ)
            print(name, "f64" if fp64 else "f32", f"{secs:.0f} s", flush=True)
    for name, (p, cp, cs, rho) in todo.items():
        out = {"params": np.array(params_json(p))}
        for fp64 in (False, True):
            seis, summ = results[(name, fp64)]
            tag = "f64" if fp64 else "f32"
            if fp64 and seis.shape[0] > 64:
                out["rec_every_f64"] = np.array(4)
                seis = seis[::4]
            out[f"seis_{tag}"] = seis
            for k, v in summ.items():
                out[f"{k}_{tag}"] = v
        np.savez_compressed(os.path.join(HERE, f"ref_{name}.npz"), **out)
        print(name, {k: v.shape for k, v in out.items()})


def main():
    import oracle

    if "--full" in sys.argv:
        rest = [a for a in sys.argv[1:] if a != "--full"]
        main_full(rest or None)
        return
    if oracle.reference_binary(False) is None:
        raise SystemExit("build the reference program first: python oracle/make_ref.py")
    for name, (p, cp, cs, rho) in cases().items():
        out = {"params": np.array(params_json(p))}
        for fp64 in (False, True):
            if fp64 and name not in ("ricker_vz_compat", "ricker_vz_clean", "explosive_gauss_deriv"):
                continue
            seis, fields, _, _ = oracle.run_reference(p, cp, cs, rho, fp64=fp64)
            tag = "f64" if fp64 else "f32"
            out[f"seis_{tag}"] = seis
            for k, v in summarize(p, fields).items():
                out[f"{k}_{tag}"] = v
        np.savez_compressed(os.path.join(HERE, f"ref_{name}.npz"), **out)
        print(name, {k: v.shape for k, v in out.items()})


if __name__ == "__main__":
    main()
