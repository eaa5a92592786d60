"""Oracle for parity tests.  TEST INFRASTRUCTURE: only tests/, the smoke entry
and bench.py's CPU-baseline leg use this package; the product never does.

Two checkers:
- ``run``: the C restatement (oracle/ela3d_oracle.c) of the reference CPU
  time loop, float32 or float64;
- ``run_reference``: the reference program itself
  (seismicCPML_3d_isotropic_simpelmodel.cpp built by oracle/make_ref.py into
  oracle/_ref/), driven through a config file.

Both take an ``ela3d_gb300.ShotParams`` and float32 model arrays [nz, ny, nx].
"""
from __future__ import annotations

import ctypes
import os
import subprocess
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
_LIB = None


class OracleParams(ctypes.Structure):
    _fields_ = [
        ("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
        ("dx", ctypes.c_double), ("dy", ctypes.c_double), ("dz", ctypes.c_double), ("dt", ctypes.c_double),
        ("npml", ctypes.c_int),
        ("npower", ctypes.c_double), ("k_max", ctypes.c_double), ("alpha_max", ctypes.c_double),
        ("rcoef", ctypes.c_double), ("vpml", ctypes.c_double),
        ("f0", ctypes.c_double), ("t0", ctypes.c_double), ("factor", ctypes.c_double),
        ("src_i", ctypes.c_int), ("src_j", ctypes.c_int), ("src_k", ctypes.c_int),
        ("src_kind", ctypes.c_int), ("stf", ctypes.c_int),
        ("src_w", ctypes.c_double * 3), ("angle_force", ctypes.c_double),
        ("nrec", ctypes.c_int), ("rec", ctypes.POINTER(ctypes.c_int)),
        ("sampgat", ctypes.c_int), ("pml_mode", ctypes.c_int),
    ]


def load():
    global _LIB
    if _LIB is None:
        from .build import build_oracle

        lib = ctypes.CDLL(build_oracle())
        for name in ("oracle_run_f32", "oracle_run_f64"):
            getattr(lib, name).restype = ctypes.c_int
            getattr(lib, name).argtypes = [ctypes.POINTER(OracleParams), ctypes.c_void_p, ctypes.c_void_p,
                                           ctypes.c_void_p, ctypes.c_int, ctypes.c_void_p, ctypes.c_void_p]
        for name in ("oracle_profiles_f32", "oracle_profiles_f64"):
            getattr(lib, name).restype = ctypes.c_int
            getattr(lib, name).argtypes = [ctypes.POINTER(OracleParams), ctypes.c_void_p]
        _LIB = lib
    return _LIB


def _params(p):
    rec = np.ascontiguousarray(np.asarray(p.rec, np.int32).reshape(-1, 3)).astype(np.intc)
    o = OracleParams()
    o.nx, o.ny, o.nz = p.nx, p.ny, p.nz
    o.dx, o.dy, o.dz, o.dt = p.dx, p.dy, p.dz, p.dt
    o.npml = p.npml
    o.npower, o.k_max, o.alpha_max, o.rcoef, o.vpml = p.npower, p.k_max, p.alpha_max, p.rcoef, p.vpml
    o.f0, o.t0, o.factor = p.f0, p.t0, p.factor
    o.src_i, o.src_j, o.src_k = (int(v) for v in p.src)
    o.src_kind, o.stf = p.src_kind, p.stf
    for q in range(3):
        o.src_w[q] = float(p.src_w[q])
    o.angle_force = p.angle_force
    o.nrec = rec.shape[0]
    o.rec = rec.ctypes.data_as(ctypes.POINTER(ctypes.c_int)) if rec.size else None
    o.sampgat = p.sampgat
    o.pml_mode = p.pml_mode
    return o, rec


def run(p, cp, cs, rho, nsteps: int | None = None, fp64: bool = False, want_fields: bool = True):
    """Returns (seismograms [nrec, 3, nsteps//sampgat], fields [9, nz, ny, nx] or None)."""
    lib = load()
    nsteps = p.nstep if nsteps is None else nsteps
    dt = np.float64 if fp64 else np.float32
    m = [np.ascontiguousarray(a, dtype=dt).reshape(-1) for a in (cp, cs, rho)]
    o, rec = _params(p)
    nsamp = nsteps // p.sampgat
    seis = np.zeros((rec.shape[0], 3, nsamp), dt)
    fields = np.zeros((9, p.nz, p.ny, p.nx), dt) if want_fields else None
    fn = lib.oracle_run_f64 if fp64 else lib.oracle_run_f32
    st = fn(ctypes.byref(o), m[0].ctypes.data, m[1].ctypes.data, m[2].ctypes.data, nsteps,
            seis.ctypes.data if seis.size else None, fields.ctypes.data if fields is not None else None)
    if st != 0:
        raise RuntimeError("oracle rejected the parameters")
    return seis, fields


def profiles(p, fp64: bool = True) -> dict:
    lib = load()
    dt = np.float64 if fp64 else np.float32
    o, _ = _params(p)
    out = np.zeros(6 * (p.nx + p.ny + p.nz), dt)
    (lib.oracle_profiles_f64 if fp64 else lib.oracle_profiles_f32)(ctypes.byref(o), out.ctypes.data)
    res = {}
    off = 0
    for ax, n in (("x", p.nx), ("y", p.ny), ("z", p.nz)):
        for name in ("a", "b", "K", "a_half", "b_half", "K_half"):
            res[f"{name}_{ax}"] = out[off:off + n].copy()
            off += n
    return res


def reference_binary(fp64: bool = False) -> str | None:
    exe = os.path.join(REF_DIR, "ref_f64" if fp64 else "ref_f32")
    return exe if os.path.exists(exe) else None


def write_config(path: str, p, nsteps: int, model_prefix: str, time_from: int = 1, clean: int | None = None,
                 ngatx: int = 1, ngaty: int = 1, it_output: int | None = None):
    lines = [f"nx {p.nx}", f"ny {p.ny}", f"nz {p.nz}", f"dx {int(round(p.dx))}", f"dt {p.dt!r}",
             f"nstep {nsteps}", f"sampgat {p.sampgat}", f"it_output {it_output or (1 << 30)}",
             f"ngatx {ngatx}", f"ngaty {ngaty}",
             f"npml {p.npml}", f"npower {p.npower!r}", f"k_max {p.k_max!r}", f"alpha_max {p.alpha_max!r}",
             f"rcoef {p.rcoef!r}", f"vpml {p.vpml!r}", f"f0 {p.f0!r}", f"t0 {p.t0!r}", f"factor {p.factor!r}",
             f"angle {p.angle_force!r}", "src %d %d %d" % tuple(int(v) for v in p.src),
             f"src_kind {p.src_kind}", f"stf {p.stf}", "w %r %r %r" % tuple(float(v) for v in p.src_w),
             f"clean {int(p.pml_mode) if clean is None else clean}", f"time_from {time_from}",
             f"model {model_prefix}"]
    for r in np.asarray(p.rec, np.int32).reshape(-1, 3):
        lines.append("rec %d %d %d" % tuple(int(v) for v in r))
    with open(path, "w") as f:
        f.write("\n".join(lines) + "\n")


def run_reference(p, cp, cs, rho, nsteps: int | None = None, fp64: bool = False, workdir: str | None = None,
                  time_from: int = 1, want_fields: bool = True, ngatx: int = 1, ngaty: int = 1,
                  it_output: int | None = None):
    """Runs the patched reference program.  Returns (seis, fields, seconds of
    the timed steps, number of timed steps)."""
    exe = reference_binary(fp64)
    if exe is None:
        raise RuntimeError("reference program not built (oracle/_ref)")
    if abs(p.dx - round(p.dx)) > 0 or p.dx != p.dy or p.dx != p.dz:
        raise ValueError("the reference program takes one integer spacing")
    nsteps = p.nstep if nsteps is None else nsteps
    dt = np.float64 if fp64 else np.float32
    own = workdir is None
    wd = tempfile.mkdtemp(prefix="ela3d_ref_") if own else workdir
    try:
        for name, a in (("cp", cp), ("cs", cs), ("rho", rho)):
            np.ascontiguousarray(a, dtype=dt).tofile(os.path.join(wd, f"m_{name}.bin"))
        write_config(os.path.join(wd, "cfg.txt"), p, nsteps, os.path.join(wd, "m_"), time_from,
                     ngatx=ngatx, ngaty=ngaty, it_output=it_output)
        subprocess.run([exe, os.path.join(wd, "cfg.txt")], cwd=wd, check=True, stdout=subprocess.DEVNULL)
        nrec = np.asarray(p.rec).reshape(-1, 3).shape[0]
        seis = np.fromfile(os.path.join(wd, "seis.bin"), dt).reshape(nrec, 3, nsteps // p.sampgat)
        fields = None
        if want_fields:
            fields = np.fromfile(os.path.join(wd, "fields.bin"), dt).reshape(9, p.nz, p.ny, p.nx)
        t0, t1, n = open(os.path.join(wd, "steps.txt")).read().split()
        return seis, fields, float(t1) - float(t0), int(n)
    finally:
        if own:
            import shutil
            shutil.rmtree(wd, ignore_errors=True)
