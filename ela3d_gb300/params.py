"""Parameter block of one shot: the reference's hard-coded locals as fields.

Mirrors ``ela3d_params`` of include/ela3d.h field by field.  The names
follow the reference CPU program seismicCPML_3d_isotropic_simpelmodel.cpp
(NIMX/NIMY/NIMZ :19-22, DELTAX :35-36, DELTATT/NSTEP/sampgat :30-33,
f0/t0/factor :61-64, NPOINTS_PML :66, I/J/KSOURCEE and ANGLE_FORCEE :68-72,
NPOWER/K_MAX_PML/ALPHA_MAX_PML :75-78, Rcoef/vpml :151-153); indices are
0-based (the reference's 1-based cell (i+1, j+1, k+1)).
"""
from __future__ import annotations

import ctypes
import math
from dataclasses import dataclass, field, replace

import numpy as np

FP32, FP64 = 0, 1
PML_COMPAT, PML_CLEAN = 0, 1
STF_RICKER, STF_GAUSS_DERIV, STF_GAUSS = 0, 1, 2
SRC_FORCE, SRC_EXPLOSIVE = 0, 1
VX, VY, VZ, SXX, SYY, SZZ, SXY, SXZ, SYZ = range(9)
FIELD_NAMES = ("vx", "vy", "vz", "sxx", "syy", "szz", "sxy", "sxz", "syz")


class CParams(ctypes.Structure):
    """ctypes mirror of ``ela3d_params`` (include/ela3d.h)."""

    _fields_ = [
        ("nx", ctypes.c_int32), ("ny", ctypes.c_int32), ("nz", ctypes.c_int32), ("nstep", ctypes.c_int32),
        ("dx", ctypes.c_double), ("dy", ctypes.c_double), ("dz", ctypes.c_double), ("dt", ctypes.c_double),
        ("npml", ctypes.c_int32), ("pml_mode", ctypes.c_int32),
        ("npower", ctypes.c_double), ("k_max", ctypes.c_double), ("alpha_max", ctypes.c_double),
        ("rcoef", ctypes.c_double), ("vpml", ctypes.c_double),
        ("f0", ctypes.c_double), ("t0", ctypes.c_double), ("factor", ctypes.c_double),
        ("stf", ctypes.c_int32), ("src_kind", ctypes.c_int32),
        ("src_i", ctypes.c_int32), ("src_j", ctypes.c_int32), ("src_k", ctypes.c_int32),
        ("sampgat", ctypes.c_int32),
        ("src_w", ctypes.c_double * 3), ("angle_force", ctypes.c_double),
        ("rec", ctypes.POINTER(ctypes.c_int32)), ("nrec", ctypes.c_int32), ("precision", ctypes.c_int32),
        ("it_output", ctypes.c_int32), ("energy_every", ctypes.c_int32),
    ]


@dataclass
class ShotParams:
    nx: int = 101
    ny: int = 101
    nz: int = 101
    nstep: int = 1000
    dx: float = 10.0
    dy: float = 10.0
    dz: float = 10.0
    dt: float = 1.6e-3
    npml: int = 10
    pml_mode: int = PML_COMPAT
    npower: float = 2.0
    k_max: float = 1.0
    alpha_max: float = -1.0      # < 0: pi * f0, as the reference computes it
    rcoef: float = 1e-3
    vpml: float = 3000.0
    f0: float = 7.0
    t0: float = 1.2 / 7.0
    factor: float = 1e7
    stf: int = STF_RICKER
    src_kind: int = SRC_FORCE
    src: tuple = (50, 50, 50)
    sampgat: int = 1
    src_w: tuple = (0.0, 0.0, 1.0)
    angle_force: float = 0.0
    rec: np.ndarray = field(default_factory=lambda: np.zeros((0, 3), np.int32))
    precision: int = FP32
    it_output: int = 0
    energy_every: int = 0

    @property
    def nsamp(self) -> int:
        return self.nstep // self.sampgat

    @property
    def nrec(self) -> int:
        return int(np.asarray(self.rec).reshape(-1, 3).shape[0])

    @property
    def cells(self) -> int:
        return self.nx * self.ny * self.nz

    def with_(self, **kw) -> "ShotParams":
        return replace(self, **kw)

    def rec_array(self) -> np.ndarray:
        return np.ascontiguousarray(np.asarray(self.rec, dtype=np.int32).reshape(-1, 3))

    def alpha_max_value(self) -> float:
        return math.pi * self.f0 if self.alpha_max < 0 else self.alpha_max

    def to_c(self) -> tuple[CParams, np.ndarray]:
        """Returns the ctypes struct and the receiver array it points into
        (keep the array alive while the struct is used)."""
        rec = self.rec_array()
        c = CParams()
        c.nx, c.ny, c.nz, c.nstep = self.nx, self.ny, self.nz, self.nstep
        c.dx, c.dy, c.dz, c.dt = self.dx, self.dy, self.dz, self.dt
        c.npml, c.pml_mode = self.npml, self.pml_mode
        c.npower, c.k_max, c.alpha_max = self.npower, self.k_max, self.alpha_max
        c.rcoef, c.vpml = self.rcoef, self.vpml
        c.f0, c.t0, c.factor = self.f0, self.t0, self.factor
        c.stf, c.src_kind = self.stf, self.src_kind
        c.src_i, c.src_j, c.src_k = (int(v) for v in self.src)
        c.sampgat = self.sampgat
        for q in range(3):
            c.src_w[q] = float(self.src_w[q])
        c.angle_force = self.angle_force
        c.rec = rec.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)) if rec.size else None
        c.nrec = rec.shape[0]
        c.precision = self.precision
        c.it_output = self.it_output
        c.energy_every = self.energy_every
        return c, rec


def reference_defaults() -> ShotParams:
    """The reference CPU program's own settings (simpelmodel.cpp:19-78):
    500^3, f0=35 Hz, Gaussian-derivative explosive source at 1-based
    (DIMX/2, DIMY/2, 11), sampgat=2."""
    return ShotParams(nx=500, ny=500, nz=500, nstep=1000, dt=1e-3, npml=10, f0=35.0, t0=1.2 / 35.0,
                      factor=1e7, stf=STF_GAUSS_DERIV, src_kind=SRC_EXPLOSIVE,
                      src=(501 // 2 - 1, 501 // 2 - 1, 11 - 1), sampgat=2, it_output=200)
