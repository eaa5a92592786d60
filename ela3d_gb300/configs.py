"""The benchmark workloads as (ShotParams, cp, cs, rho).

- homogeneous_101: 101^3 cube, cp 3300, cs cp/1.732, rho 2800, dt 1.6e-3,
  1000 steps, 10 PML cells, Ricker 7 Hz on vz at the centre, 11 receivers
  every 5 cells along x through the source.
- anticline_256: 256^3 four-layer dome model (+-2% noise, seed 0), dt 1e-3,
  2000 steps, 16 PML cells, Ricker 12 Hz on vz at (128, 128, 19), a 201-point
  receiver line along x centred on the source.
- anticline_256_shots: 64 shots of anticline_256 on a regular 8 x 8 (x, y)
  grid at z = npml + 3, sharing one model; each 201-point line is centred on
  its source and shifted to stay inside [0, nx-1].
- uneven_batch: 48 grids with edges drawn from multiples of 16 in [64, 320]
  (numpy default_rng(1)), random 3-6 layer domes, npml U{10..20}, dt half
  the CFL limit, nstep reaching t = 2 s.
- serving_request: one request of a stream with lognormal edges clipped to
  [64, 384] (mu = ln 128, sigma = 0.45), per-request seed for model, source
  and receiver line; npml U{10..20}, at most (min edge - 10) / 2.
  serving_request_spec: the same request with its model generated on the
  device.
Edge lengths, positions and seeds are those the configs name; anything they
leave open is fixed here and stated in the docstring.
"""
from __future__ import annotations

import math

import numpy as np

from . import media
from .params import FP32, PML_COMPAT, SRC_FORCE, STF_RICKER, ShotParams


def _line(xs: int, n: int, count: int, y: int, z: int) -> np.ndarray:
    start = min(max(xs - count // 2, 0), max(n - count, 0))
    xsn = np.arange(start, min(start + count, n), dtype=np.int32)
    return np.stack([xsn, np.full_like(xsn, y), np.full_like(xsn, z)], axis=1)


def homogeneous_101(precision: int = FP32, nstep: int = 1000, pml_mode: int = PML_COMPAT):
    n = 101
    cp = 3300.0
    f0 = 7.0
    rec = np.array([[50 + 5 * m, 50, 50] for m in range(-5, 6)], np.int32)
    p = ShotParams(nx=n, ny=n, nz=n, nstep=nstep, dx=10.0, dy=10.0, dz=10.0, dt=1.6e-3, npml=10,
                   pml_mode=pml_mode, npower=2.0, k_max=1.0, alpha_max=-1.0, rcoef=1e-3, vpml=3000.0,
                   f0=f0, t0=1.2 / f0, factor=1e7, stf=STF_RICKER, src_kind=SRC_FORCE, src=(50, 50, 50),
                   src_w=(0.0, 0.0, 1.0), sampgat=1, rec=rec, precision=precision)
    return (p,) + media.homogeneous(n, n, n, cp, cp / 1.732, 2800.0)


def anticline_256(precision: int = FP32, nstep: int = 2000, n: int = 256, pml_mode: int = PML_COMPAT,
                  src_xy: tuple | None = None):
    npml = 16
    f0 = 12.0
    sx, sy = (n // 2, n // 2) if src_xy is None else src_xy
    sz = npml + 3
    p = ShotParams(nx=n, ny=n, nz=n, nstep=nstep, dx=10.0, dy=10.0, dz=10.0, dt=1e-3, npml=npml,
                   pml_mode=pml_mode, f0=f0, t0=1.2 / f0, factor=1e7, stf=STF_RICKER, src_kind=SRC_FORCE,
                   src=(sx, sy, sz), src_w=(0.0, 0.0, 1.0), sampgat=1, rec=_line(sx, n, 201, sy, sz),
                   precision=precision)
    scale = n / 256.0
    cp, cs, rho = media.anticline_layers(n, n, n, depths=tuple(d * scale for d in (40, 90, 150, 210)),
                                         amp=25.0 * scale, sigma=50.0 * scale, seed=0)
    return p, cp, cs, rho


def shot_grid_positions(n: int, npml: int, per_axis: int = 8) -> list[tuple[int, int]]:
    inner = n - 2 * npml
    xs = [npml + int(round(inner * (i + 0.5) / per_axis)) for i in range(per_axis)]
    return [(x, y) for y in xs for x in xs]


def anticline_256_shots(nshots: int = 64, precision: int = FP32, nstep: int = 2000, n: int = 256):
    base, cp, cs, rho = anticline_256(precision=precision, nstep=nstep, n=n)
    per_axis = int(round(math.sqrt(nshots)))
    shots = []
    for (sx, sy) in shot_grid_positions(n, base.npml, per_axis)[:nshots]:
        shots.append(base.with_(src=(sx, sy, base.npml + 3), rec=_line(sx, n, 201, sy, base.npml + 3)))
    return shots, cp, cs, rho


def cfl_dt(cp_max: float, dx: float, dy: float, dz: float, fraction: float = 0.5) -> float:
    return fraction / (cp_max * math.sqrt(1.0 / dx ** 2 + 1.0 / dy ** 2 + 1.0 / dz ** 2))


def uneven_batch(count: int = 48, seed: int = 1, t_end: float = 2.0, precision: int = FP32,
                 edges=tuple(range(64, 321, 16)), f0: float = 10.0):
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(count):
        nx, ny, nz = (int(rng.choice(edges)) for _ in range(3))
        npml = int(rng.integers(10, 21))
        cp, cs, rho = media.random_anticline(rng, nx, ny, nz)
        dt = cfl_dt(float(cp.max()), 10.0, 10.0, 10.0, 0.5)
        nstep = int(math.ceil(t_end / dt))
        sx, sy, sz = nx // 2, ny // 2, npml + 3
        p = ShotParams(nx=nx, ny=ny, nz=nz, nstep=nstep, dt=dt, npml=npml, f0=f0, t0=1.2 / f0,
                       src=(sx, sy, sz), rec=_line(sx, nx, 201, sy, sz), precision=precision)
        out.append((p, cp, cs, rho))
    return out


def serving_request_spec(seed: int, t_end: float = 2.0, precision: int = FP32, lo: int = 64, hi: int = 384,
                         mu: float = math.log(128.0), sigma: float = 0.45, f0: float = 10.0):
    """The same request as serving_request(seed) -- the same draws from the
    same seed, so the same grid, layers, time step, source and receivers --
    with its model as a device-generator spec (ela3d_model_spec) instead of
    host arrays: the layered dome of media.random_anticline, generated on
    the GPU at admission.  Returns (ShotParams, spec)."""
    rng = np.random.default_rng(seed)
    edges = [int(min(max(round(rng.lognormal(mu, sigma)), lo), hi)) for _ in range(3)]
    nx, ny, nz = edges
    npml = min(int(rng.integers(10, 21)), (min(edges) - 10) // 2)
    # media.random_anticline's draws, in its order
    nl = int(rng.integers(3, 7))
    cps = np.sort(rng.uniform(1800.0, 4500.0, nl))
    ratios = rng.uniform(1.6, 2.0, nl)
    depths = np.sort(rng.uniform(0.15, 0.9, nl - 1)) * nz
    amp = float(rng.uniform(0.05, 0.2)) * nz
    sig = float(rng.uniform(0.15, 0.35)) * min(nx, ny)
    # nl - 1 interfaces; the device counts interfaces crossed, so a last one
    # far below the grid keeps the deepest layer to the bottom
    spec = media.dome_spec(nx, ny, list(depths) + [1e9], [float(c) for c in cps], [float(r) for r in ratios], amp,
                           sig)
    # (the host model's fastest velocity is the float32 of the layer's)
    dt = cfl_dt(float(np.float32(cps.max())), 10.0, 10.0, 10.0, 0.5)
    nstep = int(math.ceil(t_end / dt))
    sx = int(rng.integers(npml + 2, nx - npml - 2))
    sy = int(rng.integers(npml + 2, ny - npml - 2))
    sz = npml + 3
    p = ShotParams(nx=nx, ny=ny, nz=nz, nstep=nstep, dt=dt, npml=npml, f0=f0, t0=1.2 / f0, src=(sx, sy, sz),
                   rec=_line(sx, nx, min(201, nx), sy, sz), precision=precision)
    return p, spec


def serving_request(seed: int, t_end: float = 2.0, precision: int = FP32, lo: int = 64, hi: int = 384,
                    mu: float = math.log(128.0), sigma: float = 0.45, f0: float = 10.0):
    rng = np.random.default_rng(seed)
    edges = [int(min(max(round(rng.lognormal(mu, sigma)), lo), hi)) for _ in range(3)]
    nx, ny, nz = edges
    npml = min(int(rng.integers(10, 21)), (min(edges) - 10) // 2)
    cp, cs, rho = media.random_anticline(rng, nx, ny, nz)
    dt = cfl_dt(float(cp.max()), 10.0, 10.0, 10.0, 0.5)
    nstep = int(math.ceil(t_end / dt))
    sx = int(rng.integers(npml + 2, nx - npml - 2))
    sy = int(rng.integers(npml + 2, ny - npml - 2))
    sz = npml + 3
    p = ShotParams(nx=nx, ny=ny, nz=nz, nstep=nstep, dt=dt, npml=npml, f0=f0, t0=1.2 / f0, src=(sx, sy, sz),
                   rec=_line(sx, nx, min(201, nx), sy, sz), precision=precision)
    return p, cp, cs, rho
