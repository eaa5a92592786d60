"""Earth models (per-cell cp, cs, rho), float32, x fastest: arrays [nz, ny, nx].

- ``homogeneous``: the constant fill of the reference CPU program
  (seismicCPML_3d_isotropic_simpelmodel.cpp:45-59).
- ``anticline_layers``: layers whose interfaces rise in a Gaussian dome,
  z_i(x, y) = d_i - A exp(-((x-xc)^2 + (y-yc)^2) / (2 s^2)) in cells.  Layer
  L occupies z_{L-1} <= k < z_L; the half-space below the last interface used
  continues the last layer.
- ``matlab_anticline``: restatement of generate_3d_model_anticline.m (201^3,
  dome Z = ((sin X + sin Y)/2 - 0.5)/0.5 clipped at 0 (:2-13), interfaces
  h - 100 Z with h = 121/161/201 (:17-30), five media (:71-76) and the k < 80
  pocket inside medium 3 (:50-55)).
- ``random_anticline``: seeded 3-6 layer dome model with cp increasing with
  depth, for uneven batches and serving streams.
"""
from __future__ import annotations

import math

import numpy as np


def homogeneous(nx: int, ny: int, nz: int, cp: float, cs: float, rho: float):
    shape = (nz, ny, nx)
    return (np.full(shape, cp, np.float32), np.full(shape, cs, np.float32), np.full(shape, rho, np.float32))


def _layer_index(nx, ny, nz, depths, amp, sigma, xc=None, yc=None):
    xc = (nx - 1) / 2.0 if xc is None else xc
    yc = (ny - 1) / 2.0 if yc is None else yc
    x = np.arange(nx, dtype=np.float64)
    y = np.arange(ny, dtype=np.float64)
    dome = amp * np.exp(-((x[None, :] - xc) ** 2 + (y[:, None] - yc) ** 2) / (2.0 * sigma * sigma))
    k = np.arange(nz, dtype=np.float64)[:, None, None]
    layer = np.zeros((nz, ny, nx), np.int32)
    for d in depths:
        layer += (k >= (d - dome)[None, :, :]).astype(np.int32)
    return layer


def anticline_layers(nx, ny, nz, depths=(40, 90, 150, 210), cps=(2000.0, 2800.0, 3500.0, 4200.0),
                     amp=25.0, sigma=50.0, cs_ratio=1.73, rho_coef=310.0, perturb=0.02, seed=0):
    """Dome-layered model.  cs = cp / cs_ratio and rho = rho_coef cp^0.25 from
    the layer cp; then cp and rho get independent uniform +-perturb relative
    noise (cp first, then rho, from numpy default_rng(seed)); cs keeps the
    unperturbed layer value."""
    layer = _layer_index(nx, ny, nz, depths, amp, sigma)
    layer = np.minimum(layer, len(cps) - 1)
    cpl = np.asarray(cps, np.float64)[layer]
    cs = cpl / cs_ratio
    rho = rho_coef * cpl ** 0.25
    cp = cpl.copy()
    if perturb > 0:
        rng = np.random.default_rng(seed)
        cp *= 1.0 + rng.uniform(-perturb, perturb, size=cp.shape)
        rho *= 1.0 + rng.uniform(-perturb, perturb, size=rho.shape)
    return cp.astype(np.float32), cs.astype(np.float32), rho.astype(np.float32)


def matlab_anticline():
    """The five-medium 201^3 anticline of generate_3d_model_anticline.m."""
    n = 201
    x = np.linspace(0.0, math.pi, n)
    X, Y = np.meshgrid(x, x)          # X[i, j] = x[j], Y[i, j] = x[i]
    Z = ((np.sin(X) + np.sin(Y)) / 2.0 - 0.5) / 0.5
    Z[Z < 0] = 0.0
    s1, s2, s3 = 121 - 100 * Z, 161 - 100 * Z, 201 - 100 * Z
    k = np.arange(1, n + 1, dtype=np.float64)[:, None, None]   # 1-based depth index
    # MATLAB surface(i, j) with i the fastest (x) index: array [i, j] -> our [j][i]
    s1t, s2t, s3t = s1.T[None], s2.T[None], s3.T[None]
    model = np.ones((n, n, n), np.int32)
    model[np.broadcast_to(k > s1t, model.shape)] = 2
    m3 = np.broadcast_to(k > s2t, model.shape)
    model[m3] = 3
    model[m3 & np.broadcast_to(k < 80, model.shape)] = 4
    model[np.broadcast_to(k > s3t, model.shape)] = 5
    media = np.array([[0, 0, 0], [3000, 1700, 2800], [3600, 1400, 2300], [3000, 1700, 2800],
                      [3600, 1700, 2800], [3650, 1500, 2450]], np.float32)
    return media[model, 0], media[model, 1], media[model, 2]


def random_anticline(rng: np.random.Generator, nx: int, ny: int, nz: int, cp_range=(1800.0, 4500.0)):
    """3-6 layers, cp sorted increasing with depth in cp_range, cs = cp / U(1.6, 2.0)
    per layer, rho = 310 cp^0.25; interfaces spread over the depth with a dome
    of random amplitude and width."""
    nl = int(rng.integers(3, 7))
    cps = np.sort(rng.uniform(cp_range[0], cp_range[1], nl))
    ratios = rng.uniform(1.6, 2.0, nl)
    depths = np.sort(rng.uniform(0.15, 0.9, nl - 1)) * nz
    amp = float(rng.uniform(0.05, 0.2)) * nz
    sigma = float(rng.uniform(0.15, 0.35)) * min(nx, ny)
    layer = _layer_index(nx, ny, nz, depths, amp, sigma)
    cp = cps[layer]
    cs = cp / ratios[layer]
    rho = 310.0 * cp ** 0.25
    return cp.astype(np.float32), cs.astype(np.float32), rho.astype(np.float32)


# ---------------------------------------------------------------------------
# Models generated on the GPU (ela3d_model_spec in include/ela3d.h).  The
# functions below build the specs; ``generate_host`` is a host restatement
# of the device generator used to check it.
MODEL_HOMOGENEOUS, MODEL_LAYERED_DOME, MODEL_MATLAB_ANTICLINE = 0, 1, 2


def homogeneous_spec(cp: float, cs: float, rho: float) -> dict:
    return {"kind": MODEL_HOMOGENEOUS, "cp0": cp, "cs0": cs, "rho0": rho}


def dome_spec(nx: int, ny: int, depths, cps, cs_ratio, amp: float, sigma: float, rho_coef: float = 310.0,
              rho_pow: float = 0.25, perturb: float = 0.0, seed: int = 0, xc=None, yc=None) -> dict:
    """Layered dome: layer L below interface L-1; cs_ratio per layer (a
    number applies to all)."""
    n = len(cps)
    ratios = [cs_ratio] * n if np.isscalar(cs_ratio) else list(cs_ratio)
    return {"kind": MODEL_LAYERED_DOME, "nlayers": n, "cp": list(cps), "cs_ratio": ratios,
            "depth": list(depths)[:n], "dome_amp": amp, "dome_sigma": sigma,
            "dome_xc": (nx - 1) / 2.0 if xc is None else xc, "dome_yc": (ny - 1) / 2.0 if yc is None else yc,
            "rho_coef": rho_coef, "rho_pow": rho_pow, "perturb": perturb, "seed": seed}


def matlab_spec() -> dict:
    return {"kind": MODEL_MATLAB_ANTICLINE}


def anticline_256_spec(n: int = 256, seed: int = 0) -> dict:
    """The 256^3 four-layer dome of configs.anticline_256 with the device's
    hash noise (same statistics as the host model, a different realisation)."""
    s = n / 256.0
    return dome_spec(n, n, [d * s for d in (40, 90, 150, 210)], [2000.0, 2800.0, 3500.0, 4200.0], 1.73,
                     25.0 * s, 50.0 * s, perturb=0.02, seed=seed)


def _splitmix_uniform(seed: int, cell: np.ndarray, stream: int) -> np.ndarray:
    with np.errstate(over="ignore"):
        z = (np.uint64(seed) + np.uint64(0x9E3779B97F4A7C15) * (cell.astype(np.uint64) * np.uint64(2)
                                                                 + np.uint64(stream + 1)))
        z = (z ^ (z >> np.uint64(30))) * np.uint64(0xBF58476D1CE4E5B9)
        z = (z ^ (z >> np.uint64(27))) * np.uint64(0x94D049BB133111EB)
        z = z ^ (z >> np.uint64(31))
    return (z >> np.uint64(11)).astype(np.float64) * (1.0 / 9007199254740992.0)


def generate_host(spec: dict, nx: int, ny: int, nz: int):
    """Host restatement of the device generator (float32 [nz, ny, nx])."""
    kind = spec["kind"]
    shape = (nz, ny, nx)
    if kind == MODEL_HOMOGENEOUS:
        return tuple(np.full(shape, np.float32(spec[k]), np.float32) for k in ("cp0", "cs0", "rho0"))
    k = np.arange(nz, dtype=np.float64)[:, None, None]
    y = np.arange(ny, dtype=np.float64)[None, :, None]
    x = np.arange(nx, dtype=np.float64)[None, None, :]
    if kind == MODEL_LAYERED_DOME:
        dome = spec["dome_amp"] * np.exp(-((x - spec["dome_xc"]) ** 2 + (y - spec["dome_yc"]) ** 2)
                                         / (2.0 * spec["dome_sigma"] ** 2))
        L = np.zeros(shape, np.int64)
        for d in spec["depth"][: spec["nlayers"]]:
            L += (k >= d - dome)
        L = np.minimum(L, spec["nlayers"] - 1)
        cpl = np.asarray(spec["cp"], np.float64)[L]
        cs = cpl / np.asarray(spec["cs_ratio"], np.float64)[L]
        rho = spec["rho_coef"] * cpl ** spec["rho_pow"]
        cp = cpl.copy()
        if spec["perturb"] > 0:
            cell = np.arange(nx * ny * nz, dtype=np.uint64).reshape(shape)
            cp *= 1.0 + spec["perturb"] * (2.0 * _splitmix_uniform(spec["seed"], cell, 0) - 1.0)
            rho *= 1.0 + spec["perturb"] * (2.0 * _splitmix_uniform(spec["seed"], cell, 1) - 1.0)
        return cp.astype(np.float32), cs.astype(np.float32), rho.astype(np.float32)
    # MATLAB anticline, depths scaled by nz / 201
    X = math.pi * x / (nx - 1)
    Y = math.pi * y / (ny - 1)
    Z = np.maximum(((np.sin(X) + np.sin(Y)) / 2.0 - 0.5) / 0.5, 0.0)
    sc = nz / 201.0
    kk = k + 1
    m = np.ones(np.broadcast_shapes(kk.shape, Z.shape), np.int32)
    m[np.broadcast_to(kk > 121 * sc - 100 * sc * Z, m.shape)] = 2
    m3 = np.broadcast_to(kk > 161 * sc - 100 * sc * Z, m.shape)
    m[m3] = 3
    m[m3 & np.broadcast_to(kk < 80 * sc, m.shape)] = 4
    m[np.broadcast_to(kk > 201 * sc - 100 * sc * Z, m.shape)] = 5
    media = np.array([[0, 0, 0], [3000, 1700, 2800], [3600, 1400, 2300], [3000, 1700, 2800],
                      [3600, 1700, 2800], [3650, 1500, 2450]], np.float32)
    return media[m, 0], media[m, 1], media[m, 2]
