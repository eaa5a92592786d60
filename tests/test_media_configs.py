"""Workload generators: models, receiver lines, shot grids, CFL steps."""
import math

import numpy as np
import pytest


def test_anticline_256_model():
    from ela3d_gb300 import configs

    p, cp, cs, rho = configs.anticline_256(n=64)
    assert cp.shape == (64, 64, 64) and cp.dtype == np.float32
    layers = np.array([2000.0, 2800.0, 3500.0, 4200.0])
    # cs carries the unperturbed layer velocity; cp and rho are within +-2%
    cpl = cs.astype(np.float64) * 1.73
    assert np.all(np.min(np.abs(cpl[..., None] - layers), axis=-1) < 0.01)
    assert np.all(np.abs(cp / cpl - 1) <= 0.02 + 1e-6)
    assert np.all(np.abs(rho / (310 * cpl ** 0.25) - 1) <= 0.02 + 1e-6)
    # velocity increases with depth on average, dome rises at the centre
    assert cs[0].mean() < cs[-1].mean()
    depth_of_2nd = lambda x, y: np.argmax(cs[:, y, x] * 1.73 > 2400)
    assert depth_of_2nd(32, 32) < depth_of_2nd(2, 2)
    # reproducible from the seed
    _, cp2, _, _ = configs.anticline_256(n=64)
    assert np.array_equal(cp, cp2)


def test_anticline_256_receivers_and_source():
    from ela3d_gb300 import configs

    p, *_ = configs.anticline_256(nstep=10, n=256)
    assert p.src == (128, 128, 19) and p.npml == 16
    rec = p.rec_array()
    assert rec.shape == (201, 3)
    assert rec[0, 0] == 28 and rec[-1, 0] == 228 and np.all(rec[:, 1] == 128) and np.all(rec[:, 2] == 19)


def test_homogeneous_101():
    from ela3d_gb300 import configs

    p, cp, cs, rho = configs.homogeneous_101()
    assert (p.nx, p.nstep, p.dt, p.npml, p.f0) == (101, 1000, 1.6e-3, 10, 7.0)
    assert p.rec_array()[:, 0].tolist() == list(range(25, 76, 5))
    assert np.all(cp == 3300) and np.allclose(cs, 3300 / 1.732) and np.all(rho == 2800)
    courant = 3300 * p.dt * math.sqrt(3) / p.dx
    assert 0.9 < courant < 0.92


def test_shot_grid_and_lines_stay_inside():
    from ela3d_gb300 import configs

    shots, cp, cs, rho = configs.anticline_256_shots(64, nstep=10, n=256)
    assert len(shots) == 64
    pos = {(s.src[0], s.src[1]) for s in shots}
    assert len(pos) == 64
    for s in shots:
        r = s.rec_array()
        assert r.shape == (201, 3) and r[:, 0].min() >= 0 and r[:, 0].max() <= 255
        assert s.src[2] == 19


def test_uneven_batch_properties():
    from ela3d_gb300 import configs

    inst = configs.uneven_batch(count=6)
    for p, cp, cs, rho in inst:
        for n in (p.nx, p.ny, p.nz):
            assert n % 16 == 0 and 64 <= n <= 320
        assert 10 <= p.npml <= 20
        dt_cfl = 1.0 / (float(cp.max()) * math.sqrt(3) / 10.0)
        assert p.dt == pytest.approx(0.5 * dt_cfl)
        assert p.nstep * p.dt >= 2.0 - 1e-9
        ratio = cp / cs
        assert ratio.min() >= 1.6 - 1e-4 and ratio.max() <= 2.0 + 1e-4
        assert 1800 - 1e-3 <= cp.min() and cp.max() <= 4500 + 1e-3


def test_matlab_anticline_restatement():
    from ela3d_gb300 import media

    cp, cs, rho = media.matlab_anticline()
    assert cp.shape == (201, 201, 201)
    media_set = {tuple(v) for v in np.stack([cp.ravel(), cs.ravel(), rho.ravel()], 1)[::997]}
    assert (3000, 1700, 2800) in media_set and (3650, 1500, 2450) in media_set
    # top of the model is medium 1; at the bottom the dome crest (x = y = pi/2)
    # has reached medium 5 while the flat corners stay in medium 3
    assert (cp[0, 0, 0], cs[0, 0, 0]) == (3000, 1700)
    assert (cp[-1, 100, 100], cs[-1, 100, 100]) == (3650, 1500)
    assert (cp[-1, 0, 0], cs[-1, 0, 0], rho[-1, 0, 0]) == (3000, 1700, 2800)
    # the dome is symmetric in x and y
    assert np.array_equal(cp, cp.transpose(0, 2, 1))
    # the oil pocket (medium 4) only above k = 80 (1-based)
    k4 = np.nonzero((cp == 3600) & (cs == 1700))[0]
    assert k4.size > 0 and k4.max() < 79


@pytest.mark.parametrize("seed", [1000, 1007, 1333])
def test_serving_request_spec_is_the_same_request(seed):
    """The device-model form of a serving request has the same grid, time
    step, source and receivers, and its generated model (host restatement of
    the device generator) equals the host request's model."""
    from ela3d_gb300 import configs, media

    p, cp, cs, rho = configs.serving_request(seed, t_end=0.25)
    q, spec = configs.serving_request_spec(seed, t_end=0.25)
    assert (p.nx, p.ny, p.nz, p.nstep, p.npml, p.src, p.dt) == (q.nx, q.ny, q.nz, q.nstep, q.npml, q.src, q.dt)
    assert np.array_equal(p.rec, q.rec)
    for a, b in zip(media.generate_host(spec, p.nx, p.ny, p.nz), (cp, cs, rho)):
        assert np.array_equal(a, b)
