"""The oracle pinned to the reference program (CPU only).

tests/golden/ref_*.npz are outputs of the reference CPU program
seismicCPML_3d_isotropic_simpelmodel.cpp (made by tests/golden/make_golden.py);
the oracle's C restatement must reproduce them bit for bit, float32 and
float64, in every source and profile mode.  When the reference program is
built here (oracle/_ref), extra seeded cases compare the two directly.
"""
import glob
import os
import sys

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(HERE, "golden"))

import make_golden  # noqa: E402

# the small cases; the full-size workloads (ref_*_full.npz) are tested apart
GOLD = sorted(g for g in glob.glob(os.path.join(HERE, "golden", "ref_*.npz")) if not g.endswith("_full.npz"))
FULL = {os.path.basename(g)[4:-4]: g for g in glob.glob(os.path.join(HERE, "golden", "ref_*_full.npz"))}
CASES = make_golden.cases()


def test_goldens_present():
    assert len(GOLD) == len(CASES) >= 7


@pytest.mark.parametrize("path", GOLD, ids=[os.path.basename(g)[4:-4] for g in GOLD])
def test_oracle_reproduces_reference_goldens(path):
    import oracle

    name = os.path.basename(path)[4:-4]
    p, cp, cs, rho = CASES[name]
    g = np.load(path)
    assert str(g["params"]) == make_golden.params_json(p), "case definition drifted from the fixture"
    for tag, fp64 in (("f32", False), ("f64", True)):
        if f"seis_{tag}" not in g:
            continue
        seis, fields = oracle.run(p, cp, cs, rho, fp64=fp64)
        assert seis.dtype == g[f"seis_{tag}"].dtype
        assert np.array_equal(seis, g[f"seis_{tag}"]), (name, tag, "seismograms")
        s = make_golden.summarize(p, fields)
        assert np.array_equal(s["slice_xy"], g[f"slice_xy_{tag}"]), (name, tag)
        assert np.array_equal(s["slice_yz"], g[f"slice_yz_{tag}"]), (name, tag)
        assert np.array_equal(s["sum"], g[f"sum_{tag}"]), (name, tag)
        assert np.array_equal(s["sumsq"], g[f"sumsq_{tag}"]), (name, tag)


def test_oracle_reproduces_reference_on_the_full_101_cube():
    """The 101^3 homogeneous cube for all of its 1000 steps: the restatement
    equals the reference program's float32 and float64 runs bit for bit
    (about a minute of CPU)."""
    import oracle

    path = FULL.get("homogeneous_101_full")
    if path is None:
        pytest.skip("ref_homogeneous_101_full.npz not generated")
    p, cp, cs, rho = make_golden.full_cases()["homogeneous_101_full"]
    g = np.load(path)
    assert str(g["params"]) == make_golden.params_json(p), "case definition drifted from the fixture"
    for tag, fp64 in (("f32", False), ("f64", True)):
        seis, fields = oracle.run(p, cp, cs, rho, fp64=fp64)
        assert np.array_equal(seis, g[f"seis_{tag}"]), (tag, "seismograms")
        s = make_golden.summarize(p, fields)
        for key in ("slice_xy", "slice_yz", "sum", "sumsq"):
            assert np.array_equal(s[key], g[f"{key}_{tag}"]), (tag, key)


def _random_case(seed):
    from ela3d_gb300 import ShotParams, media

    rng = np.random.default_rng(seed)
    nx, ny, nz = (int(v) for v in rng.integers(12, 30, 3))
    npml = int(rng.integers(2, 6))
    src = tuple(int(rng.integers(2, n - 2)) for n in (nx, ny, nz))
    rec = np.stack([rng.integers(0, n, 6) for n in (nx, ny, nz)], axis=1).astype(np.int32)
    p = ShotParams(nx=nx, ny=ny, nz=nz, nstep=int(rng.integers(20, 60)), dt=1e-3, npml=npml,
                   pml_mode=int(rng.integers(0, 2)), f0=float(rng.uniform(15, 35)), t0=0.05,
                   stf=int(rng.integers(0, 3)), src_kind=int(rng.integers(0, 2)), src=src,
                   src_w=tuple(float(v) for v in rng.uniform(-1, 1, 3)), angle_force=float(rng.uniform(0, 90)),
                   sampgat=int(rng.integers(1, 4)), rec=rec, npower=float(rng.choice([1.0, 2.0, 3.0])),
                   k_max=float(rng.choice([1.0, 1.5])), rcoef=float(rng.choice([1e-3, 1e-4])))
    cp, cs, rho = media.random_anticline(rng, nx, ny, nz)
    return p, cp, cs, rho


@pytest.mark.parametrize("seed", range(6))
def test_oracle_matches_reference_program_directly(seed):
    import oracle

    if oracle.reference_binary(False) is None:
        pytest.skip("reference program not built in this checkout (oracle/_ref)")
    p, cp, cs, rho = _random_case(seed)
    for fp64 in (False, True):
        want_s, want_f, _, _ = oracle.run_reference(p, cp, cs, rho, fp64=fp64)
        got_s, got_f = oracle.run(p, cp, cs, rho, fp64=fp64)
        assert np.array_equal(got_s, want_s), (seed, fp64)
        assert np.array_equal(got_f, want_f), (seed, fp64)


def test_oracle_catches_a_planted_mistake():
    """A one-ulp change in the model must change the oracle's answer: the
    bit-exact comparisons above are not vacuous."""
    import oracle

    p, cp, cs, rho = CASES["ricker_vz_compat"]
    s0, _ = oracle.run(p, cp, cs, rho, want_fields=False)
    cp2 = cp.copy()
    idx = (p.src[2], p.src[1], p.src[0] + 1)
    cp2[idx] = np.nextafter(cp2[idx], np.float32(np.inf))
    s1, _ = oracle.run(p, cp2, cs, rho, want_fields=False)
    assert not np.array_equal(s0, s1)
