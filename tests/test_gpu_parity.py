"""GPU parity: the sm_103a kernels through the C ABI against the oracle.

The oracle is the C restatement of the reference CPU program
(seismicCPML_3d_isotropic_simpelmodel.cpp), pinned bit-for-bit to that
program in tests/test_oracle_pin.py.  Tolerances:
  FP32 GPU vs FP32 oracle: relative L2 <= 2e-5 on every seismogram and field
    (same formulas; the GPU fuses multiply-adds and multiplies by 1/K);
  FP64 GPU vs FP64 oracle: relative L2 <= 1e-11;
  kernel variants and schedules: bit-identical to each other.
"""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

TOL32 = 2e-5
TOL64 = 1e-11


def small_case(**kw):
    from ela3d_gb300 import ShotParams, media

    nx, ny, nz = kw.pop("shape", (40, 34, 46))
    rec = [[x, ny // 2, nz // 2 - 3] for x in range(1, nx - 1, 5)]
    rec += [[nx // 2, ny // 2, nz // 2], [0, 0, 0], [nx - 1, ny - 1, nz - 1], [3, ny - 2, 1]]
    p = ShotParams(nx=nx, ny=ny, nz=nz, nstep=100, dt=1e-3, npml=6, f0=22.0, t0=1.2 / 22.0,
                   src=(nx // 2, ny // 2, nz // 2), rec=np.array(rec, np.int32), sampgat=1)
    p = p.with_(**kw)
    cp, cs, rho = media.anticline_layers(nx, ny, nz, depths=(nz * 0.25, nz * 0.5, nz * 0.7, nz * 2),
                                         amp=nz * 0.08, sigma=nx * 0.25, seed=7)
    return p, cp, cs, rho


def run_gpu(p, cp, cs, rho, nsteps=None, **tune):
    from ela3d_gb300 import Plan

    with Plan(p, cp, cs, rho, **tune) as plan:
        plan.run(p.nstep if nsteps is None else nsteps)
        fp64 = p.precision == 1
        seis = plan.seismograms(fp64=fp64)
        fields = np.stack([plan.field(c, fp64=fp64) for c in range(9)])
    return seis, fields


def check(seis, fields, want_s, want_f, tol):
    assert rel_l2(seis, want_s) <= tol, rel_l2(seis, want_s)
    for c in range(9):
        assert rel_l2(fields[c], want_f[c]) <= tol, (c, rel_l2(fields[c], want_f[c]))


CASES = {
    "ricker_vz_compat": {},
    "ricker_vz_clean": {"pml_mode": 1},
    "explosive_gauss_deriv": {"stf": 1, "src_kind": 1},
    "explosive_angle": {"stf": 1, "src_kind": 1, "angle_force": 35.0},
    "force_xyz_gauss": {"stf": 2, "src_w": (0.7, -0.4, 1.0)},
    "sampgat3_odd_shape": {"sampgat": 3, "shape": (37, 29, 31)},
    "thin_z": {"shape": (52, 44, 14), "npml": 4},
    "pml_covers_grid": {"shape": (16, 18, 20), "npml": 9, "nstep": 60},
    "no_pml": {"npml": 0},
    "explosive_far_corner": {"stf": 1, "src_kind": 1, "src": (0, 33, 45)},
    # per-axis spacings (the reference hard-codes DELTAY = DELTAZ = DELTAX;
    # the API takes three, and both restatements use each where it belongs)
    "anisotropic_spacing_compat": {"dx": 10.0, "dy": 12.5, "dz": 8.0},
    "anisotropic_spacing_clean": {"dx": 10.0, "dy": 12.5, "dz": 8.0, "pml_mode": 1},
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_fp32_matches_oracle(built, name):
    import oracle

    p, cp, cs, rho = small_case(**CASES[name])
    seis, fields = run_gpu(p, cp, cs, rho)
    want_s, want_f = oracle.run(p, cp, cs, rho)
    check(seis, fields, want_s, want_f, TOL32)


@pytest.mark.parametrize("name", ["ricker_vz_compat", "ricker_vz_clean", "explosive_gauss_deriv"])
def test_fp64_matches_oracle(built, name):
    import oracle

    p, cp, cs, rho = small_case(**CASES[name])
    p = p.with_(precision=1)
    seis, fields = run_gpu(p, cp, cs, rho)
    want_s, want_f = oracle.run(p, cp, cs, rho, fp64=True)
    check(seis, fields, want_s, want_f, TOL64)


def test_variants_and_schedules_bit_identical(built):
    import ela3d_gb300

    p, cp, cs, rho = small_case(nstep=40, pml_mode=1)
    ref = None
    for i, v in enumerate(ela3d_gb300.variants()):
        if v.fp64:
            continue
        for sched, chunk, pf in ((0, 0, 6), (1, 5, 0), (1, 64, 2), (1, 7, 4)):
            seis, fields = run_gpu(p, cp, cs, rho, variant=i, schedule=sched, chunk=chunk, prefetch=pf)
            if ref is None:
                ref = (seis, fields)
            else:
                assert np.array_equal(seis, ref[0]), (i, sched, chunk, pf)
                assert np.array_equal(fields, ref[1]), (i, sched, chunk, pf)


def test_fp64_variants_agree(built):
    """Schedules are bit-identical within an FP64 variant; variants with one
    and two cells per thread fuse multiply-adds differently, so across them
    the results agree to round-off (1e-13 relative L2)."""
    import ela3d_gb300

    p, cp, cs, rho = small_case(nstep=30, precision=1)
    ref = None
    for i, v in enumerate(ela3d_gb300.variants()):
        if not v.fp64:
            continue
        mine = None
        for sched, chunk in ((0, 0), (1, 6)):
            seis, fields = run_gpu(p, cp, cs, rho, variant=i, schedule=sched, chunk=chunk)
            if mine is None:
                mine = (seis, fields)
            else:
                assert np.array_equal(seis, mine[0]) and np.array_equal(fields, mine[1]), (i, sched, chunk)
        if ref is None:
            ref = mine
        else:
            assert rel_l2(mine[0], ref[0]) <= 1e-13 and rel_l2(mine[1], ref[1]) <= 1e-13, i


def test_resume_equals_single_run(built):
    from ela3d_gb300 import Plan

    p, cp, cs, rho = small_case(nstep=60)
    one_s, one_f = run_gpu(p, cp, cs, rho)
    with Plan(p, cp, cs, rho) as plan:
        plan.run(17)
        plan.run(0)
        plan.run(43)
        assert plan.info().step == 60
        s = plan.seismograms()
        f = np.stack([plan.field(c) for c in range(9)])
    assert np.array_equal(s, one_s)
    assert np.array_equal(f, one_f)


def test_energy_positive_and_decays(built):
    from ela3d_gb300 import Plan

    p, cp, cs, rho = small_case(nstep=400, npml=8)
    with Plan(p, cp, cs, rho) as plan:
        plan.run(150)
        e1 = plan.energy()
        plan.run(250)
        e2 = plan.energy()
    assert np.isfinite(e1) and e1 > 0
    assert e2 < e1


def test_steps_past_nstep_propagate_without_source_or_recording(built):
    """Past nstep the wavefield keeps moving with no source and no recording:
    the seismograms and source trace stay those of the first nstep steps, and
    a checkpoint taken there resumes as usual."""
    from ela3d_gb300 import Plan

    p, cp, cs, rho = small_case(nstep=60)
    with Plan(p, cp, cs, rho) as plan:
        plan.run(60)
        s60, t60 = plan.seismograms(), plan.source_trace()
        f60 = plan.field(2)
        plan.run(25)
        assert plan.info().step == 85
        assert np.array_equal(plan.seismograms(), s60)
        assert np.array_equal(plan.source_trace(), t60)
        assert not np.array_equal(plan.field(2), f60)
        ck = plan.checkpoint()
        plan.run(10)
        want = plan.field(2)
    with Plan(p, cp, cs, rho) as again:
        again.restore(ck)
        assert again.info().step == 85
        again.run(10)
        assert np.array_equal(again.field(2), want)


@pytest.mark.parametrize("shape,npml", [((3, 3, 3), 0), ((3, 4, 5), 1), ((5, 3, 4), 1)])
def test_smallest_grids(built, shape, npml):
    """The smallest grids the API accepts (3 cells on an axis: one updated
    cell between the two edges), with and without a C-PML layer."""
    import oracle
    from ela3d_gb300 import ShotParams, media

    nx, ny, nz = shape
    rec = np.array([[x, y, z] for x in range(nx) for y in range(ny) for z in range(nz)], np.int32)
    p = ShotParams(nx=nx, ny=ny, nz=nz, nstep=30, dt=1e-3, npml=npml, f0=30.0, t0=0.04,
                   src=(nx // 2, ny // 2, nz // 2), rec=rec, sampgat=1)
    cp, cs, rho = media.anticline_layers(nx, ny, nz, depths=(1, 2, 3, 9), amp=0.5, sigma=2, seed=3)
    seis, fields = run_gpu(p, cp, cs, rho)
    want_s, want_f = oracle.run(p, cp, cs, rho)
    assert np.any(want_s != 0)
    check(seis, fields, want_s, want_f, TOL32)


def test_no_samples_and_no_receivers(built):
    """sampgat larger than nstep (no sample is ever taken) and a shot without
    receivers: empty seismograms, the same fields as with receivers."""
    from ela3d_gb300 import Plan

    p, cp, cs, rho = small_case(nstep=12)
    _, want_f = run_gpu(p, cp, cs, rho)
    for q in (p.with_(sampgat=13), p.with_(rec=np.zeros((0, 3), np.int32))):
        with Plan(q, cp, cs, rho) as plan:
            plan.run(q.nstep)
            s = plan.seismograms()
            f = np.stack([plan.field(c) for c in range(9)])
        assert s.size == 0
        assert np.array_equal(f, want_f)


def test_plans_in_concurrent_threads(built):
    """One plan per thread, four threads at once on the same device (each
    plan owns its streams and memory): every plan's results equal the same
    plan run alone."""
    import threading

    from ela3d_gb300 import Plan

    cases = [small_case(nstep=40, src=(10 + 5 * q, 17, 23)) for q in range(4)]
    want = [run_gpu(*c) for c in cases]
    got = [None] * 4
    errors = []

    def worker(q):
        try:
            p, cp, cs, rho = cases[q]
            with Plan(p, cp, cs, rho) as plan:
                for _ in range(4):
                    plan.run(10)
                got[q] = (plan.seismograms(), np.stack([plan.field(c) for c in range(9)]))
        except Exception as e:
            errors.append(repr(e))

    th = [threading.Thread(target=worker, args=(q,)) for q in range(4)]
    for x in th:
        x.start()
    for x in th:
        x.join()
    assert not errors, errors
    for q in range(4):
        assert np.array_equal(got[q][0], want[q][0]) and np.array_equal(got[q][1], want[q][1]), q
