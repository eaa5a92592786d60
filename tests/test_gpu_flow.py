"""The dataflow kernel (schedules 3 and 4): many steps per cooperative
launch, items ordered by device-side completion counters.  The per-cell
arithmetic is the two half-step kernels' own, so every result must equal
the two-kernel path bit for bit: any chunk size, gap, overlapping steps or
not, tile variant, precision, launch split, batch composition, and run
after run (a missing or misplaced dependency would show up as a
difference)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _shot(nx=70, ny=45, nz=33, npml=6, nstep=120, **kw):
    from ela3d_gb300 import ShotParams, media

    rec = np.array([[x, ny // 2, nz // 3] for x in range(1, nx - 1, 3)] + [[0, 0, 0], [nx - 1, ny - 1, nz - 1]],
                   np.int32)
    p = ShotParams(nx=nx, ny=ny, nz=nz, nstep=nstep, dt=1e-3, npml=npml, f0=22.0, t0=0.055,
                   src=(nx // 2, ny // 2, nz // 3), rec=rec, **kw)
    cp, cs, rho = media.anticline_layers(nx, ny, nz, depths=(nz * 0.3, nz * 0.55, nz * 0.8, 3 * nz), amp=3,
                                         sigma=9, seed=4)
    return p, cp, cs, rho


def _run(p, cp, cs, rho, steps=None, **tune):
    from ela3d_gb300 import Plan

    with Plan(p, cp, cs, rho, **tune) as plan:
        if steps is None:
            plan.run(p.nstep)
        else:
            for s in steps:
                plan.run(s)
        fp64 = p.precision == 1
        return (plan.seismograms(fp64=fp64), np.stack([plan.field(c, fp64=fp64) for c in range(9)]),
                plan.source_trace(fp64=fp64))


def _same(a, b):
    return all(np.array_equal(x, y) for x, y in zip(a, b))


def _variant(tx, ty, fp64=False):
    import ela3d_gb300

    return next(i for i, v in enumerate(ela3d_gb300.variants())
                if v.tile_x == tx and v.tile_y == ty and bool(v.fp64) == fp64 and v.loads == 0)


@pytest.mark.parametrize("schedule,chunk,lag", [(3, 2, 0), (3, 5, 0), (4, 8, 0), (4, 5, 3), (3, 33, 0),
                                                (4, 64, 0), (4, 4, 1), (3, 3, 1), (4, 2, 500)])
def test_flow_equals_two_kernels(built, schedule, chunk, lag):
    case = _shot()
    want = _run(*case, variant=0, schedule=1, chunk=8)
    got = _run(*case, variant=0, schedule=schedule, chunk=chunk, lag=lag)
    assert np.abs(want[0]).max() > 0
    assert _same(got, want)


@pytest.mark.parametrize("tile", [(64, 14), (128, 3), (64, 6), (128, 5), (112, 8)])
def test_flow_tile_variants(built, tile):
    case = _shot(nx=83, ny=61, nz=29, npml=7, nstep=70)
    want = _run(*case, variant=0, schedule=1, chunk=8)
    got = _run(*case, variant=_variant(*tile), schedule=4, chunk=4, lag=3)
    assert _same(got, want)


def test_flow_fp64(built):
    from ela3d_gb300 import FP64

    case = _shot(nx=40, ny=34, nz=26, npml=5, nstep=60, precision=FP64)
    want = _run(*case, variant=_variant(32, 7, True), schedule=1, chunk=8)
    got = _run(*case, variant=_variant(32, 7, True), schedule=4, chunk=6, lag=3)
    assert _same(got, want)


def test_flow_launch_splits_and_resume(built):
    """Runs of any length (lists of 50 steps launched whole or in part) and
    resumed runs equal one long run; two identical runs agree exactly."""
    case = _shot(nstep=137)
    ref = _run(*case, variant=0, schedule=4, chunk=6, lag=3)
    assert _same(_run(*case, variant=0, schedule=4, chunk=6, lag=3), ref)
    assert _same(_run(*case, steps=(1, 49, 7, 80), variant=0, schedule=4, chunk=6, lag=3), ref)
    assert _same(_run(*case, variant=0, schedule=1, chunk=8), ref)


def test_flow_edge_cases(built):
    """Smallest grids, a layer covering everything, no layer, a source on the
    corner of the grid."""
    for kw in ({"nx": 3, "ny": 3, "nz": 3, "npml": 0, "nstep": 20},
               {"nx": 5, "ny": 4, "nz": 3, "npml": 1, "nstep": 20},
               {"nx": 24, "ny": 20, "nz": 18, "npml": 12, "nstep": 40},
               {"nx": 36, "ny": 9, "nz": 40, "npml": 0, "nstep": 40}):
        p, cp, cs, rho = _shot(**kw)
        p = p.with_(src=(0, p.ny - 1, 0))
        want = _run(p, cp, cs, rho, variant=0, schedule=1, chunk=8)
        for chunk in (2, 3):
            for sched in (3, 4):
                assert _same(_run(p, cp, cs, rho, variant=0, schedule=sched, chunk=chunk, lag=0), want), (kw, chunk)


def test_flow_batch_equals_alone(built):
    """Shots of different sizes, models and lengths in one dataflow launch;
    shorter shots retire at their nstep."""
    from ela3d_gb300 import Batch

    shots = [_shot(), _shot(nx=51, ny=64, nz=40, nstep=90), _shot(nx=48, ny=40, nz=21, nstep=111)]
    shots[1] = (shots[1][0].with_(pml_mode=1),) + shots[1][1:]
    want = [_run(*s, variant=0, schedule=1, chunk=8) for s in shots]
    longest = max(s[0].nstep for s in shots)
    for sched, lag in ((3, 0), (4, 3)):
        with Batch(shots, variant=0, schedule=sched, chunk=5, lag=lag) as b:
            b.run(longest)
            for q in range(len(shots)):
                assert np.array_equal(b.seismograms(q), want[q][0]), (sched, q)
                f = np.stack([b.field(q, c) for c in range(9)])
                assert np.array_equal(f, want[q][1]), (sched, q)


def test_flow_explosive_source_runs_two_kernels(built):
    """An explosive source (injected between the steps) keeps the two-kernel
    path under schedule 3, with the same results."""
    from ela3d_gb300 import SRC_EXPLOSIVE, STF_GAUSS_DERIV

    p, cp, cs, rho = _shot(nstep=60)
    p = p.with_(src_kind=SRC_EXPLOSIVE, stf=STF_GAUSS_DERIV)
    assert _same(_run(p, cp, cs, rho, variant=0, schedule=3, chunk=5), _run(p, cp, cs, rho, variant=0))


def test_flow_timing_and_launch_count(built):
    """A launch walks its 50-step list up to four times: 450 steps take
    launches of 200, 200 and 50 steps, with the results of 50-step ones."""
    from ela3d_gb300 import Plan

    p, cp, cs, rho = _shot(nstep=450)
    with Plan(p, cp, cs, rho, variant=0, schedule=4, chunk=8) as plan:
        plan.set_kernel_timing(True)
        plan.run(450)
        ms, launches, steps = plan.flow_timing()
        got = (plan.seismograms(), plan.field(2))
    assert launches == 3 and steps == 450 and ms > 0
    with Plan(p, cp, cs, rho, variant=0, schedule=4, chunk=8) as plan:
        for _ in range(9):
            plan.run(50)
        want = (plan.seismograms(), plan.field(2))
    assert all(np.array_equal(a, b) for a, b in zip(got, want))


def test_flow_timeout_path(built):
    """Withheld loads make the dataflow kernel's bounded waits expire: the run
    reports ELA3D_ERR_TIMEOUT and the context keeps working."""
    from ela3d_gb300 import Ela3dError, Plan

    p, cp, cs, rho = _shot(nstep=40)
    with Plan(p, cp, cs, rho, variant=0, schedule=3, chunk=8) as plan:
        plan.inject_timeout(1)
        with pytest.raises(Ela3dError) as e:
            plan.run(10)
        assert e.value.status == 5   # ELA3D_ERR_TIMEOUT
    assert _same(_run(p, cp, cs, rho, variant=0, schedule=3, chunk=8), _run(p, cp, cs, rho, variant=0))


@pytest.mark.parametrize("schedule", [3, 4])
def test_flow_server_mix_equals_alone(built, schedule):
    """A server on the dataflow kernel (its work list rebuilt whenever
    requests join or finish) returns every request's seismograms exactly as
    the request run alone, with late arrivals and a model generated on the
    device."""
    import time

    from ela3d_gb300 import Plan, Server, configs

    reqs = [configs.serving_request(s, t_end=0.12, lo=40, hi=96) for s in range(6)]
    want = []
    for p, cp, cs, rho in reqs:
        with Plan(p, cp, cs, rho, variant=0, schedule=1, chunk=8) as plan:
            plan.run(p.nstep)
            want.append(plan.seismograms())
    gp, spec = configs.serving_request_spec(7, t_end=0.12, lo=40, hi=96)
    with Plan.from_model(gp, spec, variant=0, schedule=1, chunk=8) as plan:
        plan.run(gp.nstep)
        want_gen = plan.seismograms()
    with Server(steps_per_round=29, variant=0, schedule=schedule, chunk=5) as srv:
        tickets = [srv.submit(*reqs[q]) for q in range(3)]
        time.sleep(0.05)
        tickets += [srv.submit(*reqs[q]) for q in range(3, 6)]
        t_gen = srv.submit_model(gp, spec)
        for q, t in enumerate(tickets):
            srv.wait(t)
            assert np.array_equal(srv.read(t), want[q]), q
        srv.wait(t_gen)
        assert np.array_equal(srv.read(t_gen), want_gen)
        assert srv.stats()["failed"] == 0
