"""Checkpoint / resume: a plan restored from a checkpoint continues exactly
as the saved plan would have (bit for bit), in a fresh plan of the same
parameters; a checkpoint of other parameters (sizes, time step, C-PML
coefficients, source, receivers) is refused."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def case(**kw):
    from ela3d_gb300 import ShotParams, media
    from ela3d_gb300.params import SRC_EXPLOSIVE

    nx, ny, nz = 36, 30, 28
    cp, cs, rho = media.anticline_layers(nx, ny, nz, depths=(7, 14, 21, 60), amp=2, sigma=8, seed=4)
    p = ShotParams(nx=nx, ny=ny, nz=nz, nstep=70, dt=1e-3, npml=5, f0=25.0, t0=0.05, src=(17, 15, 12),
                   src_kind=SRC_EXPLOSIVE, rec=np.array([[5, 6, 7], [20, 22, 9], [30, 3, 20]], np.int32),
                   energy_every=10).with_(**kw)
    return p, cp, cs, rho


def state(plan):
    return plan.seismograms(), np.stack([plan.field(c) for c in range(9)]), plan.source_trace()


@pytest.mark.parametrize("precision", [0, 1])
def test_resume_from_checkpoint_is_bit_identical(built, precision):
    from ela3d_gb300 import Plan

    p, cp, cs, rho = case(precision=precision)
    with Plan(p, cp, cs, rho) as whole:
        whole.run(p.nstep)
        want = state(whole)
    with Plan(p, cp, cs, rho) as a:
        a.run(30)
        ck = a.checkpoint()
        a.run(40)                         # saving does not disturb the run
        for x, y in zip(state(a), want):
            assert np.array_equal(x, y)
    m = np.ones_like(cp)
    with Plan(p, m * 3000, m * 1700, m * 2000) as b:   # the model comes from the checkpoint too
        b.run(5)
        b.restore(ck)
        assert b.info().step == 30
        b.run(40)
        assert b.info().step == 70
        for x, y in zip(state(b), want):
            assert np.array_equal(x, y)


@pytest.mark.parametrize("other", [{"npml": 6}, {"dt": 9e-4}, {"rcoef": 1e-4}, {"src": (16, 15, 12)},
                                   {"f0": 24.0}, {"rec": np.array([[5, 6, 7], [20, 22, 9], [30, 3, 21]], np.int32)}],
                         ids=["npml", "dt", "rcoef", "source", "f0", "receivers"])
def test_checkpoint_of_other_parameters_is_refused(built, other):
    """Sizes, time step, C-PML coefficients, source and receivers must all
    match: the restoring plan recomputes its profiles and source table from
    its own parameters, so any difference would change the continuation."""
    from ela3d_gb300 import Ela3dError, Plan

    p, cp, cs, rho = case()
    with Plan(p, cp, cs, rho) as a:
        a.run(3)
        ck = a.checkpoint()
    q, cq, sq, rq = case(**other)
    with Plan(q, cq, sq, rq) as b:
        with pytest.raises(Ela3dError) as e:
            b.restore(ck)
        assert e.value.status == 1
        bad = ck.copy()
        bad[:8] = 0
        with pytest.raises(Ela3dError):
            b.restore(bad)
        with pytest.raises(Ela3dError):
            b.restore(ck[:16])
