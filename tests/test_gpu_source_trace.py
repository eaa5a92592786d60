"""The source-point trace (the reference FP64 GPU program's recsrc?.txt):
after each step's injection, the components the source acts on at its cell.
It must equal the fields read back at the source cell (bit for bit) and the
oracle's fields there (FP32 tolerance)."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def small(kind: int):
    from ela3d_gb300 import ShotParams, media
    from ela3d_gb300.params import SRC_EXPLOSIVE, SRC_FORCE, STF_GAUSS_DERIV, STF_RICKER

    nx, ny, nz = 30, 28, 26
    cp, cs, rho = media.anticline_layers(nx, ny, nz, depths=(6, 12, 18, 40), amp=2, sigma=7, seed=3)
    p = ShotParams(nx=nx, ny=ny, nz=nz, nstep=24, dt=1e-3, npml=4, f0=30.0, t0=0.04, src=(13, 12, 11),
                   src_kind=SRC_EXPLOSIVE if kind else SRC_FORCE, stf=STF_GAUSS_DERIV if kind else STF_RICKER,
                   angle_force=30.0, src_w=(0.3, 0.5, 1.0), rec=np.array([[5, 6, 7]], np.int32))
    return p, cp, cs, rho


@pytest.mark.parametrize("kind", [0, 1], ids=["force", "explosive"])
def test_trace_equals_source_cell_fields(built, kind):
    import oracle
    from ela3d_gb300 import Plan

    p, cp, cs, rho = small(kind)
    comps = (3, 4, 5) if kind else (0, 1, 2)
    i, j, k = p.src
    with Plan(p, cp, cs, rho) as plan:
        seen = []
        for step in range(1, p.nstep + 1):
            plan.run(1)
            seen.append([plan.field(c)[k, j, i] for c in comps])
        tr = plan.source_trace()
    assert tr.shape == (3, p.nstep + 1)
    assert np.all(tr[:, 0] == 0)
    assert np.array_equal(tr[:, 1:], np.array(seen, np.float32).T)
    for n in (3, 11, p.nstep):
        _, f = oracle.run(p, cp, cs, rho, nsteps=n)
        want = np.array([f[c][k, j, i] for c in comps])
        assert np.allclose(tr[:, n], want, rtol=1e-4, atol=1e-6 * np.abs(want).max()), (n, tr[:, n], want)


def test_batch_trace_equals_plan_trace(built):
    from ela3d_gb300 import Batch, Plan

    p, cp, cs, rho = small(1)
    q = p.with_(src=(9, 14, 8), nstep=17)
    with Plan(p, cp, cs, rho) as a:
        a.run(p.nstep)
        ta = a.source_trace()
    with Batch([(p, cp, cs, rho), (q, cp, cs, rho)]) as b:
        b.run(p.nstep)
        tb0, tb1 = b.source_trace(0), b.source_trace(1)
    assert np.array_equal(ta, tb0)
    assert tb1.shape == (3, q.nstep + 1) and np.all(tb1[:, 0] == 0) and np.any(tb1[:, 1:] != 0)
