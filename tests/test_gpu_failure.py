"""Failure detection on the GPU without faulting it: the FP64 energy
monitor flags an unstable run, and a kernel whose bounded waits expire
reports ELA3D_ERR_TIMEOUT while the context stays usable."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def case(**kw):
    from ela3d_gb300 import ShotParams, media

    n = 48
    p = ShotParams(nx=n, ny=n, nz=n, nstep=400, dt=1e-3, npml=8, f0=20.0, t0=0.06, src=(24, 24, 24),
                   rec=np.array([[30, 24, 24]], np.int32))
    p = p.with_(**kw)
    return (p,) + media.homogeneous(n, n, n, 3000.0, 1700.0, 2200.0)


def test_energy_monitor_passes_stable_run(built):
    from ela3d_gb300 import Plan

    p, cp, cs, rho = case(energy_every=50)
    with Plan(p, cp, cs, rho) as plan:
        plan.run(400)


def test_energy_monitor_flags_cfl_violation(built):
    from ela3d_gb300 import Ela3dError, Plan

    # Courant number 3000 * 4e-3 * sqrt(3) / 10 = 2.1 > 1: unstable
    p, cp, cs, rho = case(dt=4e-3, t0=0.06, energy_every=20, nstep=400)
    with Plan(p, cp, cs, rho) as plan:
        with pytest.raises(Ela3dError) as e:
            plan.run(400)
    assert e.value.status == 4  # ELA3D_ERR_UNSTABLE


def test_timeout_path_reports_and_context_survives(built):
    from ela3d_gb300 import Ela3dError, Plan

    p, cp, cs, rho = case(nstep=20)
    with Plan(p, cp, cs, rho) as plan:
        plan.run(5)
        plan.inject_timeout(1)
        with pytest.raises(Ela3dError) as e:
            plan.run(1)
        assert e.value.status == 5  # ELA3D_ERR_TIMEOUT
        plan.run(2)   # the plan keeps working (its state is partly updated)
    # a fresh plan on the same context computes the same answer as before
    with Plan(p, cp, cs, rho) as a:
        a.run(20)
        sa = a.seismograms()
    with Plan(p, cp, cs, rho) as b:
        b.run(20)
        sb = b.seismograms()
    assert np.array_equal(sa, sb) and np.any(sa)
