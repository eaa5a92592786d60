"""Page-locked host buffers (ela3d_host_alloc / ela3d_host_free): a plan
created from model arrays in them, and seismograms read into one, give the
same bits as from ordinary numpy arrays."""
import gc

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_pinned_inputs_and_readback_equal_pageable(built):
    import ela3d_gb300 as E
    from ela3d_gb300 import ShotParams, media

    nx, ny, nz = 60, 48, 40
    rec = np.array([[x, 20, 12] for x in range(2, nx - 2, 4)], np.int32)
    p = ShotParams(nx=nx, ny=ny, nz=nz, nstep=80, dt=1e-3, npml=6, f0=20.0, t0=0.06, src=(30, 24, 12), rec=rec)
    cp, cs, rho = media.anticline_layers(nx, ny, nz, depths=(10, 20, 30, 80), amp=3, sigma=9, seed=2)
    with E.Plan(p, cp, cs, rho) as plan:
        plan.run(p.nstep)
        want = plan.seismograms()
    host = [E.pinned_copy(a, np.float32) for a in (cp, cs, rho)]
    assert all(np.array_equal(h, a) for h, a in zip(host, (cp, cs, rho)))
    out = E.pinned_empty((p.nrec, 3, p.nsamp), np.float32)
    with E.Plan(p, *host) as plan:
        plan.run(p.nstep)
        got = plan.seismograms(out=out)
    assert got is out and np.abs(want).max() > 0
    assert np.array_equal(out, want)
    with E.Plan(p, cp, cs, rho) as plan:
        with pytest.raises(ValueError):
            plan.seismograms(out=np.zeros((p.nrec, 3, p.nsamp), np.float64))
    # views keep the buffer alive; dropping every view frees it
    view = host[0][1:]
    del host
    gc.collect()
    assert view.shape == (nz - 1, ny, nx) and np.array_equal(view, cp[1:])
    del view
    gc.collect()
