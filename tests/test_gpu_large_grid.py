"""A grid of more than 2^31 cells: every array's element index passes the
32-bit range (1024 x 1024 x 2112 = 2.21e9 cells, 106 GB of FP32 fields and
model on the device, generated there).  The source sits in plane 2052, so
its wavefield straddles plane 2048, the first whose cells lie beyond index
2^31.  After 10 steps the wave has not reached any C-PML layer, and cells
outside the layers update with a = 0 and 1/K = 1, where the memory-variable
terms are exact no-ops: the receivers around the source must then equal,
bit for bit, the same source in a 112^3 grid, whatever the tile each cell
falls in.  The reference indexes with int and stops at 2^31 cells."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

CP, RHO = 3300.0, 2800.0
STEPS = 10
OFFS = (-6, -3, 0, 3, 6)


def shot(shape, src):
    from ela3d_gb300 import ShotParams

    nx, ny, nz = shape
    rec = np.array([[src[0] + a, src[1] + b, src[2] + c] for a in OFFS for b in OFFS for c in OFFS], np.int32)
    return ShotParams(nx=nx, ny=ny, nz=nz, nstep=STEPS, dt=1.6e-3, npml=10, f0=7.0, t0=1.2 / 7.0,
                      src=src, rec=rec, sampgat=1)


def run(shape, src):
    from ela3d_gb300 import Plan
    from ela3d_gb300._abi import Ela3dError

    spec = {"kind": 0, "cp0": CP, "cs0": CP / 1.732, "rho0": RHO}
    try:
        plan = Plan.from_model(shot(shape, src), spec)
    except Ela3dError as e:
        if e.status == 2:  # ELA3D_ERR_OOM: the device is shared or smaller
            pytest.skip(f"not enough device memory for {shape}: {e}")
        raise
    with plan:
        plan.run(STEPS)
        return plan.seismograms(), plan.energy()


def test_grid_beyond_int32_cells_matches_small_grid(built):
    big, small = (1024, 1024, 2112), (112, 112, 112)
    assert big[0] * big[1] * big[2] > 2**31
    assert 2048 * big[0] * big[1] <= 2**31  # plane 2048 starts at index 2^31
    src_big, src_small = (512, 700, 2052), (56, 56, 56)
    seis_s, e_s = run(small, src_small)
    seis_b, e_b = run(big, src_big)
    assert np.abs(seis_s).max() > 0
    # the receivers in planes 2049-2058 lie beyond index 2^31
    assert np.array_equal(seis_b, seis_s)
    assert e_s > 0 and abs(e_b - e_s) <= 1e-10 * e_s
