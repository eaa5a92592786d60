"""Padding poison: NaN written into every padding column (x >= nx of the
padded rows) of the fields and C-PML memory variables never reaches a grid
cell -- the tensor maps end at nx, so the stencils' loads fill zeros there
(the cp.async copies zero-fill from nx on as well) -- and the results are
bit-identical to an unpoisoned run."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def pick(kind):
    """Index of a compiled variant: the default FP32 tile, the 64-wide FP32
    tile, the FP32 tile filled by cp.async instead of TMA, the first FP64."""
    import ela3d_gb300 as E

    for i, v in enumerate(E.variants()):
        if ((kind == "fp32" and not v.fp64 and v.loads == 0) or (kind == "fp32_64" and not v.fp64 and v.tile_x == 64)
                or (kind == "cp_async" and v.loads == 1) or (kind == "fp64" and v.fp64)):
            return i
    raise LookupError(kind)


@pytest.mark.parametrize("nx,kind", [(37, "fp32"), (45, "fp32_64"), (41, "cp_async"), (29, "fp64")])
def test_nan_padding_never_reaches_the_grid(built, nx, kind):
    import ela3d_gb300 as E
    from ela3d_gb300 import Plan, ShotParams, media

    variant = pick(kind)
    ny, nz = 26, 22
    cp, cs, rho = media.anticline_layers(nx, ny, nz, depths=(5, 11, 17, 40), amp=2, sigma=6, seed=7)
    fp64 = E.variants()[variant].fp64
    p = ShotParams(nx=nx, ny=ny, nz=nz, nstep=50, dt=1e-3, npml=4, f0=30.0, t0=0.04, src=(nx // 2, 12, 10),
                   rec=np.array([[1, 2, 3], [nx - 1, 20, 10], [nx - 2, 5, 21]], np.int32), precision=int(fp64))

    def run(poison):
        with Plan(p, cp, cs, rho, variant=variant) as plan:
            if poison:
                plan.poison_padding(float("nan"))
            plan.run(p.nstep)
            return plan.seismograms(fp64=fp64), np.stack([plan.field(c, fp64=fp64) for c in range(9)])

    s0, f0 = run(False)
    s1, f1 = run(True)
    assert np.all(np.isfinite(s1)) and np.all(np.isfinite(f1))
    assert np.array_equal(s0, s1) and np.array_equal(f0, f1)
