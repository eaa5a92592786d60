"""Guard zones (a stand-in for a memory sanitizer, which is closed on this
pool): with ELA3D_GUARD_ZONES set, every array of a shot's device pool is
fenced by zones of a known byte pattern; after runs over odd shapes, every
kernel variant, both source kinds, edge receivers, no-PML and all-PML grids,
no zone may have been written.  A deliberately corrupted zone is caught."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GUARD = "8192"


def shot(nx, ny, nz, npml, src, src_kind=0, sampgat=1, precision=0):
    from ela3d_gb300 import ShotParams, media

    cp, cs, rho = media.anticline_layers(nx, ny, nz, depths=(nz * 0.25, nz * 0.5, nz * 0.75, 3 * nz), amp=2,
                                         sigma=max(2, nx // 4), seed=nx)
    rec = np.array([[0, 0, 0], [nx - 1, ny - 1, nz - 1], [nx - 1, 0, nz // 2], [0, ny - 1, 1]], np.int32)
    p = ShotParams(nx=nx, ny=ny, nz=nz, nstep=36, dt=5e-4, npml=npml, f0=30.0, t0=0.04, src=src,
                   src_kind=src_kind, src_w=(0.4, 0.6, 1.0), rec=rec, sampgat=sampgat, precision=precision,
                   energy_every=12)
    return p, cp, cs, rho


CASES = {
    "odd": dict(nx=37, ny=26, nz=22, npml=4, src=(18, 12, 10)),
    "corner_force": dict(nx=33, ny=20, nz=18, npml=3, src=(0, 19, 0)),
    "corner_explosive": dict(nx=33, ny=20, nz=18, npml=3, src=(32, 0, 17), src_kind=1),
    "no_pml": dict(nx=29, ny=31, nz=13, npml=0, src=(14, 15, 6), sampgat=3),
    "all_pml": dict(nx=20, ny=20, nz=20, npml=9, src=(10, 10, 10)),
    "thin_z": dict(nx=40, ny=24, nz=3, npml=1, src=(20, 12, 1)),
}


@pytest.mark.parametrize("name", sorted(CASES))
def test_no_write_leaves_its_array(built, monkeypatch, name):
    import ela3d_gb300 as E

    monkeypatch.setenv("ELA3D_GUARD_ZONES", GUARD)
    for i, v in enumerate(E.variants()):
        if v.fp64 and i != next(j for j, w in enumerate(E.variants()) if w.fp64):
            continue   # every FP32 variant and the FP64 default
        p, cp, cs, rho = shot(**CASES[name], precision=int(v.fp64))
        with E.Plan(p, cp, cs, rho, variant=i) as plan:
            plan.run(p.nstep)
            plan.check_guards()


def test_corrupted_guard_is_reported(built, monkeypatch):
    import ela3d_gb300 as E

    monkeypatch.setenv("ELA3D_GUARD_ZONES", GUARD)
    p, cp, cs, rho = shot(**CASES["odd"])
    with E.Plan(p, cp, cs, rho) as plan:
        plan.run(4)
        plan.check_guards()
        ck = plan.checkpoint()
        ck[-1] ^= 0xFF          # the pool image ends with the last array's guard zone
        plan.restore(ck)
        with pytest.raises(E.Ela3dError) as e:
            plan.check_guards()
        assert e.value.status == 11 and "source trace" in str(e.value)
