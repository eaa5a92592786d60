"""The autotuner: times every variant x schedule on the caller's shots,
returns the fastest, and the tuned plan computes the same bits."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_autotune_picks_a_valid_choice_and_results_do_not_change(built, tmp_path, monkeypatch):
    import ela3d_gb300 as E
    from ela3d_gb300 import configs

    monkeypatch.setenv("ELA3D_TUNE_CACHE", str(tmp_path / "tune.txt"))
    p, cp, cs, rho = configs.anticline_256(nstep=60, n=96)
    best, ms, cand = E.autotune([(p, cp, cs, rho)], steps=5)
    n32 = sum(1 for v in E.variants() if not v.fp64 and v.loads == 0)   # TMA-loaded
    # nine two-kernel and twelve dataflow schedules x two prefetch modes for a
    # single shot, the dataflow schedules again without prefetch, and the
    # built-in choice when it is none of those
    assert cand in (n32 * 54, n32 * 54 + 1)
    assert 0 <= best.variant < len(E.variants()) and not E.variants()[best.variant].fp64
    assert ms > 0
    assert best.prefetch in (0, 2, 6)
    with E.Plan(p, cp, cs, rho, **best.as_dict()) as a:
        a.run(60)
        sa = a.seismograms()
    with E.Plan(p, cp, cs, rho) as b:   # picks the cached choice
        b.run(60)
        sb = b.seismograms()
    assert np.array_equal(sa, sb)


def test_autotune_batch_includes_interleaved_schedules(built):
    import ela3d_gb300 as E
    from ela3d_gb300 import configs

    shots, cp, cs, rho = configs.anticline_256_shots(4, nstep=20, n=64)
    best, ms, cand = E.autotune([(s, cp, cs, rho) for s in shots], steps=3)
    n32 = sum(1 for v in E.variants() if not v.fp64 and v.loads == 0)   # TMA-loaded
    # eleven two-kernel schedules x two prefetch modes for a batch (the
    # dataflow schedules are tried for single shots)
    assert cand == n32 * 22
    assert best.schedule in (0, 1, 2)


CHILD = r"""
import sys
sys.path.insert(0, sys.argv[1])
import numpy as np
from ela3d_gb300 import Plan, ShotParams, media
p = ShotParams(nx=40, ny=36, nz=44, nstep=20, npml=8, src=(20, 18, 20), rec=np.array([[10, 18, 20]], np.int32))
cp, cs, rho = media.anticline_layers(40, 36, 44, depths=(10, 20, 30, 60), amp=4, sigma=8, seed=0)
with Plan(p, cp, cs, rho) as a:
    a.run(p.nstep)
    np.save(sys.argv[2], a.seismograms())
"""


def test_cache_entry_the_library_cannot_run_is_ignored(built, tmp_path):
    """A tuning cache file written by another library (a variant index this
    one lacks, a schedule kind it does not know) counts as a miss: the plan
    is created with the built-in choice instead of failing."""
    import os
    import subprocess
    import sys

    from ela3d_gb300 import Plan, ShotParams, media

    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    cache = tmp_path / "tune.txt"
    cache.write_text("0:1:40x36x44p8*1, 999 1 10 0 6\n")
    prog = tmp_path / "child.py"
    prog.write_text(CHILD)
    out = tmp_path / "seis.npy"
    env = dict(os.environ, ELA3D_TUNE_CACHE=str(cache))
    env.pop("ELA3D_AUTOTUNE", None)
    r = subprocess.run([sys.executable, str(prog), root, str(out)], env=env, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    p = ShotParams(nx=40, ny=36, nz=44, nstep=20, npml=8, src=(20, 18, 20), rec=np.array([[10, 18, 20]], np.int32))
    cp, cs, rho = media.anticline_layers(40, 36, 44, depths=(10, 20, 30, 60), amp=4, sigma=8, seed=0)
    with Plan(p, cp, cs, rho) as a:
        a.run(p.nstep)
        want = a.seismograms()
    assert np.array_equal(np.load(out), want)
    cache.write_text("0:1:40x36x44p8*1, 0 7 10 0 6\n")
    r = subprocess.run([sys.executable, str(prog), root, str(out)], env=env, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert np.array_equal(np.load(out), want)
