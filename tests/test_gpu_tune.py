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
    n32 = sum(1 for v in E.variants() if not v.fp64)
    assert cand == n32 * 14         # seven schedules x two prefetch modes for a single shot
    assert 0 <= best.variant < len(E.variants()) and not E.variants()[best.variant].fp64
    assert ms > 0
    assert best.prefetch in (2, 6)
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
    n32 = sum(1 for v in E.variants() if not v.fp64)
    assert cand == n32 * 18         # nine schedules x two prefetch modes for a batch
    assert best.schedule in (0, 1, 2)
