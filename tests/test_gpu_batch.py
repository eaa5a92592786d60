"""Batched shots: every shot's result equals the same shot run alone.

The per-cell arithmetic does not depend on how work is split, so a shot in
a batch (any mix of sizes, models, sources, receivers and lengths, any
schedule) must reproduce its single-shot result bit for bit; CUDA-graph
replay must reproduce direct launches bit for bit."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def shots():
    from ela3d_gb300 import PML_CLEAN, ShotParams, media

    out = []
    shared = media.anticline_layers(48, 40, 36, depths=(9, 18, 27, 80), amp=3, sigma=10, seed=1)
    for q, (sx, sy) in enumerate([(12, 10), (30, 25), (24, 20)]):
        rec = np.array([[x, sy, 12] for x in range(2, 46, 4)], np.int32)
        p = ShotParams(nx=48, ny=40, nz=36, nstep=90 + 17 * q, dt=1e-3, npml=6, f0=20.0, t0=0.06,
                       src=(sx, sy, 10), rec=rec, pml_mode=q % 2)
        out.append((p,) + shared)
    other = media.anticline_layers(33, 57, 29, depths=(7, 14, 21, 60), amp=2, sigma=8, seed=2)
    rec = np.array([[x, 30, 8] for x in range(1, 32, 3)], np.int32)
    out.append((ShotParams(nx=33, ny=57, nz=29, nstep=75, dt=8e-4, npml=5, f0=25.0, t0=0.05,
                           src=(16, 28, 9), rec=rec, stf=1, src_kind=1, pml_mode=PML_CLEAN),) + other)
    return out


def alone(p, cp, cs, rho, variant):
    from ela3d_gb300 import Plan

    with Plan(p, cp, cs, rho, variant=variant) as plan:
        plan.run(p.nstep)
        return plan.seismograms(), np.stack([plan.field(c) for c in range(9)])


@pytest.mark.parametrize("schedule,chunk", [(0, 0), (1, 8), (2, 8)])
def test_batch_equals_alone(built, schedule, chunk):
    from ela3d_gb300 import Batch

    sh = shots()
    want = [alone(*s, variant=0) for s in sh]
    longest = max(s[0].nstep for s in sh)
    with Batch(sh, variant=0, schedule=schedule, chunk=chunk) as b:
        b.run(longest + 5)   # shorter shots retire at their nstep
        for q, (p, *_ ) in enumerate(sh):
            assert b.info(q).step == longest + 5
            assert np.array_equal(b.seismograms(q), want[q][0]), q
            f = np.stack([b.field(q, c) for c in range(9)])
            assert np.array_equal(f, want[q][1]), q


def test_batch_in_pieces_equals_one_run(built):
    from ela3d_gb300 import Batch

    sh = shots()
    longest = max(s[0].nstep for s in sh)
    with Batch(sh, variant=0) as a:
        a.run(longest)
        ref = [a.seismograms(q) for q in range(len(sh))]
    with Batch(sh, variant=0) as b:
        for n in (3, 51, 20, longest):
            b.run(n)
        for q in range(len(sh)):
            assert np.array_equal(b.seismograms(q), ref[q])


def test_graph_replay_equals_direct_launches(built):
    """Runs of 50+ steps of the two half-step kernels replay a captured
    graph; with kernel timing on the same steps launch directly."""
    from ela3d_gb300 import Plan

    p, cp, cs, rho = shots()[0]
    p = p.with_(nstep=173)
    with Plan(p, cp, cs, rho, schedule=1, chunk=8) as g:
        g.run(173)
        sg = g.seismograms()
        fg = g.field(2)
    with Plan(p, cp, cs, rho, schedule=1, chunk=8) as d:
        d.set_kernel_timing(True)
        d.run(173)
        sd = d.seismograms()
        fd = d.field(2)
        _, _, ns, nv = d.kernel_timing()
    assert ns == 173 and nv == 173
    assert np.array_equal(sg, sd) and np.array_equal(fg, fd)
