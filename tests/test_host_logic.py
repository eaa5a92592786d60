"""Host-side planning logic of the engine, exercised through the C ABI
without a GPU: C-PML slab sizing and the work schedule."""
import numpy as np
import pytest


def test_slab_extent_basic(built):
    from ela3d_gb300._abi import slab_extent

    z = np.zeros(20)
    assert slab_extent(z, z) == (0, 20)          # no layer: nothing stored
    a = z.copy(); a[:3] = 1; a[-4:] = 1
    assert slab_extent(a, z) == (3, 16)
    h = z.copy(); h[:2] = 1; h[-5:] = 1
    assert slab_extent(a, h) == (3, 15)
    # activity at the middle cell widens the upper slab down to it
    m = a.copy(); m[10] = 1
    assert slab_extent(m, z) == (3, 10)
    # activity on both sides of the middle leaves no gap: all stored
    m[9] = 1
    assert slab_extent(m, z) == (20, 20)
    # a layer covering everything
    assert slab_extent(np.ones(7), np.ones(7)) == (7, 7)


@pytest.mark.parametrize("mode", [0, 1])
@pytest.mark.parametrize("shape,npml", [((101, 101, 101), 10), ((256, 200, 64), 16), ((40, 33, 27), 6)])
def test_slab_covers_every_nonzero_memory_variable(built, mode, shape, npml):
    """Cells outside the stored slabs must have a = 0 in both profiles, so
    the reference's memory variables stay exactly 0 there (oracle profiles)."""
    import oracle
    from ela3d_gb300 import ShotParams
    from ela3d_gb300._abi import slab_extent

    nx, ny, nz = shape
    p = ShotParams(nx=nx, ny=ny, nz=nz, npml=npml, pml_mode=mode, src=(nx // 2, ny // 2, nz // 2))
    prof = oracle.profiles(p, fp64=True)
    for ax, n in (("x", nx), ("y", ny), ("z", nz)):
        a, ah = prof[f"a_{ax}"], prof[f"a_half_{ax}"]
        lo, hi = slab_extent(a, ah)
        assert np.all(a[lo:hi] == 0) and np.all(ah[lo:hi] == 0)
        active = np.nonzero((a != 0) | (ah != 0))[0]
        assert len(active) > 0
        # tight: the extents touch active cells on both sides
        assert lo == active[active < n // 2].max() + 1
        assert hi == active[active >= n // 2].min()
    if mode == 0:
        # the reference's zmin half-node test never fires (stale y abscissa)
        assert np.all(prof["a_half_z"][: nz // 2] == 0)
        # and a_x_half is never assigned
        assert np.all(prof["a_half_x"] == 0)


@pytest.mark.parametrize("kind,chunk", [(0, 0), (1, 5), (1, 16), (1, 1000)])
@pytest.mark.parametrize("shape,tile", [((256, 256, 256), (128, 7)), ((101, 101, 101), (64, 6)),
                                         ((37, 29, 31), (128, 3)), ((300, 64, 17), (64, 14))])
@pytest.mark.parametrize("max_blocks", [1, 152, 100000])
def test_schedule_covers_each_plane_of_each_tile_once(built, kind, chunk, shape, tile, max_blocks):
    from ela3d_gb300._abi import schedule

    nx, ny, nz = shape
    tx, ty = tile
    items, first = schedule(nx, ny, nz, tx, ty, kind, chunk, max_blocks)
    ntiles = -(-nx // tx) * -(-ny // ty)
    assert len(first) - 1 <= max_blocks
    assert first[0] == 0 and first[-1] == len(items) and np.all(np.diff(first) >= 1)
    assert np.all(items[:, 1] < items[:, 2])
    count = np.zeros((ntiles, nz), np.int32)
    for t, k0, k1 in items:
        count[t, k0:k1] += 1
    assert np.all(count == 1)
    if kind == 0:
        per_block = [int((items[first[b]:first[b + 1], 2] - items[first[b]:first[b + 1], 1]).sum())
                     for b in range(len(first) - 1)]
        assert max(per_block) - min(per_block) <= 1


def test_bytes_per_cell_definition():
    from ela3d_gb300.metrics import bytes_per_cell

    assert bytes_per_cell(101, 101, 101, 10)["step"] == pytest.approx(152.5, abs=0.05)
    assert bytes_per_cell(256, 256, 256, 16)["step"] == pytest.approx(142.0)
    assert bytes_per_cell(256, 256, 256, 0)["step"] == 124.0
    assert bytes_per_cell(256, 256, 256, 16, word=8)["step"] == 284.0
