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


def _flow_deps(item, J, txs, tys):
    """The items a dataflow item waits for, restated independently of the
    library: stress (chunk j, tile t, step r) reads the velocities written by
    velocity chunks j and j+1 of step r-1 on t and its four neighbours (and
    overwrites the stresses they read); velocity (j, t, r) reads the
    stresses of stress chunks j-1 and j of step r there."""
    kind, step, chunk, tile = (int(v) for v in item[:4])
    tx, ty = tile % txs, tile // txs
    r = step - 1 if kind == 0 else step
    if r < 0:
        return []
    chunks = [chunk, chunk + 1] if kind == 0 else [chunk, chunk - 1]
    out = []
    for x, y in ((tx, ty), (tx - 1, ty), (tx + 1, ty), (tx, ty - 1), (tx, ty + 1)):
        if 0 <= x < txs and 0 <= y < tys:
            for c in chunks:
                if 0 <= c < J:
                    out.append((1 - kind, r, c, y * txs + x))
    return out


@pytest.mark.parametrize("shape,tile,chunk,gap,overlap", [((101, 101, 101), (128, 7), 8, 152, False),
                                                          ((101, 101, 101), (128, 7), 8, 152, True),
                                                          ((70, 45, 33), (64, 14), 5, 3, True),
                                                          ((40, 30, 9), (128, 3), 2, 1, False),
                                                          ((40, 30, 9), (128, 3), 16, 40, True),
                                                          # keys too sparse for the counting sort: the
                                                          # comparison-sort path
                                                          ((40, 30, 9), (128, 3), 2, 100000, False)])
def test_flow_schedule_covers_every_update_once_in_dependency_order(built, shape, tile, chunk, gap, overlap):
    from ela3d_gb300._abi import flow_schedule

    nx, ny, nz = shape
    K = 4
    items = flow_schedule(nx, ny, nz, tile[0], tile[1], chunk, gap, overlap, K)
    txs, tys = -(-nx // tile[0]), -(-ny // tile[1])
    J = -(-nz // chunk)
    keys = [tuple(int(v) for v in it[:4]) for it in items]
    assert len(set(keys)) == len(keys) == K * 2 * J * txs * tys
    pos = {k: q for q, k in enumerate(keys)}
    # every cell plane is updated exactly once per half-step and step
    for kind in (0, 1):
        for r in range(K):
            for t in range(txs * tys):
                cover = np.zeros(nz, np.int32)
                for it in items:
                    if it[0] == kind and it[1] == r and it[3] == t:
                        cover[it[4]:it[5]] += 1
                assert np.all(cover == 1)
    # velocity chunks sit one plane below the stress chunks
    for it in items:
        kind, _, j, _, k0, k1 = (int(v) for v in it)
        if kind == 0:
            assert (k0, k1) == (j * chunk, min((j + 1) * chunk, nz))
        else:
            assert k0 == max(j * chunk - 1, 0) and k1 == (nz if j == J - 1 else (j + 1) * chunk - 1)
    for q, it in enumerate(items):
        for d in _flow_deps(it, J, txs, tys):
            assert pos[d] < q, (it, d)
    # steps overlap only when asked to (and then they do, on deep grids)
    first_of = {r: min(q for q, k in enumerate(keys) if k[1] == r) for r in range(K)}
    last_of = {r: max(q for q, k in enumerate(keys) if k[1] == r) for r in range(K)}
    overlapped = any(first_of[r + 1] < last_of[r] for r in range(K - 1))
    if not overlap:
        assert not overlapped
    elif J >= 4:
        assert overlapped


@pytest.mark.parametrize("chunk,gap,steps", [(1, 10, 2), (4, 0, 2), (0, 5, 2), (4, 10, 0), (4, 10, 256)])
def test_flow_schedule_rejects_bad_arguments(built, chunk, gap, steps):
    from ela3d_gb300 import Ela3dError
    from ela3d_gb300._abi import flow_schedule

    with pytest.raises(Ela3dError):
        flow_schedule(40, 40, 40, 128, 7, chunk, gap, False, steps)


def test_builtin_tuning_by_size():
    """The built-in choice (ela3d_builtin_tuning, 152 SMs without a device):
    the dataflow kernel with about 1.5 work items per block (three or more
    z-chunks per tile column while the columns are fewer, whole columns
    beyond); the two kernels for an explosive source and for FP64."""
    import ela3d_gb300 as E
    from ela3d_gb300 import configs

    def pick(p):
        t = E.builtin_tuning(p)
        v = E.variants()[t.variant]
        return (v.tile_x, v.tile_y), t.schedule, t.chunk

    assert pick(configs.homogeneous_101()[0]) == ((112, 8), 4, 6)
    assert pick(configs.anticline_256()[0]) == ((128, 7), 4, 86)
    assert pick(configs.anticline_256(n=192)[0]) == ((112, 8), 4, 39)
    assert pick(configs.anticline_256(n=288)[0]) == ((112, 8), 4, 96)
    assert pick(configs.anticline_256(n=320)[0]) == ((112, 8), 4, 107)   # three chunks per column at least
    assert pick(configs.anticline_256(n=512)[0])[1:] == (4, 512)          # whole columns: 296 tiles
    assert pick(configs.anticline_256()[0].with_(src_kind=E.SRC_EXPLOSIVE))[1:] == (1, 10)
    # memory-variable prefetch: none while the arrays fit in L2, x slab up
    # to about twice that, all slabs beyond
    assert [E.builtin_tuning(p).prefetch for p in (configs.homogeneous_101()[0], configs.anticline_256(n=128)[0],
                                                   configs.anticline_256()[0])] == [0, 2, 6]
    t = E.builtin_tuning(configs.anticline_256(precision=E.FP64)[0])
    assert E.variants()[t.variant].fp64 and t.schedule == 1
