"""Multi-process (gloo, world size 2, CPU) coverage of the rank logic used
when several GPUs split independent shots: the shards partition the shot
list, the barrier and the max/sum reductions agree on every rank."""
import os
import socket

import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, out):
    os.environ.update({"RANK": str(rank), "WORLD_SIZE": str(world), "LOCAL_RANK": str(rank),
                       "MASTER_ADDR": "127.0.0.1", "MASTER_PORT": str(port)})
    from ela3d_gb300 import configs
    from ela3d_gb300.dist import Group, env, shard

    r, w, lr = env()
    g = Group()
    shots, *_ = configs.anticline_256_shots(16, nstep=10, n=64)
    mine = shard(shots, r, w)
    g.barrier()
    cells = g.sum(sum(p.cells for p in mine))
    slowest = g.max(1.0 + r)          # the rank-r "elapsed time"
    out.put((r, [tuple(p.src) for p in mine], cells, slowest))
    g.close()


def test_two_ranks_split_shots_and_reduce():
    import torch.multiprocessing as mp

    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = sorted(q.get(timeout=120) for _ in procs)
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    from ela3d_gb300 import configs

    shots, *_ = configs.anticline_256_shots(16, nstep=10, n=64)
    all_src = [tuple(p.src) for p in shots]
    got = res[0][1] + res[1][1]
    assert sorted(got) == sorted(all_src) and not set(res[0][1]) & set(res[1][1])
    assert res[0][2] == res[1][2] == sum(p.cells for p in shots)
    assert res[0][3] == res[1][3] == 2.0


def test_shard_validation():
    from ela3d_gb300.dist import shard

    assert shard(range(7), 1, 3) == [1, 4]
    with pytest.raises(ValueError):
        shard(range(3), 3, 3)
