"""One process per GPU: shot sharding and rank-level reductions.

Shots are independent, so several GPUs split a set of shots with no
data-path collective: rank r of W takes shots r, r+W, r+2W, ...  The only
communication is control: a barrier before and after a timed region and
max/sum reductions of scalars (elapsed time, counts), done over
torch.distributed (gloo on CPU tensors, so the same code runs without GPUs).
Launch with torchrun; RANK, WORLD_SIZE, LOCAL_RANK and MASTER_ADDR/PORT come
from the environment.
"""
from __future__ import annotations

import os


def env() -> tuple[int, int, int]:
    """(rank, world size, local rank) from the launcher's environment."""
    return (int(os.environ.get("RANK", "0")), int(os.environ.get("WORLD_SIZE", "1")),
            int(os.environ.get("LOCAL_RANK", "0")))


def shard(seq, rank: int, world: int) -> list:
    """The items of `seq` this rank runs (round-robin, so sizes balance)."""
    if world < 1 or not 0 <= rank < world:
        raise ValueError("bad rank/world")
    return list(seq)[rank::world]


class Group:
    """Barrier and scalar reductions across ranks (no-ops for one rank)."""

    def __init__(self, world: int | None = None, backend: str = "gloo"):
        self.world = env()[1] if world is None else world
        self._d = None
        if self.world > 1:
            import torch.distributed as d

            if not d.is_initialized():
                d.init_process_group(backend=backend)
            self._d = d

    def barrier(self) -> None:
        if self._d:
            self._d.barrier()

    def _reduce(self, v: float, op) -> float:
        import torch

        t = torch.tensor([float(v)], dtype=torch.float64)
        self._d.all_reduce(t, op=op)
        return float(t.item())

    def max(self, v: float) -> float:
        return self._reduce(v, self._d.ReduceOp.MAX) if self._d else float(v)

    def sum(self, v: float) -> float:
        return self._reduce(v, self._d.ReduceOp.SUM) if self._d else float(v)

    def close(self) -> None:
        if self._d and self._d.is_initialized():
            self._d.destroy_process_group()
