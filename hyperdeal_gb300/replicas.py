"""Rank bookkeeping and timing for ``bench.py --gpus N`` (one process per GPU,
launched by torchrun): every rank advances its own part of the problem (a
v-slab of the partitioned operator, hyperdeal_gb300/partition.py, whose ghost
faces it exchanges with its neighbours once per stage); the timed region is
bracketed by a barrier and a device synchronisation on both sides and the
reported time is the maximum over the ranks.

The same helpers run with the ``gloo`` backend and a host clock, which is how
the multi-rank logic is tested without GPUs.
"""
from __future__ import annotations

import os
import time
from typing import Callable, Optional


class Replicas:
    """Rank/world from the torchrun environment; ``dist`` is None for one process."""

    def __init__(self, backend: str = "nccl"):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local_rank = int(os.environ.get("LOCAL_RANK", "0"))
        self.dist = None
        self.backend = backend
        if self.world > 1:
            import torch.distributed as dist
            if not dist.is_initialized():
                dist.init_process_group(backend)
            self.dist = dist

    def barrier(self) -> None:
        if self.dist is not None:
            self.dist.barrier()

    def max_over_ranks(self, value: float) -> float:
        if self.dist is None:
            return float(value)
        import torch
        dev = "cuda" if self.backend == "nccl" else "cpu"
        t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def close(self) -> None:
        if self.dist is not None:
            self.dist.destroy_process_group()
            self.dist = None


def time_steps(rep: Replicas, step: Callable[[], None], steps: int, warmup: int,
               sync: Callable[[], None], clock: Optional[Callable[[], tuple]] = None) -> float:
    """Run `warmup` untimed steps, then `steps` timed ones between barriers and
    synchronisations; returns the time per step (ms), the maximum over ranks.
    `clock()` returns (start, stop) callables of a timer in ms (default: host
    clock; bench.py passes CUDA events on the launching stream)."""
    for _ in range(warmup):
        step()
    sync()
    rep.barrier()
    if clock is None:
        t = {}

        def start():
            t["a"] = time.perf_counter()

        def stop():
            return (time.perf_counter() - t["a"]) * 1e3
    else:
        start, stop = clock()
    sync()
    rep.barrier()
    start()
    for _ in range(steps):
        step()
    ms = stop()
    sync()
    return rep.max_over_ranks(ms) / steps


def whole_job_rate(units_per_rank_step: float, world: int, ms_per_step: float) -> float:
    """Units of all ranks per second (weak scaling: every rank does the same work)."""
    return units_per_rank_step * world / (ms_per_step / 1e3)
