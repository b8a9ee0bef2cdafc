"""Weak scaling over GPUs: one process per GPU, each integrating its own cells.

Grid cells are independent, so N ranks need no data exchange: rank r takes
its own block of cells (seeded workload ``SEED + r`` in the benchmark, or a
host model's own decomposition) and runs the single-GPU path on it.  The only
collectives are a barrier around the timed region and the reductions of the
timing and of the processed units, which give the whole-job throughput
``sum of units / max of times``.

The reductions use the process group's backend: CUDA tensors under NCCL,
host tensors under gloo (used by the CPU tests).
"""

from __future__ import annotations

import os
from dataclasses import dataclass


@dataclass(frozen=True)
class RankEnv:
    world: int
    rank: int
    local: int


def rank_env() -> RankEnv:
    """World size, rank and local rank from the torchrun environment."""
    return RankEnv(int(os.environ.get("WORLD_SIZE", "1")), int(os.environ.get("RANK", "0")),
                   int(os.environ.get("LOCAL_RANK", "0")))


def init(env: RankEnv, backend: str) -> None:
    """Join the process group (rendezvous from MASTER_ADDR / MASTER_PORT)."""
    if env.world > 1:
        import torch.distributed as dist

        dist.init_process_group(backend)


def shard_seed(base: int, rank: int) -> int:
    """Seed of rank `rank`'s cells: every rank draws different cells."""
    return base + rank


def cell_block(total: int, world: int, rank: int) -> tuple[int, int]:
    """[begin, end) of rank `rank`'s share of `total` cells (contiguous blocks,
    sizes differing by at most one)."""
    q, r = divmod(total, world)
    begin = rank * q + min(rank, r)
    return begin, begin + q + (rank < r)


def _reduce(x: float, op: str) -> float:
    import torch
    import torch.distributed as dist

    if not (dist.is_available() and dist.is_initialized()) or dist.get_world_size() == 1:
        return float(x)
    device = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX if op == "max" else dist.ReduceOp.SUM)
    return float(t.item())


def max_over_ranks(x: float) -> float:
    return _reduce(x, "max")


def sum_over_ranks(x: float) -> float:
    return _reduce(x, "sum")


def barrier() -> None:
    import torch.distributed as dist

    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        dist.barrier()


def job_throughput(units_this_rank: float, seconds_this_rank: float) -> tuple[float, float, float]:
    """(units of all ranks, slowest rank's seconds, units / second)."""
    units = sum_over_ranks(units_this_rank)
    seconds = max_over_ranks(seconds_this_rank)
    return units, seconds, units / seconds
