"""Several GPUs as replicas.

One relaxation fits one GB300 (256x256x512 in FP32 is about 4 GB), so the
relaxation itself is not split across GPUs.  Under torchrun every rank runs
its own work with no exchange on the data path:
- the single-case bench: one independent relaxation per rank;
- the batched bench: the cases whose index is the rank modulo the world size.

Only the timing is combined, on the host after each timed region.  The job
takes as long as the slowest rank (max), and its work is the sum over ranks.
The helpers work on any process group: NCCL on GPUs, gloo in the CPU tests.
"""
from __future__ import annotations

import os


def init(backend: str | None = None):
    """(dist, rank, world_size), joining the process group when WORLD_SIZE > 1
    (RANK, WORLD_SIZE, MASTER_ADDR and MASTER_PORT from the environment, as
    torchrun sets them).  dist is None for a single process."""
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if ws <= 1:
        return None, rank, ws
    import torch.distributed as dist
    if not dist.is_initialized():
        dist.init_process_group(backend or "nccl")
    return dist, dist.get_rank(), dist.get_world_size()


def _reduce(dist, value: float, op_name: str) -> float:
    if dist is None:
        return float(value)
    import torch
    device = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=getattr(dist.ReduceOp, op_name))
    return float(t.item())


def max_over_ranks(dist, value: float) -> float:
    """The largest value over all ranks (a time: the slowest rank's)."""
    return _reduce(dist, value, "MAX")


def sum_over_ranks(dist, value: float) -> float:
    """The sum over all ranks (work done)."""
    return _reduce(dist, value, "SUM")


def gather_lists(dist, values: list) -> list:
    """The concatenation of every rank's list, in rank order (per-case
    timings of the batched cases, for percentiles over the whole job)."""
    if dist is None:
        return list(values)
    parts = [None] * dist.get_world_size()
    dist.all_gather_object(parts, list(values))
    return [v for part in parts for v in part]


def shard(n: int, rank: int, world_size: int) -> list[int]:
    """The indices of n independent cases that this rank runs: i with
    i mod world_size == rank.  Every case runs on exactly one rank."""
    if world_size < 1 or not 0 <= rank < world_size:
        raise ValueError(f"rank {rank} outside a world of {world_size}")
    return list(range(rank, n, world_size))
