"""Independent replicas across processes (one per GPU).

The path shards only as independent runs: configurations, seeds or pulses
have no data to exchange, so N GPUs run N replicas and no collective touches
the data path. What the processes share is the timing: every rank times its
own run, the job's time is the slowest rank's, and the job's throughput is
all ranks' work over that time ("weak" scaling, fixed work per GPU).

Works with any torch.distributed backend: NCCL between GPUs, gloo on CPU
(the tests).
"""

from __future__ import annotations


def replica_seed(base_seed: int, rank: int) -> int:
    """Seed of rank ``rank``'s replica: distinct tracks per GPU."""
    return int(base_seed) + int(rank)


def _dist():
    import torch.distributed as dist

    return dist if dist.is_available() and dist.is_initialized() else None


def max_over_ranks(value: float) -> float:
    """The largest ``value`` over all ranks (the value itself without a
    process group)."""
    dist = _dist()
    if dist is None or dist.get_world_size() == 1:
        return float(value)
    import torch

    device = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def sum_over_ranks(value: float) -> float:
    """The sum of ``value`` over all ranks."""
    dist = _dist()
    if dist is None or dist.get_world_size() == 1:
        return float(value)
    import torch

    device = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(t.item())


def whole_job_rate(units: float, seconds: float) -> float:
    """All ranks' units of work per second of the slowest rank: each rank
    passes its own units and its own time."""
    return sum_over_ranks(units) / max_over_ranks(seconds)
