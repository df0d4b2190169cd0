"""Host-side logic for running independent problems on several GPUs (replicas, one process per GPU).

The path has no data exchange between problems, so ranks never communicate on the data path: each
rank takes a share of the problems (largest first, by DoF weight), solves it on its own GPU, and the
only collectives are the timing barrier and the max/sum reductions of the reported numbers.
"""
from __future__ import annotations


def partition_by_weight(weights, world_size):
    """Deterministic longest-processing-time split: indices of `weights` per rank, heaviest first,
    each item to the currently lightest rank (ties to the lower rank)."""
    order = sorted(range(len(weights)), key=lambda i: (-weights[i], i))
    load = [0.0] * world_size
    parts = [[] for _ in range(world_size)]
    for i in order:
        r = min(range(world_size), key=lambda k: (load[k], k))
        parts[r].append(i)
        load[r] += weights[i]
    return parts


def _reduce(value, op, device):
    import torch
    import torch.distributed as dist

    if not dist.is_available() or not dist.is_initialized():
        return float(value)
    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=op)
    return float(t.item())


def max_over_ranks(value, device="cpu"):
    import torch.distributed as dist

    return _reduce(value, dist.ReduceOp.MAX, device)


def sum_over_ranks(value, device="cpu"):
    import torch.distributed as dist

    return _reduce(value, dist.ReduceOp.SUM, device)


def whole_job_throughput(local_units, local_ms, device="cpu"):
    """Units processed by all ranks divided by the slowest rank's time (per second)."""
    units = sum_over_ranks(local_units, device)
    ms = max_over_ranks(local_ms, device)
    return units / (ms / 1e3), ms
