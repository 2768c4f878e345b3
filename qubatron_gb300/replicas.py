"""Several GPUs: independent replicas.

The path does not shard: every pixel and every view is independent and the
scene is read-only during a frame, so each GPU holds a full copy of the scene
and renders its own frames, with no collective on the data path. The only
cross-rank step is the timing of a multi-GPU run: a barrier on both sides of
the timed region, the slowest rank's time, and the whole job's throughput
(the units all ranks processed over that time).

Works with any initialised torch.distributed group (NCCL on GPUs, gloo on the
host); without one it is the single-process identity.
"""
from __future__ import annotations


def _group():
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        return dist
    return None


def world_size() -> int:
    d = _group()
    return d.get_world_size() if d else 1


def barrier() -> None:
    d = _group()
    if d:
        d.barrier()


def _reduce(x: float, op: str, device=None) -> float:
    d = _group()
    if d is None:
        return float(x)
    import torch
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    d.all_reduce(t, op=d.ReduceOp.MAX if op == "max" else d.ReduceOp.SUM)
    return float(t.item())


def max_over_ranks(x: float, device=None) -> float:
    """The largest value any rank passes (every rank gets it)."""
    return _reduce(x, "max", device)


def sum_over_ranks(x: float, device=None) -> float:
    return _reduce(x, "sum", device)


def job_throughput(units: float, seconds: float, device=None):
    """(whole-job units per second, slowest rank's seconds): the units all
    ranks processed over the slowest rank's time. `device` is where the
    reduction tensors live (the GPU for NCCL, None for gloo)."""
    total = sum_over_ranks(units, device)
    slowest = max_over_ranks(seconds, device)
    return (total / slowest if slowest > 0 else 0.0), slowest
