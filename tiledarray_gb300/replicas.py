"""Replica aggregation for multi-GPU runs.

The contraction path does not shard: with N GPUs every rank runs its own
replica of the workload (no collective on the data path).  The only
cross-rank step is the timing reduction of bench.py: the job time is the
maximum over ranks and the throughput the work of all ranks over that time.
"""
from __future__ import annotations


def aggregate(local_ms: float, local_flops: float, dist=None, device=None):
    """Returns (job_ms, total_flops, world_size)."""
    if dist is None or not dist.is_initialized():
        return local_ms, local_flops, 1
    import torch
    t = torch.tensor([local_ms, local_flops], dtype=torch.float64, device=device)
    ms = t[:1].clone()
    fl = t[1:].clone()
    dist.all_reduce(ms, op=dist.ReduceOp.MAX)
    dist.all_reduce(fl, op=dist.ReduceOp.SUM)
    return float(ms.item()), float(fl.item()), dist.get_world_size()
