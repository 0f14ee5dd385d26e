"""Replicas on several GPUs of one node (one process per GPU).

The path has no data exchange between instances (single cells, strands and
whole tissues are independent), so N GPUs run N replicas, or shards of a batch
of instances, with no collective on the data path.  The only collectives are
for reporting: the throughput over ranks (work summed, time = the slowest
rank) and gathering per-instance results on rank 0.
"""
from __future__ import annotations

import numpy as np


def shard_bounds(n: int, rank: int, world: int, weights=None):
    """[lo, hi) of the instances rank `rank` of `world` takes: contiguous
    blocks with about equal total weight (default: equal counts)."""
    if world <= 1:
        return 0, n
    w = np.ones(n) if weights is None else np.asarray(weights, np.float64)
    c = np.concatenate([[0.0], np.cumsum(w)])
    cuts = [int(np.searchsorted(c, c[-1] * r / world, side="left")) for r in range(world + 1)]
    cuts[0], cuts[-1] = 0, n
    for r in range(1, world + 1):
        cuts[r] = max(cuts[r], cuts[r - 1])
    return cuts[rank], cuts[rank + 1]


def _dist():
    try:
        import torch.distributed as dist
    except ImportError:
        return None
    return dist if dist.is_available() and dist.is_initialized() else None


def aggregate_throughput(work_local: float, ms_local: float):
    """(whole-job units/s, max ms over ranks, total work): work summed over
    ranks and divided by the slowest rank's time."""
    dist = _dist()
    if dist is None:
        return work_local / (ms_local / 1e3), ms_local, work_local
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([ms_local], dtype=torch.float64, device=dev)
    w = torch.tensor([work_local], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    dist.all_reduce(w, op=dist.ReduceOp.SUM)
    ms, work = float(t.item()), float(w.item())
    return work / (ms / 1e3), ms, work


def gather_rows(local: np.ndarray, n_total: int, lo: int):
    """Rows [lo, lo + len(local)) of every rank assembled into an array of
    n_total rows on every rank (per-instance results of a sharded batch)."""
    dist = _dist()
    local = np.ascontiguousarray(local, np.float64)
    if dist is None:
        out = np.zeros((n_total,) + local.shape[1:])
        out[lo:lo + len(local)] = local
        return out
    import torch
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    full = torch.zeros((n_total,) + local.shape[1:], dtype=torch.float64, device=dev)
    full[lo:lo + len(local)] = torch.from_numpy(local).to(dev)
    dist.all_reduce(full, op=dist.ReduceOp.SUM)      # disjoint row ranges: the sum assembles them
    return full.cpu().numpy()
