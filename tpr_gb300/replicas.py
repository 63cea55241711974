"""Multi-GPU use of the solver: replicas, no data-path collective.

Independent systems need no exchange, so a global batch is split across
ranks by system, balanced by total equations (the work), and every rank
solves its share on its own GPU.  The only collective is the bookkeeping at
the end: max-over-ranks time and worst error (`aggregate`).
"""
from __future__ import annotations

import numpy as np


def partition(ns, world: int) -> list[np.ndarray]:
    """Indices of the systems each rank solves: greedy longest-first onto the
    least-loaded rank (balanced by sum of n); each rank's list is sorted."""
    ns = np.asarray(ns, np.int64)
    load = np.zeros(world, np.int64)
    parts = [[] for _ in range(world)]
    for k in np.argsort(-ns, kind="stable"):
        r = int(np.argmin(load))
        parts[r].append(int(k))
        load[r] += ns[k]
    return [np.array(sorted(p), np.int64) for p in parts]


def aggregate(values, group=None):
    """Element-wise max over ranks of a list of floats (time, error, ...)."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(v) for v in values], dtype=torch.float64)
    if dist.is_available() and dist.is_initialized():
        if dist.get_backend(group) == "nccl":
            t = t.cuda()
        dist.all_reduce(t, op=dist.ReduceOp.MAX, group=group)
    return t.cpu().tolist()
