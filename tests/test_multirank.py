"""Replica sharding on 2 gloo ranks (CPU): the partition covers every system
once with balanced work, and the max-over-ranks aggregation is what bench.py
reports.  Each rank solves its share with the CPU oracle (no GPU here)."""
import os

import numpy as np
import pytest
import torch.distributed as dist
import torch.multiprocessing as mp

from tpr_gb300 import generate as G
from tpr_gb300 import replicas


def test_partition_balanced_and_complete():
    ns = G.uneven_sizes(4096, 6, 16, 3)
    for world in (1, 2, 4, 8):
        parts = replicas.partition(ns, world)
        allk = np.sort(np.concatenate(parts))
        np.testing.assert_array_equal(allk, np.arange(len(ns)))
        loads = [ns[p].sum() for p in parts]
        assert max(loads) - min(loads) <= ns.max()


def _worker(rank, world, port, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port),
                      RANK=str(rank), WORLD_SIZE=str(world))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from oracle import oracle as O
    P = O.port()
    ns = G.uneven_sizes(64, 6, 10, 1)
    mine = replicas.partition(ns, world)[rank]
    bt = G.batch(ns[mine], 1000 + rank, "dominant")
    x = P.batch_thomas(bt, threads=1)
    worst, _ = P.batch_rel_l2(bt, x, bt.xt, threads=1)
    t_ms, err = replicas.aggregate([10.0 * (rank + 1), worst])
    out[rank] = (t_ms, err, len(mine), int(ns[mine].sum()))
    dist.destroy_process_group()


def test_two_gloo_ranks():
    mp.set_start_method("spawn", force=True)
    mgr = mp.Manager()
    out = mgr.dict()
    port = 29500 + os.getpid() % 1000
    mp.spawn(_worker, args=(2, port, out), nprocs=2, join=True)
    assert out[0][0] == out[1][0] == 20.0        # max over ranks
    assert out[0][1] == out[1][1] < 1e-6
    assert out[0][2] + out[1][2] == 64
