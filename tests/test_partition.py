"""Host-side multi-rank plumbing (finitevolumesolver_gb300/partition.py):
the Morton partition of an AMR patch table, and the MIN / MAX reductions
across two gloo ranks on the CPU."""
import os
import socket

import numpy as np
import pytest

from finitevolumesolver_gb300 import partition, workloads


def _hier():
    h, _ = workloads.amr_blast_2d(128, 3, target=300, sizes=(8, 16, 32))
    return h


@pytest.mark.parametrize("nranks", [1, 2, 3, 8])
def test_partition_covers_once_and_balances(nranks):
    h = _hier()
    parts = partition.partition(h, nranks)
    allp = np.concatenate(parts)
    assert len(parts) == nranks
    assert sorted(allp.tolist()) == list(range(h.npatches))
    w = partition.patch_weights(h)
    loads = np.array([w[p].sum() for p in parts])
    assert loads.max() <= w.sum() / nranks + w.max()


def test_morton_order_keeps_neighbours_close():
    k = partition.morton_key(np.array([0, 1, 0, 1, 2]), np.array([0, 0, 1, 1, 0]))
    assert k.tolist() == [0, 1, 2, 3, 4]


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        h = _hier()
        mine = partition.partition(h, world)[rank]
        # a per-patch stable dt (synthetic) reduced with MinAll
        dt = 1e-3 * (1.0 + np.arange(h.npatches) % 17) / (1 + h.levels)
        local = float(dt[mine].min()) if len(mine) else float("inf")
        gmin = partition.allreduce_min(local)
        slow = partition.slowest(10.0 + rank)
        q.put((rank, len(mine), gmin, float(dt.min()), slow))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_reduce_dt_and_time():
    import torch.multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res.sort()
    h = _hier()
    assert res[0][1] + res[1][1] == h.npatches
    for r in res:
        assert r[2] == r[3]      # global min dt on every rank
        assert r[4] == 11.0      # slowest rank's time
