"""Sharding of batch instances across ranks: the assignment is a partition,
balanced, and identical on every rank (checked with two gloo processes on
the CPU; no GPU)."""
import os
import socket

import numpy as np
import torch.distributed as dist
import torch.multiprocessing as mp

from pdal_gb300.shard import lpt_partition


def test_lpt_partition_is_a_balanced_partition():
    rng = np.random.default_rng(0)
    w = np.exp(rng.uniform(np.log(50), np.log(5000), 4096))
    for k in (1, 2, 4, 8):
        parts = lpt_partition(w, k)
        flat = sorted(i for p in parts for i in p)
        assert flat == list(range(len(w)))
        loads = [w[p].sum() for p in parts]
        assert max(loads) - min(loads) <= w.max()


def _worker(rank, world, port, q):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    rng = np.random.default_rng(1)
    w = rng.uniform(1, 100, 257)
    mine = lpt_partition(w, world)[rank]
    t = torch_tensor(len(mine))
    dist.all_reduce(t)
    gathered = [None] * world
    dist.all_gather_object(gathered, mine)
    q.put((rank, int(t.item()), gathered))
    dist.destroy_process_group()


def torch_tensor(v):
    import torch

    return torch.tensor([v], dtype=torch.int64)


def test_ranks_agree_on_the_assignment():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in procs]
    for p in procs:
        p.join(timeout=60)
    for rank, total, gathered in res:
        assert total == 257
        flat = sorted(i for part in gathered for i in part)
        assert flat == list(range(257))
    assert res[0][2] == res[1][2]
