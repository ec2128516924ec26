"""Sharding of batch instances across ranks: the assignment is a partition,
balanced, and identical on every rank (checked with two gloo processes on
the CPU; no GPU)."""
import os
import socket

import numpy as np
import torch.distributed as dist
import torch.multiprocessing as mp

from pdal_gb300.shard import assemble, instance_weight, lpt_partition


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


def _solve_worker(rank, world, port, q):
    """One rank of a sharded batch: solve its LPT share with the CPU oracle
    (standing in for the persistent GPU launch), gather every rank's results
    over gloo and put them back in instance order."""
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from oracle import oracle as O
    from pdal_gb300 import instances

    items = instances.batch_lps(count=12, seed=77, m_range=(20, 80))
    parts = lpt_partition([instance_weight(d) for d in items], world)
    mine = [O.solve_lp(items[i], {"eps": 1e-6, "l_inf_ruiz_iterations": 4}) for i in parts[rank]]
    rows = [(r.status, r.iterations, r.primal_objective) for r in mine]
    gathered = [None] * world
    dist.all_gather_object(gathered, rows)
    q.put((rank, assemble(parts, gathered)))
    dist.destroy_process_group()


def test_sharded_results_gathered_equal_single_rank():
    """Two ranks each solve their share; gathered and reassembled, the results
    equal one rank solving every instance in order."""
    from oracle import oracle as O
    from pdal_gb300 import instances

    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    procs = [ctx.Process(target=_solve_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=300) for _ in procs]
    for p in procs:
        p.join(timeout=60)
    items = instances.batch_lps(count=12, seed=77, m_range=(20, 80))
    single = [(r.status, r.iterations, r.primal_objective)
              for r in (O.solve_lp(d, {"eps": 1e-6, "l_inf_ruiz_iterations": 4}) for d in items)]
    for _, rows in res:
        assert [tuple(x) for x in rows] == single
