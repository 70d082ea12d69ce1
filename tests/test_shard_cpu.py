"""CPU: sets across ranks (LPT assignment, gather on rank 0) with gloo, world
size 2.  The builder is the oracle here (no GPU); on GPUs it is the batched
build."""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from voronoids_gb300 import shard
from voronoids_gb300 import workloads as W


def test_lpt_balances_and_covers():
    sizes = W.c4_sizes(4096)
    parts = shard.lpt_assign(sizes, 8)
    flat = sorted(i for p in parts for i in p)
    assert flat == list(range(len(sizes)))
    loads = [int(sizes[p].sum()) for p in parts]
    assert max(loads) - min(loads) <= int(sizes.max())
    assert shard.lpt_assign([5], 3) == [[0], [], []]


def _oracle_build(sets, seed=0):
    from oracle import oracle as O
    return [O.Triangulation(p, seed=seed).edges() for p in sets]


def _worker(rank, world, port, q):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    sets = [W.uniform_points(n, 3, 50 + i) for i, n in enumerate([300, 40, 900, 120, 55])]
    out = shard.batch_distributed(sets, seed=1, build=_oracle_build)
    if rank == 0:
        q.put([e.tolist() for e in out])
    dist.barrier()
    dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_batch_distributed_gloo_two_ranks():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = q.get(timeout=120)
    for p in procs:
        p.join(timeout=120)
        assert p.exitcode == 0
    sets = [W.uniform_points(n, 3, 50 + i) for i, n in enumerate([300, 40, 900, 120, 55])]
    want = _oracle_build(sets, seed=1)
    assert len(got) == len(want)
    for g, w in zip(got, want):
        assert np.array_equal(np.array(g, dtype=np.int64).reshape(-1, 2), w)
