"""GPU: sets across ranks through the GPU's batched build.

``shard.batch_distributed`` gives each rank an LPT share of the sets; every
rank builds its share with the batched GPU build and rank 0 gathers the edge
lists.  Here two gloo ranks run as two processes on the one GPU of this
machine (their builds are independent: no kernel of one waits on the other),
and the gathered lists must equal the oracle's, set by set.  The partitioning
and gather logic alone is covered on the CPU in tests/test_shard_cpu.py.
"""
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from voronoids_gb300 import workloads as W

pytestmark = pytest.mark.gpu

SIZES = [3000, 40, 9000, 1200, 55, 700, 20000]


def _sets():
    return [W.uniform_points(n, 3, 90 + i) for i, n in enumerate(SIZES)]


def _worker(rank, world, port, q):
    import torch
    import torch.distributed as dist
    from voronoids_gb300 import shard
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    torch.cuda.set_device(0)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    out = shard.batch_distributed(_sets(), seed=4)  # the default builder: the batched GPU build
    if rank == 0:
        q.put([e.tolist() for e in out])
    dist.barrier()
    dist.destroy_process_group()


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_sets_across_two_ranks_match_oracle(oracle):
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    got = q.get(timeout=300)
    for p in procs:
        p.join(timeout=300)
        assert p.exitcode == 0
    sets = _sets()
    assert len(got) == len(sets)
    for g, p in zip(got, sets):
        assert np.array_equal(np.array(g, dtype=np.int64).reshape(-1, 2), oracle.Triangulation(p, seed=4).edges())
