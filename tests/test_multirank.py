"""Multi-rank host logic on CPU (gloo, world size 2): every unit is assigned
exactly once, ranks agree on the assignment without exchanging it, and the
job time is the max over ranks."""

import os
import socket

import numpy as np
import torch.distributed as dist
import torch.multiprocessing as mp

from fastpli_gb300 import shard


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, costs, out):
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    mine = shard.rank_units(costs, world, rank)
    # gather every rank's shard to check coverage (test only; the product
    # path exchanges nothing)
    gathered = [None] * world
    dist.all_gather_object(gathered, mine)
    elapsed = 1.0 + rank  # stand-in per-rank time
    job = shard.max_over_ranks(elapsed, dist)
    dist.barrier()
    out[rank] = (gathered, job)
    dist.destroy_process_group()


def test_balanced_shards_cover_units_once():
    rng = np.random.default_rng(0)
    costs = rng.integers(1, 100, 257)
    for world in (1, 2, 3, 8):
        s = shard.balanced_shards(costs, world)
        flat = sorted(i for part in s for i in part)
        assert flat == list(range(costs.size))
        loads = [costs[p].sum() for p in s]
        assert max(loads) - min(loads) <= costs.max()


def test_gloo_two_ranks_agree_and_take_max():
    ctx = mp.get_context("spawn")
    manager = ctx.Manager()
    out = manager.dict()
    costs = list(np.random.default_rng(1).integers(1, 50, 33))
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, 2, port, costs, out)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    g0, job0 = out[0]
    g1, job1 = out[1]
    assert g0 == g1
    assert sorted(g0[0] + g0[1]) == list(range(len(costs)))
    assert job0 == job1 == 2.0
