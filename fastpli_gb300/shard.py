"""Work partitioning across GPUs (one process per GPU).

The forward model shards with no data exchange: tiles, requests and tilts
are independent, and rays within a volume are independent.  A multi-GPU run
therefore assigns whole work units (tiles or volumes) to ranks and needs only
a barrier plus a max-over-ranks of the elapsed time — no collective on the
data path (the reference's MPI image merge, simulator.cpp:407-408, has no
counterpart because no volume is split).
"""

import numpy as np


def balanced_shards(costs, world_size):
    """Greedy longest-processing-time assignment of units with the given
    costs to ``world_size`` ranks.  Returns one sorted index list per rank;
    deterministic (ties broken by unit index, then rank)."""
    costs = np.asarray(costs, dtype=np.float64)
    if world_size < 1:
        raise ValueError("world_size must be >= 1")
    order = sorted(range(costs.size), key=lambda i: (-costs[i], i))
    load = np.zeros(world_size)
    shards = [[] for _ in range(world_size)]
    for i in order:
        r = int(np.argmin(load))
        shards[r].append(i)
        load[r] += costs[i]
    return [sorted(s) for s in shards]


def rank_units(costs, world_size, rank):
    return balanced_shards(costs, world_size)[rank]


def max_over_ranks(value, dist=None, device=None):
    """Max of a float over all ranks of the default process group (the
    job's elapsed time is the slowest rank's)."""
    if dist is None or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(value)
    import torch
    t = torch.tensor([float(value)], dtype=torch.float64,
                     device=device if device is not None else "cpu")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
