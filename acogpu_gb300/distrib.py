"""Several GPUs, one process each (torchrun): the single-instance path runs
independent replicas (the pheromone matrix is shared state and the reference
has no multi-colony exchange), batches of instances are sharded by instance
with no data-path collective.  Only the timing and the work counts cross
ranks, once, at the end."""
import numpy as np


def instance_cost(n, m, k):
    """Estimated construction work of one iteration: m ants x n steps x k
    candidates."""
    return float(m) * float(n) * float(k)


def shard_instances(sizes, ants, k, world):
    """Instances -> ranks, longest processing time first: every instance goes
    to the rank with the least estimated work so far (ties to the lower rank,
    so every rank computes the same assignment).  Returns one sorted index
    list per rank."""
    sizes = np.asarray(sizes, dtype=np.int64)
    ants = np.asarray(ants, dtype=np.int64)
    if world < 1:
        raise ValueError("world must be >= 1")
    kk = np.minimum(np.int64(k), sizes - 1)
    cost = ants.astype(np.float64) * sizes.astype(np.float64) * kk.astype(np.float64)
    order = sorted(range(len(sizes)), key=lambda i: (-cost[i], i))
    load = [0.0] * world
    out = [[] for _ in range(world)]
    for i in order:
        r = min(range(world), key=lambda q: (load[q], q))
        out[r].append(i)
        load[r] += cost[i]
    return [sorted(s) for s in out]


def replica_seed(base, rank):
    """Seed of replica `rank`: independent random streams per GPU."""
    return int(base) + 7919 * int(rank)


def reduce_times_and_counts(times, counts, device=None):
    """Max over ranks of each timing and sum of each count (one all-reduce
    each); a no-op without an initialised process group."""
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(v) for v in times], dtype=torch.float64, device=device)
    c = torch.tensor([float(v) for v in counts], dtype=torch.float64, device=device)
    if dist.is_available() and dist.is_initialized() and dist.get_world_size() > 1:
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        dist.all_reduce(c, op=dist.ReduceOp.SUM)
    return t.tolist(), c.tolist()
