"""The N > 1 path on CPU: instance sharding of batches (every rank derives
the same disjoint, complete, cost-balanced assignment) and the one reduction
the bench makes (max of the times, sum of the work), run as world_size-2
gloo process groups."""
import json
import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp

from acogpu_gb300 import distrib, instances


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


@pytest.mark.parametrize("world", [1, 2, 3, 8])
def test_shards_are_disjoint_complete_and_balanced(world):
    sizes = instances.batch_sizes(512 * world, seed=7)
    ants = np.minimum(sizes, 1024)
    shards = distrib.shard_instances(sizes, ants, 20, world)
    flat = sorted(i for s in shards for i in s)
    assert flat == list(range(len(sizes)))
    load = [sum(distrib.instance_cost(sizes[i], ants[i], min(20, sizes[i] - 1)) for i in s)
            for s in shards]
    assert max(load) <= 1.02 * min(load)
    assert shards == distrib.shard_instances(sizes, ants, 20, world)  # deterministic


def test_replica_seeds_differ():
    seeds = {distrib.replica_seed(1234, r) for r in range(8)}
    assert len(seeds) == 8


def _worker(rank, world, port, out_dir):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        times, counts = distrib.reduce_times_and_counts([1.0 + rank, 10.0 - rank],
                                                        [100 * (rank + 1), 7])
        sizes = instances.batch_sizes(64 * world, seed=3)
        shard = distrib.shard_instances(sizes, np.minimum(sizes, 1024), 20, world)[rank]
        with open(os.path.join(out_dir, f"r{rank}.json"), "w") as f:
            json.dump({"times": times, "counts": counts, "shard": shard}, f)
    finally:
        dist.destroy_process_group()


def test_gloo_world2_reduction_and_sharding(tmp_path):
    world = 2
    mp.spawn(_worker, args=(world, _free_port(), str(tmp_path)), nprocs=world, join=True)
    res = [json.load(open(tmp_path / f"r{r}.json")) for r in range(world)]
    for r in res:
        assert r["times"] == [2.0, 10.0]          # max over ranks
        assert r["counts"] == [300.0, 14.0]       # sum over ranks
    shards = [set(r["shard"]) for r in res]
    assert not (shards[0] & shards[1])
    assert sorted(shards[0] | shards[1]) == list(range(64 * world))
