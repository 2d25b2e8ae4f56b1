"""The multi-GPU path of the batched solve on the CPU: two `gloo` ranks
shard a batch of instances (no collective on the data path) and gather
their per-instance stats at the end.  The solves themselves are stood in
for by a host function of the instance, so no GPU is needed."""

import os
import socket

import numpy as np
import pytest
import torch.multiprocessing as mp


def _free_port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    port = s.getsockname()[1]
    s.close()
    return port


def _worker(rank, world, port, sizes, out):
    import torch.distributed as dist
    from opymize_gb300.solvers.batch import shard, gather_stats
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        mine = shard(sizes, rank, world)
        # stand-in for the solves: a value per instance and the rank that did it
        stats = {int(i): (rank, int(sizes[i]) * 3 + 1) for i in mine}
        allstats = gather_stats(stats)
        out[rank] = (mine, allstats)
    finally:
        dist.destroy_process_group()


@pytest.mark.parametrize("world", [2])
def test_sharded_batch_covers_every_instance_once(world):
    rng = np.random.default_rng(0)
    sizes = (np.exp(rng.uniform(np.log(64), np.log(1024), 40)) ** 2).astype(np.int64)
    ctx = mp.get_context("spawn")
    mgr = ctx.Manager()
    out = mgr.dict()
    port = _free_port()
    procs = [ctx.Process(target=_worker, args=(r, world, port, sizes, out)) for r in range(world)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
        assert p.exitcode == 0
    shards = [out[r][0] for r in range(world)]
    # disjoint and complete
    flat = sorted(i for sh in shards for i in sh)
    assert flat == list(range(len(sizes)))
    # balanced: no rank carries more than the largest instance above the mean
    loads = [int(sizes[sh].sum()) for sh in shards]
    assert max(loads) - min(loads) <= int(sizes.max())
    # every rank gathered every rank's stats, identical everywhere
    for r in range(world):
        gathered = out[r][1]
        merged = {}
        for d in gathered:
            merged.update(d)
        assert sorted(merged) == list(range(len(sizes)))
        assert all(merged[i][1] == int(sizes[i]) * 3 + 1 for i in merged)
        assert all(merged[i][0] == next(k for k, sh in enumerate(shards) if i in sh) for i in merged)


def test_shard_without_process_group():
    from opymize_gb300.solvers.batch import shard, gather_stats
    sizes = [5, 1, 4, 2, 3]
    assert shard(sizes, 0, 1) == [0, 1, 2, 3, 4]
    assert sorted(shard(sizes, 0, 2) + shard(sizes, 1, 2)) == [0, 1, 2, 3, 4]
    assert gather_stats({"a": 1}) == [{"a": 1}]
    with pytest.raises(ValueError):
        shard(sizes, 2, 2)
