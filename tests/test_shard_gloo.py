"""Multi-process host logic of the sharded batch (gloo, two ranks on CPU):
every scene is solved by exactly one rank, the loads are balanced, and the
whole-job totals combine as the bench reports them."""
import os
import socket

import numpy as np
import pytest


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, sizes, out):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from siconos_gb300.shard import combine, shard_scenes
        mine = shard_scenes(sizes, rank, world)
        shards = [None] * world
        dist.all_gather_object(shards, mine)
        # each rank "solves" its scenes: 10 sweeps of each, 1 s per 1e6 contact-sweeps
        cs = 10.0 * sum(sizes[k] for k in mine)
        total, tmax = combine(cs, cs / 1e6, world)
        out[rank] = (shards, total, tmax)
    finally:
        dist.destroy_process_group()


def test_two_ranks_partition_and_combine():
    pytest.importorskip("torch")
    import torch.multiprocessing as mp
    rng = np.random.default_rng(3)
    sizes = [int(x) for x in rng.integers(20, 10000, 64)]
    world = 2
    ctx = mp.get_context("spawn")
    with ctx.Manager() as man:
        out = man.dict()
        port = _free_port()
        procs = [ctx.Process(target=_worker, args=(r, world, port, sizes, out)) for r in range(world)]
        for p in procs:
            p.start()
        for p in procs:
            p.join(120)
            assert p.exitcode == 0
        res = dict(out)
    shards, total, tmax = res[0]
    assert shards == res[1][0]
    flat = sorted(k for s in shards for k in s)
    assert flat == list(range(len(sizes)))
    loads = [sum(sizes[k] for k in s) for s in shards]
    assert max(loads) - min(loads) <= max(sizes)
    assert total == pytest.approx(10.0 * sum(sizes))
    assert tmax == pytest.approx(max(loads) * 10.0 / 1e6)
    assert res[1][1] == total and res[1][2] == tmax


def test_shard_single_rank_and_errors():
    from siconos_gb300.shard import shard_scenes
    assert shard_scenes([5, 3, 9], 0, 1) == [0, 1, 2]
    assert shard_scenes([], 0, 2) == []
    with pytest.raises(ValueError):
        shard_scenes([1], 2, 2)
