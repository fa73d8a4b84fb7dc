"""Two-rank (gloo, CPU) check of the generation sharding: disjoint roads and
random streams per rank, and the max-over-ranks timing reduction."""
import os

import numpy as np
import pytest
import torch.multiprocessing as mp


def _worker(rank, world, port, q):
    import torch
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from transportoptimiser_gb300 import shard, synth
    sc = synth.generation(0, n_roads=1)
    roads = shard.rank_roads(sc, 16, rank)
    digest = torch.tensor([float(np.sum(r.points)) for r in roads], dtype=torch.float64)
    got = [torch.zeros_like(digest) for _ in range(world)]
    dist.all_gather(got, digest)
    t = shard.max_over_ranks(10.0 + rank)
    q.put((rank, [g.numpy() for g in got], t, shard.road0(rank)))
    dist.destroy_process_group()


def test_two_rank_sharding():
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = 29500 + os.getpid() % 1000
    procs = [ctx.Process(target=_worker, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    res = [q.get(timeout=120) for _ in range(2)]
    for p in procs:
        p.join(timeout=60)
        assert p.exitcode == 0
    res.sort()
    g0, g1 = res[0][1]
    assert not np.intersect1d(g0, g1).size            # different roads per rank
    assert np.array_equal(res[0][1][1], res[1][1][1])  # all ranks see the same gather
    assert res[0][2] == res[1][2] == 11.0             # max over ranks
    assert res[1][3] - res[0][3] >= 1_000_000         # disjoint road-id streams
