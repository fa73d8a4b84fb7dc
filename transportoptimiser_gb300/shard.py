"""Sharding of a GA generation over ranks (one process per GPU).

Roads are independent, so each rank values its own roads with no exchange
on the data path (weak scaling, as the reference's per-GPU host threads do,
RoadGA.cpp:1687-1748).  Every rank holds the same scene; its roads come from
its own seeded stream and its Monte Carlo streams start at road id
rank * ROAD_STRIDE, so no two ranks share random numbers.  The only
collective is the timing reduction (maximum over ranks) of the bench.
"""
from __future__ import annotations

import numpy as np

ROAD_STRIDE = 1_000_000


def rank_roads(scene, n_roads: int, rank: int, seed: int = 0):
    """The rank's generation: n_roads roads of 8-64 control points."""
    from . import synth
    rng = np.random.Generator(np.random.Philox(key=[seed, 0x5eed + rank]))
    return [synth.random_road(scene.W, scene.H, int(rng.integers(8, 65)), rng)
            for _ in range(n_roads)]


def road0(rank: int) -> int:
    """Stream id of the rank's first road."""
    return rank * ROAD_STRIDE


def max_over_ranks(x: float) -> float:
    """Maximum of a per-rank number (the step time) over the process group."""
    import torch
    import torch.distributed as dist
    if not dist.is_available() or not dist.is_initialized() or dist.get_world_size() == 1:
        return float(x)
    dev = "cuda" if dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(x)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())
