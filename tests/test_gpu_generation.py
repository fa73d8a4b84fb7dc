"""Batched generation (one launch per stage for all roads) against the
single-road entry points and the oracle."""
import math

import numpy as np
import pytest

from oracle import pyoracle as po
from transportoptimiser_gb300 import simulate_gpu as sg
from transportoptimiser_gb300 import synth
from transportoptimiser_gb300._capi import MIG_AUTO, MIG_SIMT_FP32, MIG_SPARSE_FP32
from transportoptimiser_gb300.generation import Generation, pack_roads

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mig", [MIG_SIMT_FP32, MIG_SPARSE_FP32])
def test_generation_matches_single_road_calls(ctx, mig):
    sc = synth.mte_road(0)
    rng = np.random.Generator(np.random.Philox(9))
    sc.roads = [synth.random_road(sc.W, sc.H, n, rng) for n in (4, 10, 17)]
    gen = Generation(sc, max_roads=8, max_patches=256, ctx=ctx)
    P, Y = 200, 30
    res = gen.evaluate(pack_roads(sc, sc.roads),
                       gen.opts(P, Y, seed=5, road0=100, migration=mig))
    for r, rd in enumerate(sc.roads):
        m = po.species_model(sc, sc.species[0], rd, sem=0)
        assert int(res[r, 0, 0]) == m["N"]
        assert int(res[r, 0, 1]) == m["n_transitions"]
        end, st = sg.simulateMTECUDA([m], [sc.species[0].params], P, Y, seed=5, road=100 + r,
                                     migration=mig, ctx=ctx)
        assert res[r, 0, 2] == st[0]["mean"]
        ref = po.simulate_mte(P, Y, m["N"], 1.0, sc.species[0].params, m["init_pops"],
                              m["caps"], m["mmm"][2], 5, 100 + r, 0, 0)
        assert math.isclose(res[r, 0, 2], ref.astype(np.float64).mean(), rel_tol=1e-12)
    gen.close()


def test_generation_three_species_grid(ctx):
    sc = synth.generation(0, n_roads=3)
    gen = Generation(sc, max_roads=3, max_patches=512, ctx=ctx)
    res = gen.evaluate(pack_roads(sc, sc.roads), gen.opts(64, 10, seed=1, migration=MIG_AUTO))
    for r in range(3):
        for s in range(3):
            m = po.species_model(sc, sc.species[s], sc.roads[r], sem=0, max_patches=1024)
            assert int(res[r, s, 0]) == m["N"]
            assert int(res[r, s, 1]) == m["n_transitions"]
    gen.close()
