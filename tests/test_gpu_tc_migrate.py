"""MTE with the migration on the tensor cores (tcgen05 kind::tf32, 3xTF32)
against the oracle and the reference kernels' golden outputs.  3xTF32 sums
in a different order than the SIMT path, so agreement is to FP32 rounding
(stated tolerances), not bit for bit."""
import numpy as np
import pytest

from oracle import pyoracle as po
from transportoptimiser_gb300 import simulate_gpu as sg
from transportoptimiser_gb300 import synth
from transportoptimiser_gb300._capi import MIG_SPARSE_FP32, MIG_TC_3XTF32
from transportoptimiser_gb300.generation import Generation, pack_roads

pytestmark = pytest.mark.gpu
PATH_RTOL = 1e-4      # one path after 50 years of logistic growth with noise
MEAN_RTOL = 1e-5      # expected end population


def _check(end, ref):
    ref = ref.astype(np.float64)
    np.testing.assert_allclose(end, ref, rtol=PATH_RTOL, atol=1e-3)
    assert abs(end.mean() - ref.mean()) <= MEAN_RTOL * abs(ref.mean())


@pytest.mark.parametrize("sem", [0, 1])
def test_tc_mte_matches_oracle(ctx, sem):
    sc = synth.mte_road(0)
    sp = sc.species[0]
    m = po.species_model(sc, sp, sc.roads[0], sem=0)
    P, Y = 300, 50
    end, st = sg.simulateMTECUDA([m], [sp.params], P, Y, seed=11, road=2, sem=sem,
                                 migration=MIG_TC_3XTF32, ctx=ctx)
    ref = po.simulate_mte(P, Y, m["N"], 1.0, sp.params, m["init_pops"], m["caps"], m["mmm"][2],
                          11, 2, 0, sem)
    _check(end[:, 0], ref)


def test_tc_mte_matches_reference_golden(ctx, golden):
    g = golden["mte"]
    m = dict(N=int(g["N"]), init_pops=g["init"], caps=g["caps"], mmm=g["mmm"][None])
    end, _ = sg.simulateMTECUDA([m], [g["params"]], int(g["P"]), int(g["Y"]), seed=int(g["seed"]),
                                road=0, sem=0, migration=MIG_TC_3XTF32, control=0, ctx=ctx)
    np.testing.assert_allclose(end[:, 0], g["end"], rtol=PATH_RTOL)
    assert abs(end[:, 0].mean() - g["end"].mean()) <= MEAN_RTOL * g["end"].mean()


def test_tc_mte_multi_species_ragged_tiles(ctx):
    sc = synth.rov_road(2, n_species=2)
    ms = [po.species_model(sc, sc.species[s], sc.roads[0], sem=0) for s in range(2)]
    m1 = dict(ms[1])
    n = m1["N"] - 5
    m1.update(N=n, init_pops=m1["init_pops"][:n], caps=m1["caps"][:n],
              mmm=np.ascontiguousarray(m1["mmm"][:, :n, :n]))
    P, Y = 150, 20              # 150 paths: a partial path tile
    end, _ = sg.simulateMTECUDA([ms[0], m1], [sc.species[0].params, sc.species[1].params], P, Y,
                                seed=3, road=1, migration=MIG_TC_3XTF32, ctx=ctx)
    for s, m in enumerate([ms[0], m1]):
        ref = po.simulate_mte(P, Y, m["N"], 1.0, sc.species[s].params, m["init_pops"], m["caps"],
                              m["mmm"][2], 3, 1, s, 0)
        _check(end[:, s], ref)


def test_tc_mte_three_destination_tiles(ctx):
    # ~300 patches: three 128-destination tiles, 19+ source groups
    sc = synth.generation(0, n_roads=2)
    sp = sc.species[0]
    m = po.species_model(sc, sp, sc.roads[0], sem=0, max_patches=1024)
    assert m["N"] > 256
    P, Y = 64, 50
    end, _ = sg.simulateMTECUDA([m], [sp.params], P, Y, seed=5, road=0, sem=0,
                                migration=MIG_TC_3XTF32, ctx=ctx)
    ref = po.simulate_mte(P, Y, m["N"], 1.0, sp.params, m["init_pops"], m["caps"], m["mmm"][-1],
                          5, 0, 0, 0)
    _check(end[:, 0], ref)


def test_tc_generation_matches_sparse(ctx):
    sc = synth.generation(1, n_roads=16)
    gen = Generation(sc, max_roads=16, max_patches=512, ctx=ctx)
    packed = pack_roads(sc, sc.roads)
    a = gen.evaluate(packed, gen.opts(64, 50, seed=2, migration=MIG_SPARSE_FP32))
    b = gen.evaluate(packed, gen.opts(64, 50, seed=2, migration=MIG_TC_3XTF32))
    gen.close()
    np.testing.assert_array_equal(a[:, :, :2], b[:, :, :2])          # patches, transitions
    np.testing.assert_allclose(b[:, :, 2], a[:, :, 2], rtol=MEAN_RTOL)  # mean end population
    np.testing.assert_allclose(b[:, :, 6], a[:, :, 6], rtol=1e-12)     # initial population
