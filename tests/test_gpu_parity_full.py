"""Parity at the benchmark shapes.

* Batched GA generation (200 x 200 grid, 5 habitat types, 3 species, 256
  roads of 8-64 control points, 201-368 patches per species model, 50
  years): every (road, species) of the generation, in direct and in graph
  mode, against the oracle road by road - species model (patch count,
  transitions, migration matrices), per-path end populations against the
  oracle fed the same matrices (bit for bit) and against the oracle's own
  species model, and against the single-road entry point.
* Plain MTE, one road, 2000 paths x 50 years.
* Plain ROV, one road, 10^4 paths x 50 years, 2 species, 16 bins per state
  dimension (corrected semantics): every decision, continuation value and
  regression coefficient.
"""
import math

import numpy as np
import pytest

from oracle import pyoracle as po
from transportoptimiser_gb300 import simulate_gpu as sg
from transportoptimiser_gb300 import synth
from transportoptimiser_gb300._capi import MIG_SIMT_FP32, MIG_SPARSE_FP32
from transportoptimiser_gb300.generation import Generation, pack_roads
from transportoptimiser_gb300.rov import rov_problem_from_models

pytestmark = pytest.mark.gpu

# FP32 migration matrices: the GPU's FP64 exp may differ from glibc's by one
# ulp, which moves a float entry by at most one ulp
MATRIX_ULP = 1.2e-7
# end populations from matrices that differ by one ulp somewhere
END_RTOL = 1e-5


@pytest.fixture(scope="module")
def gen_scene():
    return synth.generation(0)


def _oracle_models(sc, roads, sem):
    return {(r, s): po.species_model(sc, sc.species[s], sc.roads[r], sem=sem, max_patches=1024)
            for r in roads for s in range(len(sc.species))}


def _check_generation(ctx, gen, sc, res, roads, models, P, Y, seed, road0, sem, single=()):
    S = len(sc.species)
    for r in roads:
        for s in range(S):
            om = models[(r, s)]
            N = om["N"]
            assert int(res[r, s, 0]) == N, (r, s)
            assert int(res[r, s, 1]) == om["n_transitions"], (r, s)
            gm = gen.species_model(r, s)
            assert gm["N"] == N
            assert np.array_equal(gm["init_pops"], om["init_pops"])
            assert np.array_equal(gm["caps"], om["caps"])
            # same non-zero pattern, values within one ulp
            assert np.array_equal(gm["mmm"] > 0, om["mmm"] > 0), (r, s)
            rel = np.abs(gm["mmm"].astype(np.float64) - om["mmm"]) / np.maximum(om["mmm"], 1e-30)
            assert rel.max() <= MATRIX_ULP, (r, s, rel.max())
            end = gen.end_pops(r, s, P)
            # the batched kernel against the oracle on the same matrices: bits
            ref_same = po.simulate_mte(P, Y, N, 1.0, sc.species[s].params, gm["init_pops"],
                                       gm["caps"], gm["mmm"][-1], seed, road0 + r, s, sem,
                                       threads=16)
            assert np.array_equal(end, ref_same), (r, s)
            # against the oracle's own species model
            ref_own = po.simulate_mte(P, Y, N, 1.0, sc.species[s].params, om["init_pops"],
                                      om["caps"], om["mmm"][-1], seed, road0 + r, s, sem,
                                      threads=16)
            if np.array_equal(gm["mmm"], om["mmm"]):
                assert np.array_equal(end, ref_own), (r, s)
            else:
                np.testing.assert_allclose(end, ref_own, rtol=END_RTOL)
            e = end.astype(np.float64)
            assert math.isclose(res[r, s, 2], e.mean(), rel_tol=1e-12)
        if r in single:
            # the same road alone, one call for its species, as the reference runs it
            gms = [gen.species_model(r, s) for s in range(S)]
            one, _ = sg.simulateMTECUDA(gms, [sp.params for sp in sc.species], P, Y, seed=seed,
                                        road=road0 + r, sem=sem, migration=MIG_SPARSE_FP32,
                                        ctx=ctx)
            for s in range(S):
                assert np.array_equal(one[:, s].astype(np.float32), gen.end_pops(r, s, P)), (r, s)


def test_generation_every_road_at_bench_paths(ctx, gen_scene):
    """All 256 roads x 3 species at the benchmark's N* = 64 paths, 50 years,
    reference semantics, graph replay and direct planning, sparse kernel."""
    sc = gen_scene
    R, P, Y, seed, road0 = len(sc.roads), 64, 50, 0, 0
    gen = Generation(sc, max_roads=R, max_patches=512, ctx=ctx)
    packed = pack_roads(sc, sc.roads)
    models = _oracle_models(sc, range(R), sem=0)
    for graph in (False, True, True):
        res = gen.evaluate(packed, gen.opts(P, Y, seed=seed, road0=road0, sem=0,
                                            migration=MIG_SPARSE_FP32, graph=graph))
        _check_generation(ctx, gen, sc, res, range(R), models, P, Y, seed, road0, 0,
                          single=range(0, R, 16))
    gen.close()


def test_generation_2000_paths_widest_roads(ctx, gen_scene):
    """Sixteen roads - the widest species models of the generation among
    them - at the configuration's 2000 MTE paths, in both semantics."""
    sc = gen_scene
    probe = Generation(sc, max_roads=len(sc.roads), max_patches=512, ctx=ctx)
    res = probe.evaluate(pack_roads(sc, sc.roads), probe.opts(32, 2, migration=MIG_SPARSE_FP32))
    probe.close()
    widest = np.argsort(-res[:, :, 0].max(axis=1))[:8]
    picks = sorted(set(int(i) for i in widest) | set(range(3, 256, 32)))[:16]
    assert int(res[picks, :, 0].max()) == int(res[:, :, 0].max())
    sub = synth.Scene(W=sc.W, H=sc.H, res=sc.res, base_map=sc.base_map, species=sc.species,
                      n_controls=sc.n_controls, flows=sc.flows, seed=sc.seed,
                      roads=[sc.roads[i] for i in picks])
    P, Y = 2000, 50
    for sem in (0, 1):
        gen = Generation(sub, max_roads=len(picks), max_patches=512, ctx=ctx)
        models = _oracle_models(sub, range(len(picks)), sem=sem)
        packed = pack_roads(sub, sub.roads)
        for graph in (False, True):
            out = gen.evaluate(packed, gen.opts(P, Y, seed=9, road0=40, sem=sem,
                                                migration=MIG_SPARSE_FP32, graph=graph))
            _check_generation(ctx, gen, sub, out, range(len(picks)), models, P, Y, 9, 40, sem,
                              single=(0, 5))
        gen.close()


@pytest.mark.parametrize("mig", [MIG_SIMT_FP32, MIG_SPARSE_FP32])
@pytest.mark.parametrize("sem", [0, 1])
def test_plain_mte_2000_paths_50_years(ctx, mig, sem):
    """One road on the 64 x 64 grid, 2000 paths x 50 years, bit for bit."""
    sc = synth.mte_road(0)
    sp = sc.species[0]
    m = po.species_model(sc, sp, sc.roads[0], sem=sem)
    P, Y = 2000, 50
    end, st = sg.simulateMTECUDA([m], [sp.params], P, Y, seed=0, road=0, sem=sem,
                                 migration=mig, ctx=ctx)
    ref = po.simulate_mte(P, Y, m["N"], 1.0, sp.params, m["init_pops"], m["caps"], m["mmm"][2],
                          0, 0, 0, sem, threads=16)
    assert np.array_equal(end[:, 0].astype(np.float32), ref)
    e = ref.astype(np.float64)
    assert math.isclose(st[0]["mean"], e.mean(), rel_tol=1e-12)
    thr = 0.2 * m["init_pops"].astype(np.float64).sum()
    assert math.isclose(st[0]["p_below"], float((e < thr).mean()))


def test_plain_rov_full_shape(ctx):
    """10^4 paths x 50 years, 2 species, 3 processes, 3 controls, 16 bins
    per state dimension, corrected semantics, sparse migration: identical
    decisions and continuation values, identical regression surfaces."""
    from test_gpu_rov import _compare_exact
    sc = synth.rov_road(0, n_species=2)
    models = [po.species_model(sc, sc.species[s], sc.roads[0], sem=1) for s in range(2)]
    P, Y = 10000, 50
    rp = rov_problem_from_models(models, sc, n_paths=P, n_years=Y, dim_res=16, sem=1,
                                 n_processes=3, demand=True)
    gpu = sg.simulateROVCUDA(rp, migration=MIG_SPARSE_FP32, ctx=ctx)
    orc = po.simulate_rov(rp, threads=16)
    assert np.isfinite(orc["stats"][0])
    _compare_exact(gpu, orc, P, Y, 2)
