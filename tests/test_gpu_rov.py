"""GPU ROV valuation (ALGO4) and kNN against the oracle (SIMT path: bit for
bit on identical inputs) and against the reference's golden outputs."""
import math

import numpy as np
import pytest

from oracle import pyoracle as po
from rov_util import problem_from_golden, ref_outputs
from transportoptimiser_gb300 import simulate_gpu as sg
from transportoptimiser_gb300 import synth
from transportoptimiser_gb300._capi import MIG_SIMT_FP32, MIG_SPARSE_FP32
from transportoptimiser_gb300.rov import rov_problem_from_models

MIGS = [MIG_SIMT_FP32, MIG_SPARSE_FP32]

pytestmark = pytest.mark.gpu


def _compare_exact(gpu, orc, P, Y, S):
    assert np.array_equal(gpu["opt_cont"], orc["opt_cont"])
    assert np.array_equal(gpu["cond_exp"].astype(np.float32), orc["cond_exp"])
    assert np.array_equal(gpu["unit_profits"].astype(np.float32)[P:], orc["unit_profits"][P:])
    assert np.array_equal(gpu["adj_pops"].astype(np.float32).reshape(Y, S, P)[1:],
                          orc["adj_pops"].reshape(Y, S, P)[1:])
    assert np.array_equal(gpu["regression"].astype(np.float32), orc["regression"])
    assert gpu["stats"][1] == orc["stats"][1]
    assert math.isclose(gpu["stats"][0], orc["stats"][0], rel_tol=1e-7)
    assert math.isclose(gpu["stats"][2], orc["stats"][2], rel_tol=1e-9)
    assert math.isclose(gpu["value_se"], orc["value_se"], rel_tol=1e-9)


@pytest.mark.parametrize("mig", MIGS)
def test_rov_reference_semantics_bit_exact(ctx, golden, mig):
    rp = problem_from_golden(golden["rov"])
    gpu = sg.simulateROVCUDA(rp, migration=mig, ctx=ctx)
    orc = po.simulate_rov(rp)
    _compare_exact(gpu, orc, rp["n_paths"], rp["n_years"], 1)


@pytest.mark.parametrize("case", ["rov", "rov_y50"])
def test_rov_matches_reference_golden(ctx, golden, case):
    g = golden[case]
    rp = problem_from_golden(g)
    ref = ref_outputs(g)
    gpu = sg.simulateROVCUDA(rp, ctx=ctx)
    assert np.array_equal(gpu["opt_cont"], ref["opt_cont"])
    assert abs(gpu["stats"][0] - ref["stats"][0]) <= 1e-5 * abs(ref["stats"][0])
    assert np.abs(gpu["regression"] - ref["regression"]).max() <= 1e-5 * np.abs(ref["regression"]).max()


@pytest.mark.parametrize("mig", MIGS)
@pytest.mark.parametrize("S,R,P,Y", [(2, 8, 900, 10), (1, 16, 1500, 8), (2, 8, 700, 50)])
def test_rov_corrected_semantics_bit_exact(ctx, S, R, P, Y, mig):
    sc = synth.rov_road(3, n_species=S)
    models = [po.species_model(sc, sc.species[s], sc.roads[0], sem=1) for s in range(S)]
    rp = rov_problem_from_models(models, sc, n_paths=P, n_years=Y, dim_res=R, sem=1,
                                 n_processes=3, demand=True, seed=4, road=7)
    gpu = sg.simulateROVCUDA(rp, migration=mig, ctx=ctx)
    orc = po.simulate_rov(rp, threads=8)
    assert np.isfinite(orc["stats"][0])
    _compare_exact(gpu, orc, P, Y, S)


def test_rov_independent_seeds(ctx):
    """Independent seeds agree within 3 standard errors.  The value is a
    regression (LSM) estimate, so its standard error is measured by
    replication: two groups of independent runs at different path counts."""
    sc = synth.mte_road(1)
    m = po.species_model(sc, sc.species[0], sc.roads[0], sem=0)
    groups = []
    for P, seeds in ((2000, range(100, 106)), (4000, range(200, 206))):
        v = []
        for seed in seeds:
            rp = rov_problem_from_models([m], sc, n_paths=P, n_years=15, dim_res=8, seed=seed)
            out = sg.simulateROVCUDA(rp, want=(), ctx=ctx)
            assert out["value_se"] > 0
            v.append(out["stats"][0])
        groups.append(np.array(v))
    a, b = groups
    se = math.sqrt(a.var(ddof=1) / len(a) + b.var(ddof=1) / len(b))
    assert abs(a.mean() - b.mean()) < 3 * se


def test_knn_matches_oracle_and_reference(ctx, golden):
    g = golden["knn"]
    k = int(g["k"])
    dist, ind = sg.knn(g["ref"], g["query"], k, ctx=ctx)
    od, oi = po.knn(g["ref"], g["ref"].shape[1], g["query"], g["query"].shape[1], 3, k)
    assert np.array_equal(ind.reshape(-1), oi)
    assert np.array_equal(dist.reshape(-1), od)
    assert np.array_equal(ind.reshape(-1), g["ind"])
    rng = np.random.default_rng(5)
    for n, Q, dim, k in [(5000, 300, 4, 100), (40, 17, 1, 40), (3000, 64, 2, 256)]:
        ref_pts = rng.integers(0, 20, (dim, n)).astype(np.float32)   # many exact ties
        q = rng.random((dim, Q)).astype(np.float32) * 20
        dist, ind = sg.knn(ref_pts, q, k, ctx=ctx)
        od, oi = po.knn(ref_pts, n, q, Q, dim, k)
        assert np.array_equal(ind.reshape(-1), oi)
        assert np.array_equal(dist.reshape(-1), od)


def test_rov_many_chunks_repeatable_and_exact(ctx):
    """Paths compacted in many chunks (20,000 paths = 20 chunks of 1024) over
    50 years: repeated valuations agree bit for bit; a 12,000-path, 10-year
    case matches the oracle exactly (regression coefficients, continuation
    values, decisions)."""
    sc = synth.rov_road(0, n_species=2)
    models = [po.species_model(sc, sc.species[s], sc.roads[0], sem=1) for s in range(2)]
    rp = rov_problem_from_models(models, sc, n_paths=20000, n_years=50, dim_res=16, sem=1,
                                 n_processes=3, demand=True)
    runs = [sg.simulateROVCUDA(rp, want=("regression", "cond_exp"), ctx=ctx) for _ in range(3)]
    for r in runs[1:]:
        assert r["stats"][0] == runs[0]["stats"][0]
        assert np.array_equal(r["regression"], runs[0]["regression"])
        assert np.array_equal(r["cond_exp"], runs[0]["cond_exp"])
    P, Y = 12000, 10
    rp = rov_problem_from_models(models, sc, n_paths=P, n_years=Y, dim_res=16, sem=1,
                                 n_processes=3, demand=True, seed=11)
    gpu = sg.simulateROVCUDA(rp, ctx=ctx)
    orc = po.simulate_rov(rp, threads=16)
    _compare_exact(gpu, orc, P, Y, 2)


@pytest.mark.parametrize("S,R,P,Y", [(2, 8, 700, 10), (1, 16, 900, 8), (2, 8, 1100, 25)])
def test_rov_algo6_bit_exact(ctx, S, R, P, Y):
    """ALGO6: every path re-simulated from each year under the regression-
    optimal controls; values, decisions and regressions equal the oracle's."""
    sc = synth.rov_road(3, n_species=S)
    models = [po.species_model(sc, sc.species[s], sc.roads[0], sem=1) for s in range(S)]
    rp = rov_problem_from_models(models, sc, n_paths=P, n_years=Y, dim_res=R, sem=1,
                                 n_processes=3, demand=True, seed=4, road=7, algo=6)
    gpu = sg.simulateROVCUDA(rp, migration=MIG_SPARSE_FP32, ctx=ctx)
    orc = po.simulate_rov(rp, threads=16)
    assert np.isfinite(orc["stats"][0])
    _compare_exact(gpu, orc, P, Y, S)


def test_rov_algo6_refuses_dense_forms(ctx):
    from transportoptimiser_gb300._capi import TransOptError
    sc = synth.rov_road(3, n_species=1)
    models = [po.species_model(sc, sc.species[0], sc.roads[0], sem=1)]
    rp = rov_problem_from_models(models, sc, n_paths=200, n_years=6, dim_res=8, sem=1, algo=6)
    with pytest.raises(TransOptError):
        sg.simulateROVCUDA(rp, migration=MIG_SIMT_FP32, ctx=ctx)


def test_rov_batch_equals_single_roads(ctx):
    """Three roads of one scene valued in one batch (chunks of the
    compaction straddle roads: 700 paths each) give each road exactly the
    single-road results."""
    sc = synth.rov_road(3, n_species=2)
    rng = np.random.Generator(np.random.Philox(5))
    roads = [sc.roads[0]] + [synth.random_road(sc.W, sc.H, n, rng) for n in (6, 12)]
    probs = []
    for i, rd in enumerate(roads):
        models = [po.species_model(sc, sc.species[s], rd, sem=1) for s in range(2)]
        probs.append(rov_problem_from_models(models, sc, n_paths=700, n_years=12, dim_res=8,
                                             sem=1, n_processes=3, demand=True, seed=4,
                                             road=10 + i))
    assert len({p["species"][0]["N"] for p in probs}) > 1      # different patch sets
    want = ("cond_exp", "opt_cont", "regression", "unit_profits", "adj_pops")
    batch = sg.simulateROVCUDA_batch(probs, want=want, ctx=ctx)
    for p, b in zip(probs, batch):
        one = sg.simulateROVCUDA(p, want=want, ctx=ctx)
        for k in want:
            assert np.array_equal(b[k], one[k]), k
        assert np.array_equal(b["stats"], one["stats"])
        assert b["value_se"] == one["value_se"]


def test_rov_batch_edges(ctx):
    """Ragged path tiles (130 paths per road), a batch of one road, and the
    refusals: roads that differ in a shared setting, too few paths per road."""
    from transportoptimiser_gb300._capi import TransOptError
    sc = synth.rov_road(3, n_species=1)
    rng = np.random.Generator(np.random.Philox(9))
    roads = [sc.roads[0], synth.random_road(sc.W, sc.H, 9, rng)]
    models = [[po.species_model(sc, sc.species[0], rd, sem=1)] for rd in roads]

    def prob(m, P, Y=8, road=0):
        return rov_problem_from_models(m, sc, n_paths=P, n_years=Y, dim_res=8, sem=1,
                                       n_processes=3, demand=True, seed=2, road=road)
    want = ("cond_exp", "opt_cont", "regression")
    probs = [prob(m, 130, road=i) for i, m in enumerate(models)]
    for p, b in zip(probs, sg.simulateROVCUDA_batch(probs, want=want, ctx=ctx)):
        one = sg.simulateROVCUDA(p, want=want, ctx=ctx)
        for k in want:
            assert np.array_equal(b[k], one[k]), k
        assert np.array_equal(b["stats"], one["stats"])
    single = sg.simulateROVCUDA_batch([prob(models[0], 60)], want=want, ctx=ctx)[0]
    one = sg.simulateROVCUDA(prob(models[0], 60), want=want, ctx=ctx)
    for k in want:
        assert np.array_equal(single[k], one[k]), k
    with pytest.raises(TransOptError):
        sg.simulateROVCUDA_batch([prob(models[0], 130), prob(models[1], 130, Y=9)], ctx=ctx)
    with pytest.raises(TransOptError):
        sg.simulateROVCUDA_batch([prob(models[0], 64), prob(models[1], 64, road=1)], ctx=ctx)


@pytest.mark.parametrize("S,R,P,Y", [(2, 16, 3000, 50), (1, 8, 900, 20)])
def test_rov_touched_queries_match_full_grid(ctx, S, R, P, Y):
    """Without the regression surfaces in the output, each year's regressions
    are fitted only at the grid queries the backward pass reads.  Decisions,
    continuation values, the road value and its statistics stay identical
    to the run that fits (and returns) the whole grid, and to the oracle."""
    sc = synth.rov_road(1, n_species=S)
    models = [po.species_model(sc, sc.species[s], sc.roads[0], sem=1) for s in range(S)]
    rp = rov_problem_from_models(models, sc, n_paths=P, n_years=Y, dim_res=R, sem=1,
                                 n_processes=3, demand=True, seed=21, road=3)
    full = sg.simulateROVCUDA(rp, migration=MIG_SPARSE_FP32, ctx=ctx)
    part = sg.simulateROVCUDA(rp, want=("cond_exp", "opt_cont", "unit_profits", "adj_pops"),
                              migration=MIG_SPARSE_FP32, ctx=ctx)
    for k in ("cond_exp", "opt_cont", "unit_profits", "adj_pops"):
        assert np.array_equal(full[k], part[k]), k
    assert np.array_equal(full["stats"], part["stats"])
    assert full["value_se"] == part["value_se"] and full["n_best"] == part["n_best"]
    orc = po.simulate_rov(rp, threads=16)
    assert np.array_equal(part["opt_cont"], orc["opt_cont"])
    assert np.array_equal(part["cond_exp"].astype(np.float32), orc["cond_exp"])


def test_rov_batch_touched_queries_match_full_grid(ctx):
    """The batched form (one road per (road, control) regression group) with
    and without the surfaces: identical results for every road."""
    sc = synth.rov_road(0, n_species=2)
    rng = np.random.Generator(np.random.Philox(5))
    roads = [sc.roads[0]] + [synth.random_road(sc.W, sc.H, int(rng.integers(8, 40)), rng)
                             for _ in range(5)]
    probs = []
    for i, rd in enumerate(roads):
        ms = [po.species_model(sc, sp, rd, sem=1) for sp in sc.species]
        probs.append(rov_problem_from_models(ms, sc, n_paths=640, n_years=30, dim_res=16, sem=1,
                                             n_processes=3, demand=True, road=10 + i))
    full = sg.simulateROVCUDA_batch(probs, ctx=ctx)
    part = sg.simulateROVCUDA_batch(probs, want=("cond_exp", "opt_cont"), ctx=ctx)
    for f, p in zip(full, part):
        assert np.array_equal(f["cond_exp"], p["cond_exp"])
        assert np.array_equal(f["opt_cont"], p["opt_cont"])
        assert np.array_equal(f["stats"], p["stats"])
        assert f["value_se"] == p["value_se"]
