"""Edge cases of the path against the oracle: degenerate and maximal label
images, empty and degenerate line sets, the smallest population problems,
one-road generations."""
import numpy as np
import pytest

from oracle import pyoracle as po
from transportoptimiser_gb300 import simulate_gpu as sg
from transportoptimiser_gb300 import synth
from transportoptimiser_gb300._capi import MIG_SIMT_FP32, MIG_SPARSE_FP32
from transportoptimiser_gb300.generation import Generation, pack_roads

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", ["checkerboard", "all_foreground", "stripes", "one_row", "largest"])
def test_label_image_degenerate_and_largest(ctx, name):
    if name == "checkerboard":          # every foreground pixel its own region
        W = H = 64
        inp = ((np.arange(W)[None, :] + np.arange(H)[:, None]) % 2).astype(np.int32).ravel()
    elif name == "all_foreground":      # one region over the whole image
        W = H = 200
        inp = np.ones(W * H, np.int32)
    elif name == "stripes":             # one region per row
        W = H = 97
        inp = np.tile((np.arange(H) % 2).astype(np.int32)[:, None], (1, W)).ravel()
    elif name == "one_row":
        W, H = 50000, 1
        inp = (np.random.default_rng(5).random(W * H) < 0.5).astype(np.int32)
    else:                               # the largest square image shared memory holds
        W = H = 240
        inp = (np.random.default_rng(3).random(W * H) < 0.59).astype(np.int32)
    a, na = sg.labelImage(W, H, inp, ctx=ctx)
    b, nb = po.label_image(W, H, inp)
    assert na == nb
    assert np.array_equal(a, b)
    if name == "checkerboard":
        assert na == W * H // 2
    if name == "all_foreground":
        assert na == 1


def _cm(a):
    return np.ascontiguousarray(np.asarray(a, np.float64).T.reshape(-1))


def test_line_segment_intersect_empty_and_degenerate(ctx):
    road = np.array([[0.0, 0.0, 20.0, 0.0], [20.0, 0.0, 30.0, 10.0]])   # G x 4: x1, y1, x2, y2
    rng = np.random.default_rng(4)
    lines = rng.uniform(-5.0, 35.0, (64, 4))
    lines[0] = [0.0, 1.0, 20.0, 1.0]       # parallel to the first segment
    lines[1] = [0.0, 0.0, 20.0, 0.0]       # collinear with it
    lines[2] = [5.0, 5.0, 5.0, 5.0]        # a point
    lines[3] = [10.0, -3.0, 10.0, 0.0]     # ends on the first segment
    lines[4] = [20.0, 0.0, 20.0, -4.0]     # starts at the shared vertex
    a = sg.lineSegmentIntersect(lines, road, ctx=ctx)
    b = po.line_segment_intersect(_cm(lines), len(lines), _cm(road), len(road))
    assert np.array_equal(a, b)
    assert a[0] == 0
    # no lines, and no road segments
    assert len(sg.lineSegmentIntersect(np.zeros((0, 4)), road, ctx=ctx)) == 0
    z = sg.lineSegmentIntersect(lines, np.zeros((0, 4)), ctx=ctx)
    assert np.array_equal(z, np.zeros(len(lines), np.int32))


@pytest.mark.parametrize("mig", [MIG_SIMT_FP32, MIG_SPARSE_FP32])
@pytest.mark.parametrize("P,Y", [(1, 1), (1, 50), (33, 2)])
def test_mte_smallest_problems(ctx, mig, P, Y):
    sc = synth.mte_road(0)
    sp = sc.species[0]
    m = po.species_model(sc, sp, sc.roads[0], sem=0)
    end, st = sg.simulateMTECUDA([m], [sp.params], P, Y, seed=5, road=1, sem=1,
                                 migration=mig, ctx=ctx)
    ref = po.simulate_mte(P, Y, m["N"], 1.0, sp.params, m["init_pops"], m["caps"], m["mmm"][2],
                          5, 1, 0, 1)
    assert np.array_equal(end[:, 0].astype(np.float32), ref)


@pytest.mark.parametrize("mig", [MIG_SIMT_FP32, MIG_SPARSE_FP32])
def test_mte_one_patch(ctx, mig):
    sp = synth.mte_road(0).species[0]
    C = 3
    m = {"N": 1, "init_pops": np.array([40.0], np.float32), "caps": np.array([60.0], np.float32),
         "mmm": np.tile(np.array([[[0.9]]], np.float32), (C, 1, 1))}
    end, _ = sg.simulateMTECUDA([m], [sp.params], 64, 30, seed=2, road=0, sem=1,
                                migration=mig, ctx=ctx)
    ref = po.simulate_mte(64, 30, 1, 1.0, sp.params, m["init_pops"], m["caps"], m["mmm"][2],
                          2, 0, 0, 1)
    assert np.array_equal(end[:, 0].astype(np.float32), ref)


def _roads():
    sc = synth.mte_road(0)
    empty = synth.Road(points=np.zeros((0, 2)), segments=np.zeros((0, 4)))
    one = synth.Road(points=np.array([[3.0, 20.0], [60.0, 21.0]]),
                     segments=np.array([[3.0, 20.0, 60.0, 21.0]]))
    return sc, {"empty": empty, "one_segment": one, "polyline": sc.roads[0]}


@pytest.mark.parametrize("kind", ["empty", "one_segment"])
def test_species_model_of_empty_and_one_segment_roads(ctx, kind):
    sc, roads = _roads()
    sp, road = sc.species[0], roads[kind]
    hab = sc.hab_map(road)
    a = sg.createSpeciesModel(hab, sc.pop_map(sp, hab), sc.W, sc.H, sc.res, sp.habitats,
                              road.colmajor(), road.G, sp.hazard, sp.lambda_mean, sp.lambda_sd,
                              sp.lambda_mult, sp.hab_pref_mult, sem=0, ctx=ctx)
    b = po.species_model(sc, sp, road, sem=0)
    assert a["N"] == b["N"] and a["n_transitions"] == b["n_transitions"]
    for k in ("area", "cap", "pop", "cx", "cy", "type", "crossings"):
        assert np.array_equal(a[k], b[k]), k
    if kind == "empty":
        assert not a["crossings"].any()


@pytest.mark.parametrize("kinds", [("polyline",), ("empty",), ("one_segment",),
                                   ("empty", "polyline", "empty", "one_segment")])
def test_generation_with_one_road_and_empty_roads(ctx, kinds):
    """One-road generations and generations holding roads without segments
    give what the single-road calls give for each road."""
    sc, roads = _roads()
    rds = [roads[k] for k in kinds]
    sc.roads = rds
    gen = Generation(sc, max_roads=len(rds), max_patches=256, ctx=ctx)
    P, Y = 64, 20
    res = gen.evaluate(pack_roads(sc, rds), gen.opts(P, Y, seed=3, road0=7,
                                                     migration=MIG_SPARSE_FP32))
    gen.close()
    for r, rd in enumerate(rds):
        m = po.species_model(sc, sc.species[0], rd, sem=0)
        assert int(res[r, 0, 0]) == m["N"]
        assert int(res[r, 0, 1]) == m["n_transitions"]
        _, st = sg.simulateMTECUDA([m], [sc.species[0].params], P, Y, seed=3, road=7 + r,
                                   migration=MIG_SPARSE_FP32, ctx=ctx)
        assert res[r, 0, 2] == st[0]["mean"]
