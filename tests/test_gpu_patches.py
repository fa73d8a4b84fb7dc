"""GPU labels, patches, crossings and species model against the oracle:
integer results bit-exact, FP64 probabilities to 1e-12."""
import math

import numpy as np
import pytest

from oracle import pyoracle as po
from transportoptimiser_gb300 import simulate_gpu as sg
from transportoptimiser_gb300 import synth
from transportoptimiser_gb300._capi import TransOptError

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("W,H,p,seed", [(64, 64, 0.55, 0), (200, 200, 0.6, 1), (37, 37, 0.5, 2),
                                        (1, 1, 1.0, 3), (16, 16, 0.0, 4), (128, 128, 0.59, 5)])
def test_label_image_matches_oracle(ctx, W, H, p, seed):
    rng = np.random.default_rng(seed)
    inp = (rng.random(W * H) < p).astype(np.int32)
    a, na = sg.labelImage(W, H, inp, ctx=ctx)
    b, nb = po.label_image(W, H, inp)
    assert na == nb
    assert np.array_equal(a, b)


def test_label_image_too_large_is_rejected(ctx):
    with pytest.raises(TransOptError):
        sg.labelImage(400, 400, np.ones(400 * 400, np.int32), ctx=ctx)


@pytest.mark.parametrize("case", ["patches_crossings", "patches_crossings_gen"])
def test_build_patches_matches_golden(ctx, golden, case):
    g = golden[case]
    W = int(g["W"]); res = int(g["res"])
    xres = res if W % res == 0 else res + 1
    skp = (W - 1) // res
    hab, popm = g["hab"], g["pop_map"]
    got = {k: [] for k in ("area", "cap", "pop", "cx", "cy")}
    for t, typ in enumerate(g["types"]):
        lab, nr = sg.labelImage(W, W, (hab == typ).astype(np.int32), ctx=ctx)
        assert np.array_equal(lab, g["labels"][t])
        r, _ = sg.buildPatches(W, W, skp, skp, xres, xres, nr, 1.0, 1.0, 1.0, 50.0, lab, popm,
                               ctx=ctx)
        for k in got:
            got[k].append(r[k])
    for k in got:
        assert np.array_equal(np.concatenate(got[k]), g[k]), k


@pytest.mark.parametrize("case", ["patches_crossings", "patches_crossings_gen"])
def test_line_segment_intersect_matches_oracle(ctx, golden, case):
    g = golden[case]
    T = len(g["pairs"])
    xy1 = g["xy1"].reshape(4, T).T
    xy2 = g["road"].reshape(4, int(g["G"])).T
    cr = sg.lineSegmentIntersect(xy1, xy2, ctx=ctx)
    assert np.array_equal(cr, g["pair_crossings"])
    rng = np.random.default_rng(3)
    a = rng.uniform(0, 100, (5000, 4))
    b = rng.uniform(0, 100, (40, 4))
    c1 = sg.lineSegmentIntersect(a, b, ctx=ctx)
    c2 = po.line_segment_intersect(a.T.reshape(-1).copy(), 5000, b.T.reshape(-1).copy(), 40)
    assert np.array_equal(c1, c2)


def _gpu_model(ctx, sc, sp, road, sem):
    hab = sc.hab_map(road)
    return sg.createSpeciesModel(hab, sc.pop_map(sp, hab), sc.W, sc.H, sc.res, sp.habitats,
                                 road.colmajor(), road.G, sp.hazard, sp.lambda_mean,
                                 sp.lambda_sd, sp.lambda_mult, sp.hab_pref_mult, sem=sem,
                                 ctx=ctx)


@pytest.mark.parametrize("maker,seed,sem", [(synth.mte_road, 0, 0), (synth.mte_road, 5, 1),
                                            (synth.rov_road, 1, 0)])
def test_species_model_matches_oracle(ctx, maker, seed, sem):
    sc = maker(seed)
    sp, road = sc.species[0], sc.roads[0]
    a = _gpu_model(ctx, sc, sp, road, sem)
    b = po.species_model(sc, sp, road, sem=sem)
    assert a["N"] == b["N"] and a["n_transitions"] == b["n_transitions"]
    for k in ("area", "cap", "pop", "cx", "cy", "type"):
        assert np.array_equal(a[k], b[k]), k
    assert np.array_equal(a["crossings"], b["crossings"])
    np.testing.assert_allclose(a["trans"], b["trans"], rtol=1e-12, atol=1e-300)
    np.testing.assert_allclose(a["surv"], b["surv"], rtol=1e-12)
    # float migration matrices: identical up to a one-ulp FP64 exp difference
    diff = np.abs(a["mmm"].astype(np.float64) - b["mmm"]) / np.maximum(np.abs(b["mmm"]), 1e-30)
    assert diff.max() <= 1.2e-7
