"""The oracle against the reference's own kernels.

tests/golden/*.npz hold outputs of the reference kernels compiled for the
CPU (oracle/build_ref.sh, tests/golden/make_golden.py).  Integer results must
match exactly; floating-point results within 1e-5 relative (the reference
kernels run there without fused multiply-adds, the oracle with them)."""
import math

import numpy as np
import pytest

from oracle import pyoracle as po
from transportoptimiser_gb300 import synth

RTOL = 1e-5


@pytest.mark.parametrize("case", ["patches_crossings", "patches_crossings_gen"])
def test_labels_patches_crossings_golden(golden, case):
    g = golden[case]
    W = int(g["W"]); res = int(g["res"])
    hab, popm = g["hab"], g["pop_map"]
    xres = res if W % res == 0 else res + 1
    skp = (W - 1) // res
    area, cx, cy, pop, cap = [], [], [], [], []
    for t, typ in enumerate(g["types"]):
        lab, nr = po.label_image(W, W, (hab == typ).astype(np.int32))
        assert nr == int(g["nregs"][t])
        assert np.array_equal(lab, g["labels"][t])
        r = po.build_patches(W, W, skp, skp, xres, xres, nr, 1.0, 1.0, 1.0, 50.0, lab, popm)
        area.append(r["area"]); cx.append(r["cx"]); cy.append(r["cy"])
        pop.append(r["pop"]); cap.append(r["cap"])
    for k, v in (("area", area), ("cx", cx), ("cy", cy), ("pop", pop), ("cap", cap)):
        assert np.array_equal(np.concatenate(v), g[k]), k
    cr = po.line_segment_intersect(g["xy1"], len(g["pairs"]), g["road"], int(g["G"]))
    assert np.array_equal(cr, g["pair_crossings"])


@pytest.mark.parametrize("case,scene", [("patches_crossings", lambda: synth.mte_road(0)),
                                        ("patches_crossings_gen",
                                         lambda: synth.generation(0, n_roads=1))])
def test_species_model_crossing_matrix_golden(golden, case, scene):
    g = golden[case]
    sc = scene()
    m = po.species_model(sc, sc.species[0], sc.roads[0], sem=0, max_patches=1024)
    N = m["N"]
    Cm = np.zeros((N, N), np.int32)
    for q, (i, j) in enumerate(g["pairs"]):
        Cm[i, j] = Cm[j, i] = g["pair_crossings"][q]
    assert np.array_equal(Cm, m["crossings"])
    # rows of the transition matrix are normalised
    assert np.allclose(m["trans"].sum(axis=1), 1.0, rtol=1e-12)


@pytest.mark.parametrize("case", ["mte", "mte_y50", "mte_gen"])
def test_mte_golden(golden, case):
    g = golden[case]
    out = po.simulate_mte(int(g["P"]), int(g["Y"]), int(g["N"]), 1.0, g["params"], g["init"],
                          g["caps"], g["mmm"], int(g["seed"]), 0, 0, 0)
    np.testing.assert_allclose(out, g["end"], rtol=RTOL)


def test_exppv_golden(golden):
    g = golden["exppv"]
    vals, m, s = po.exp_pv(int(g["P"]), int(g["Y"]), g["prm"], int(g["seed"]), 0, 0)
    np.testing.assert_allclose(vals, g["values"], rtol=RTOL)
    assert math.isclose(m, float(g["mean"]), rel_tol=RTOL)
    assert math.isclose(s, float(g["sd"]), rel_tol=RTOL)


@pytest.mark.skipif(not po.ref_available(), reason="reference tree not mounted")
def test_oracle_vs_reference_kernels_live():
    """Against the live reference build (only where the reference is mounted)."""
    sc = synth.mte_road(3)
    sp, road = sc.species[0], sc.roads[0]
    m = po.species_model(sc, sp, road, sem=0)
    a = po.simulate_mte(100, 50, m["N"], 1.0, sp.params, m["init_pops"], m["caps"],
                        m["mmm"][2], 7, 0, 0, 0)
    b = po.ref_simulate_mte(100, 50, m["N"], 1.0, sp.params, m["init_pops"], m["caps"],
                            m["mmm"][2], 7, 0, 0)
    np.testing.assert_allclose(a, b, rtol=RTOL)
