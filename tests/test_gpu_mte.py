"""GPU MTE and expected-PV against the oracle (SIMT path bit-exact) and
against the reference kernels' golden outputs (1e-5 relative)."""
import math

import numpy as np
import pytest

from oracle import pyoracle as po
from transportoptimiser_gb300 import simulate_gpu as sg
from transportoptimiser_gb300 import synth
from transportoptimiser_gb300._capi import MIG_SIMT_FP32, MIG_SPARSE_FP32, TransOptError

MIGS = [MIG_SIMT_FP32, MIG_SPARSE_FP32]

pytestmark = pytest.mark.gpu
RTOL = 1e-5


def _model(sc, s=0):
    return po.species_model(sc, sc.species[s], sc.roads[0], sem=0)


@pytest.mark.parametrize("mig", MIGS)
@pytest.mark.parametrize("sem", [0, 1])
def test_mte_simt_bit_exact_vs_oracle(ctx, sem, mig):
    sc = synth.mte_road(0)
    sp = sc.species[0]
    m = _model(sc)
    P, Y = 300, 50
    end, st = sg.simulateMTECUDA([m], [sp.params], P, Y, seed=11, road=2, sem=sem,
                                 migration=mig, ctx=ctx)
    ref = po.simulate_mte(P, Y, m["N"], 1.0, sp.params, m["init_pops"], m["caps"], m["mmm"][2],
                          11, 2, 0, sem)
    assert np.array_equal(end[:, 0].astype(np.float32), ref)
    e = ref.astype(np.float64)
    assert math.isclose(st[0]["mean"], e.mean(), rel_tol=1e-12)
    assert math.isclose(st[0]["sd"], e.std(), rel_tol=1e-9)
    assert math.isclose(st[0]["p_below"], float((e < 0.2 * m["init_pops"].astype(np.float64).sum()).mean()))


@pytest.mark.parametrize("case", ["mte", "mte_y50", "mte_gen"])
@pytest.mark.parametrize("mig", MIGS)
def test_mte_matches_reference_golden(ctx, golden, mig, case):
    g = golden[case]
    m = dict(N=int(g["N"]), init_pops=g["init"], caps=g["caps"], mmm=g["mmm"][None])
    end, _ = sg.simulateMTECUDA([m], [g["params"]], int(g["P"]), int(g["Y"]), seed=int(g["seed"]),
                                road=0, sem=0, migration=mig, control=0, ctx=ctx)
    np.testing.assert_allclose(end[:, 0], g["end"], rtol=RTOL)


@pytest.mark.parametrize("mig", MIGS)
def test_mte_multi_species_and_padding(ctx, mig):
    sc = synth.rov_road(2, n_species=2)
    ms = [po.species_model(sc, sc.species[s], sc.roads[0], sem=0) for s in range(2)]
    # give species 1 a different patch count by dropping patches
    m1 = dict(ms[1])
    n = m1["N"] - 5
    m1.update(N=n, init_pops=m1["init_pops"][:n], caps=m1["caps"][:n],
              mmm=np.ascontiguousarray(m1["mmm"][:, :n, :n]))
    P, Y = 150, 20
    end, _ = sg.simulateMTECUDA([ms[0], m1], [sc.species[0].params, sc.species[1].params], P, Y,
                                seed=3, road=1, migration=mig, ctx=ctx)
    for s, m in enumerate([ms[0], m1]):
        ref = po.simulate_mte(P, Y, m["N"], 1.0, sc.species[s].params, m["init_pops"], m["caps"],
                              m["mmm"][2], 3, 1, s, 0)
        assert np.array_equal(end[:, s].astype(np.float32), ref), s


def test_mte_independent_seeds_agree(ctx):
    sc = synth.mte_road(0)
    m = _model(sc)
    P = 4000
    _, a = sg.simulateMTECUDA([m], [sc.species[0].params], P, 50, seed=1, ctx=ctx)
    _, b = sg.simulateMTECUDA([m], [sc.species[0].params], P, 50, seed=2, ctx=ctx)
    se = math.hypot(a[0]["se"], b[0]["se"])
    assert abs(a[0]["mean"] - b[0]["mean"]) < 3 * se


def test_mte_rejects_nonfinite(ctx):
    sc = synth.mte_road(0)
    m = dict(_model(sc))
    bad = m["init_pops"].copy()
    bad[3] = np.nan
    m["init_pops"] = bad
    with pytest.raises(TransOptError) as e:
        sg.simulateMTECUDA([m], [sc.species[0].params], 10, 5, ctx=ctx)
    assert e.value.status == 4


@pytest.mark.parametrize("sem", [0, 1])
def test_exppv_bit_exact_and_golden(ctx, golden, sem):
    g = golden["exppv"]
    prm = g["prm"]
    m, s, vals = sg.expPV(*[float(x) for x in prm], int(g["P"]), int(g["Y"]), seed=int(g["seed"]),
                          sem=sem, return_values=True, ctx=ctx)
    ov, om, osd = po.exp_pv(int(g["P"]), int(g["Y"]), prm, int(g["seed"]), 0, sem)
    assert np.array_equal(vals, ov)
    assert math.isclose(m, om, rel_tol=1e-12) and math.isclose(s, osd, rel_tol=1e-9)
    if sem == 0:
        np.testing.assert_allclose(vals, g["values"], rtol=RTOL)
