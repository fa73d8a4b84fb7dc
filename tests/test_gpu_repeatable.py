"""Repeated calls on the same inputs give the same bits, at the sizes the
benchmark runs (many CTAs, many waves).  The bit-exact oracle tests run at
small sizes; a missing barrier shows up only when warps of one CTA drift
apart, which needs long launches."""
import numpy as np
import pytest

from oracle import pyoracle as po
from transportoptimiser_gb300 import simulate_gpu as sg
from transportoptimiser_gb300 import synth
from transportoptimiser_gb300._capi import (MIG_AUTO, MIG_SIMT_FP32, MIG_SPARSE_FP32,
                                            MIG_TC_3XTF32)
from transportoptimiser_gb300.generation import Generation, pack_roads
from transportoptimiser_gb300.rov import rov_problem_from_models

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("mig", [MIG_SPARSE_FP32, MIG_SIMT_FP32, MIG_TC_3XTF32, MIG_AUTO])
def test_generation_of_256_roads_repeatable(ctx, mig):
    sc = synth.generation(0, n_roads=256)
    gen = Generation(sc, max_roads=256, max_patches=512, ctx=ctx)
    packed = pack_roads(sc, sc.roads)
    opts = gen.opts(1024, 50, seed=2, migration=mig)
    a = gen.evaluate(packed, opts)
    b = gen.evaluate(packed, opts)
    gen.close()
    C = sc.n_controls
    # slots 10..14 (no ROV) and the animals-at-risk slots past C are NaN
    assert np.isfinite(a[:, :, :10]).all() and np.isfinite(a[:, :, 16:16 + C]).all()
    assert np.array_equal(a, b, equal_nan=True)


def test_single_road_mte_many_paths_repeatable(ctx):
    sc = synth.mte_road(0)
    m = po.species_model(sc, sc.species[0], sc.roads[0], sem=0)
    runs = [sg.simulateMTECUDA([m], [sc.species[0].params], 40000, 50, seed=3, road=1,
                               migration=MIG_SPARSE_FP32, ctx=ctx) for _ in range(2)]
    assert np.array_equal(runs[0][0], runs[1][0])
    assert runs[0][1][0]["mean"] == runs[1][1][0]["mean"]


def test_adjoint_many_paths_repeatable(ctx):
    from transportoptimiser_gb300.adjoint import FrozenPolicy, theta_from_problem
    sc = synth.rov_road(0, n_species=2)
    models = [po.species_model(sc, sc.species[s], sc.roads[0], sem=1) for s in range(2)]
    rp = rov_problem_from_models(models, sc, n_paths=20000, n_years=50, dim_res=16, sem=1,
                                 n_processes=3, demand=True)
    rov = sg.simulateROVCUDA(rp, want=("opt_cont",), ctx=ctx)
    ctl = rov["opt_cont"].reshape(rp["n_years"], rp["n_paths"]).astype(np.int32)
    hz = np.asarray(sc.species[0].hazard, np.float64)
    fp = FrozenPolicy(rp, ctl, [m["crossings"] for m in models], hz, ctx)
    th = theta_from_problem(rp, hz)
    o1, J1 = fp.jacobian(th)
    o2, J2 = fp.jacobian(th)
    assert np.array_equal(o1, o2)
    assert np.array_equal(J1, J2)
