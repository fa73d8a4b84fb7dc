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


def test_autotuner_records_choice_and_matches_that_kernel(ctx):
    from transportoptimiser_gb300._capi import MIG_TC_3XTF32
    sc = synth.generation(2, n_roads=8)
    gen = Generation(sc, max_roads=8, max_patches=512, ctx=ctx)
    packed = pack_roads(sc, sc.roads)
    auto = gen.evaluate(packed, gen.opts(64, 20, seed=4, migration=MIG_AUTO))
    lines = [l for l in ctx.tuning().splitlines() if l.startswith("generation") and "paths=64" in l]
    assert lines, ctx.tuning()
    chosen = lines[-1].split("-> ")[1].split()[0]
    mig = {"sparse": MIG_SPARSE_FP32, "simt": MIG_SIMT_FP32, "tc": MIG_TC_3XTF32}[chosen]
    ref = gen.evaluate(packed, gen.opts(64, 20, seed=4, migration=mig))
    np.testing.assert_array_equal(auto[:, :, :7], ref[:, :, :7])
    gen.close()


def test_graph_replay_matches_direct_and_replans(ctx):
    sc = synth.generation(3, n_roads=48)
    gen = Generation(sc, max_roads=16, max_patches=512, ctx=ctx)
    # patch counts of every road (direct path), to build two generations
    # whose second one exceeds the plan captured on the first
    nmax = []
    for r0 in range(0, 48, 16):
        res = gen.evaluate(pack_roads(sc, sc.roads[r0:r0 + 16]), gen.opts(32, 5, seed=1))
        nmax += list(res[:, :, 0].max(axis=1))
    order = np.argsort(nmax)
    small = [sc.roads[i] for i in order[:16]]
    big = [sc.roads[i] for i in order[-16:]]
    assert max(nmax) > sorted(nmax)[15] + 16, "need a generation beyond the plan margin"
    for roads in (small, big):
        packed = pack_roads(sc, roads)
        direct = gen.evaluate(packed, gen.opts(64, 30, seed=7))
        g1 = gen.evaluate(packed, gen.opts(64, 30, seed=7, graph=True))
        g2 = gen.evaluate(packed, gen.opts(64, 30, seed=7, graph=True))
        np.testing.assert_array_equal(g1, direct)
        np.testing.assert_array_equal(g2, direct)
    # replay of the first generation's graph on the second generation's roads
    packed_s, packed_b = pack_roads(sc, small), pack_roads(sc, big)
    gen.evaluate(packed_s, gen.opts(64, 30, seed=7, graph=True))      # capture on small
    out = gen.evaluate(packed_b, gen.opts(64, 30, seed=7, graph=True))  # violates, re-plans
    np.testing.assert_array_equal(out, gen.evaluate(packed_b, gen.opts(64, 30, seed=7)))
    gen.close()


def test_device_form_reports_an_outgrown_plan_at_synchronize(ctx):
    """to_evaluate_roads_d replays the captured graph without reading anything
    back: roads beyond the plan captured on the first generation raise the
    device flag, which to_ctx_synchronize reports (TO_ERR_UNSUPPORTED) and
    clears."""
    import torch
    from transportoptimiser_gb300._capi import RESULT_STRIDE, TransOptError
    sc = synth.generation(3, n_roads=48)
    gen = Generation(sc, max_roads=16, max_patches=512, ctx=ctx)
    nmax = []
    for r0 in range(0, 48, 16):
        res = gen.evaluate(pack_roads(sc, sc.roads[r0:r0 + 16]), gen.opts(32, 5, seed=1))
        nmax += list(res[:, :, 0].max(axis=1))
    order = np.argsort(nmax)
    small = pack_roads(sc, [sc.roads[i] for i in order[:16]])
    big = pack_roads(sc, [sc.roads[i] for i in order[-16:]])
    assert max(nmax) > sorted(nmax)[15] + 16, "need a generation beyond the plan margin"
    S = len(sc.species)
    # one set of device buffers for both generations: the graph is keyed on
    # their addresses, so the second call replays the first one's plan
    dev = {k: torch.zeros(max(small[k].size, big[k].size),
                          dtype=torch.from_numpy(small[k]).dtype, device="cuda")
           for k in small}
    d_res = torch.zeros(16 * S * RESULT_STRIDE, dtype=torch.float64, device="cuda")
    opts = gen.opts(64, 30, seed=7, graph=True)

    def run_device(packed):
        for k, v in packed.items():
            dev[k][:v.size].copy_(torch.from_numpy(v))
        torch.cuda.synchronize()
        gen.evaluate_device(16, dev["cell_off"].data_ptr(), dev["cells"].data_ptr(),
                            dev["seg_off"].data_ptr(), dev["segs"].data_ptr(), opts,
                            d_res.data_ptr())

    run_device(small)                              # plans and captures
    ctx.synchronize()
    np.testing.assert_array_equal(d_res.cpu().numpy().reshape(16, S, RESULT_STRIDE),
                                  gen.evaluate(small, gen.opts(64, 30, seed=7)))
    run_device(big)                                # replays the small roads' plan
    with pytest.raises(TransOptError) as e:
        ctx.synchronize()
    assert e.value.status == 6                     # TO_ERR_UNSUPPORTED
    assert "plan" in str(e.value)
    ctx.synchronize()                              # the flag was cleared
    # the host form re-plans by itself and agrees with the direct path
    out = gen.evaluate(big, gen.opts(64, 30, seed=7, graph=True))
    np.testing.assert_array_equal(out, gen.evaluate(big, gen.opts(64, 30, seed=7)))
    gen.close()
