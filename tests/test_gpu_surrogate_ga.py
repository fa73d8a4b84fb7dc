"""Device road rasterisation and surrogate features against host restatements."""
import numpy as np
import pytest

from transportoptimiser_gb300 import synth
from transportoptimiser_gb300.generation import Generation, pack_roads, pack_segments

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("sem", [0, 1])
def test_device_rasterisation_equals_host_cells(ctx, sem):
    """RoadCells::computeRoadCells on the device (cells computed from the
    segments inside to_evaluate_roads) against the host restatement the
    scenes use, which the CPU tests pin to the oracle: the species models
    and valuations of 48 roads are identical."""
    sc = synth.generation(4, n_roads=48)
    gen = Generation(sc, max_roads=48, max_patches=512, ctx=ctx)
    a = gen.evaluate(pack_roads(sc, sc.roads, sem=sem), gen.opts(32, 10, seed=3, sem=sem))
    b = gen.evaluate_segments(pack_segments(sc.roads), gen.opts(32, 10, seed=3, sem=sem))
    np.testing.assert_array_equal(a, b)
    gen.close()


def test_features_match_host_computation(ctx):
    sc = synth.generation(5, n_roads=16)
    gen = Generation(sc, max_roads=16, max_patches=512, ctx=ctx)
    f = gen.features(pack_segments(sc.roads))
    pm = sc.pop_map(sc.species[0], sc.base_map)
    W = sc.W
    occ = (pm.reshape(W, W) > 0)        # [y][x]
    for r, rd in enumerate(sc.roads):
        cells = synth.road_cells(rd, W, sc.H)
        seg = rd.segments
        length = np.hypot(seg[:, 2] - seg[:, 0], seg[:, 3] - seg[:, 1]).sum()
        assert np.isclose(f[r, 0], length / W, rtol=1e-6)
        assert np.isclose(f[r, 2], len(cells) / W, rtol=1e-6)
        codes = np.array([sc.base_map[x + y * W] for x, y in cells])
        for b, code in enumerate((2, 3, 5)):
            assert np.isclose(f[r, 5 + b], (codes == code).mean(), atol=1e-6)
        assert np.isclose(f[r, 8], sum(pm[x + y * W] for x, y in cells) / pm.sum(),
                          rtol=1e-5, atol=1e-7)
        # animals within 6 cells (Chebyshev) of the road
        road = np.zeros((W, W), bool)
        for x, y in cells:
            road[y, x] = True
        near = np.zeros_like(road)
        ys, xs = np.nonzero(road)
        for y, x in zip(ys, xs):
            near[max(0, y - 6):y + 7, max(0, x - 6):x + 7] = True
        assert np.isclose(f[r, 10], pm.reshape(W, W)[near].sum() / pm.sum(), rtol=1e-5)
        assert 0.0 <= f[r, 3] and 0.0 <= f[r, 4]
    assert occ.any()
    gen.close()


def test_surrogate_gain_over_local_linear_and_plain_ga(ctx):
    from transportoptimiser_gb300 import simulate_gpu as sg
    from transportoptimiser_gb300 import surrogate_ga as sga
    sc = synth.generation(0, n_roads=1)
    gen = Generation(sc, max_roads=256, max_patches=512, ctx=ctx)
    X, Y = sga.generate_dataset(gen, sc, 3072, paths=256, rng=np.random.default_rng(11))
    ens = sga.Ensemble(2).fit(X, Y, epochs=100, batch=256, lr=2e-3, ctx=ctx)
    Xt, Yt = sga.generate_dataset(gen, sc, 512, paths=1024, rng=np.random.default_rng(12), seed=5)
    pred, _ = ens.predict(Xt, ctx)
    err_mlp = np.median(np.abs(pred[:, 0] - Yt[:, 0]) / Yt[:, 0])
    # the method without it: the reference's local-linear surrogate of the
    # end population against the initial animals at risk (buildSurrogateMTECUDA
    # looks a species up by its IAR), here their mean over species at full flow
    iar, iar_t = X[:, 11:14].mean(1), Xt[:, 11:14].mean(1)
    om, _ = sg.buildSurrogateMTECUDA(iar.astype(np.float64), Y[:, 0].astype(np.float64),
                                     np.zeros(len(X)), 32, ctx=ctx)
    ll = np.interp(iar_t, om[:32], om[32:])
    err_ll = np.median(np.abs(ll - Yt[:, 0]) / Yt[:, 0])
    assert err_mlp < err_ll, (err_mlp, err_ll)
    # ranking, which the screening relies on: recall of the true top 10% of
    # held-out designs within each method's predicted top 25%
    fit_true = sga.fitness(Yt, Xt)
    true_top = set(np.argsort(-fit_true)[:51])

    def recall(pred_y0):
        yy = Yt.copy()
        yy[:, 2] = pred_y0
        return len(true_top & set(np.argsort(-sga.fitness(yy, Xt))[:128])) / 51

    assert recall(pred[:, 2]) >= recall(ll), (recall(pred[:, 2]), recall(ll))
    # GAs at equal settings (six seeds; a short GA's outcome varies from run
    # to run): screened (Monte Carlo on the top 25% by an optimistic
    # predicted fitness and on designs whose members disagree by more than
    # the tolerance, 10% or 20%) against Monte Carlo on every design: fewer
    # Monte Carlo valuations for the same outcome
    opts = gen.opts(128, 50, seed=9, sem=1)
    for tol, max_frac in ((0.10, 0.75), (0.20, 0.6)):
        fs, fp, ns, npl = [], [], 0, 0
        for seed in (3, 4, 5, 6, 7, 8):
            _, f1, n1, _ = sga.run_ga(gen, sc, 6, 128, opts, np.random.default_rng(seed), ens, tol)
            _, f2, n2, _ = sga.run_ga(gen, sc, 6, 128, opts, np.random.default_rng(seed), None)
            fs.append(f1); fp.append(f2); ns += n1; npl += n2
        assert ns < max_frac * npl, (tol, ns, npl)
        assert np.mean(fs) >= np.mean(fp) - 0.03 * abs(np.mean(fp)), (tol, fs, fp)
    gen.close()
