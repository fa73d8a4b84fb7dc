"""Host logic of surrogate pre-selection and the GA around it, on the CPU:
the device parts (features, network, Monte Carlo) are replaced by fakes with
known answers, so the selection rule, the replacement of predictions by
Monte Carlo values and the incumbent rule are checked exactly."""
import numpy as np

from transportoptimiser_gb300 import surrogate_ga as sga
from transportoptimiser_gb300 import synth
from transportoptimiser_gb300._capi import RESULT_STRIDE


class FakeGen:
    """Features: [length-like, key, 0...]; Monte Carlo: a known value per
    road (its first control point's x, scaled), in the result-block layout."""

    ctx = None

    class scene:
        n_controls = 3

    def __init__(self, n_species=3, scale=1.0):
        self.S = n_species
        self.scale = scale
        self.evaluated = []

    @staticmethod
    def opts(paths, years=50, **kw):
        return ("opts", paths, years)

    @staticmethod
    def _key(packed, r):
        a, b = packed["seg_off"][r], packed["seg_off"][r + 1]
        segs = np.asarray(packed["segs"]).reshape(-1, 4)[a:b]
        return float(segs[0, 0]) if len(segs) else 0.0

    def features(self, packed):
        R = len(packed["seg_off"]) - 1
        f = np.zeros((R, 16), np.float32)
        for r in range(R):
            f[r, 0] = 0.0                      # no length cost: fitness = y[:, 2]
            f[r, 1] = self._key(packed, r)
        return f

    def evaluate_segments(self, packed, opts):
        R = len(packed["seg_off"]) - 1
        out = np.zeros((R, self.S, RESULT_STRIDE))
        model_only = isinstance(opts, tuple) and opts[2] == 0   # the species-model pass
        for r in range(R):
            v = self._key(packed, r)
            if not model_only:
                self.evaluated.append(v)
            v *= self.scale
            out[r, :, 6] = 100.0               # initial population
            out[r, :, 2] = 100.0 * (1.0 + v)   # end population: ratio 1 + v
            out[r, :, 5] = 0.1
        return out


class FakeEnsemble:
    """Prediction: ratio 1 + pred[key]; spread given per key."""

    def __init__(self, pred, spread):
        self.pred, self.spread = pred, spread

    def predict(self, feats, ctx=None):
        keys = feats[:, 1]
        y = np.zeros((len(keys), 3), np.float32)
        s = np.zeros((len(keys), 3), np.float32)
        for i, k in enumerate(keys):
            y[i] = [1.0 + self.pred[k], 0.1, 1.0 + self.pred[k]]
            s[i, 0] = s[i, 2] = self.spread[k]
        return y, s


def _roads(keys):
    return [synth.Road(points=np.array([[k, 1.0], [k + 1.0, 2.0]]),
                       segments=np.array([[k, 1.0, k + 1.0, 2.0]])) for k in keys]


def test_screening_selects_top_fraction_and_uncertain_designs():
    keys = [float(k) for k in range(8)]
    pred = {k: 0.1 * k for k in keys}              # road 7 predicted best
    spread = {k: 0.0 for k in keys}
    spread[0.0] = 0.11                              # uncertain: must be valued, although
    gen, ens = FakeGen(), FakeEnsemble(pred, spread)   # 1.0 + 0.11 is far from the top
    y, fit, sel, feats = sga.screened_values(gen, ens, _roads(keys), opts=None,
                                             tol=0.10, top=0.25)
    # top 25% of 8 = the two best by optimistic score (7, 6), plus road 0
    assert set(np.flatnonzero(sel)) == {0, 6, 7}
    assert sorted(gen.evaluated) == [0.0, 6.0, 7.0]
    # valued designs carry the Monte Carlo targets, the others the prediction
    for i, k in enumerate(keys):
        want = 1.0 + (k if sel[i] else pred[k])
        assert np.isclose(y[i, 2], want)
        assert np.isclose(fit[i], want)


def test_optimistic_score_lifts_uncertain_designs_into_the_top():
    keys = [float(k) for k in range(4)]
    pred = {0.0: 0.30, 1.0: 0.29, 2.0: 0.25, 3.0: 0.10}
    spread = {k: 0.0 for k in keys}
    gen, ens = FakeGen(), FakeEnsemble(pred, spread)
    # top 1 of 4 with no spread: road 0 (1.30)
    _, _, sel, _ = sga.screened_values(gen, ens, _roads(keys), None, tol=0.10, top=0.25)
    assert set(np.flatnonzero(sel)) == {0}
    # road 2 with a spread below the tolerance: 1.25 + 0.08 * 1.25 = 1.35 takes the top
    spread[2.0] = 0.08
    _, _, sel, _ = sga.screened_values(gen, ens, _roads(keys), None, tol=0.10, top=0.25)
    assert set(np.flatnonzero(sel)) == {2}
    # a low prediction with a spread above the tolerance is valued as well
    pred[2.0], spread[2.0] = 0.0, 0.2
    _, _, sel, _ = sga.screened_values(gen, ens, _roads(keys), None, tol=0.10, top=0.25)
    assert set(np.flatnonzero(sel)) == {0, 2}


def test_only_monte_carlo_values_become_the_incumbent():
    # a surrogate that overrates every design by a wide margin and is sure of
    # itself: the screened-out designs have high predictions but the
    # incumbent must still be a Monte Carlo value
    class Overrating(FakeEnsemble):
        def predict(self, feats, ctx=None):
            y, s = super().predict(feats, ctx)
            y[:, 0] += 10.0
            y[:, 2] += 10.0
            return y, s

    scene = synth.mte_road(0)
    rng = np.random.Generator(np.random.Philox(3))

    class KeyedPred(dict):
        def __missing__(self, k):
            return 0.0

    gen = FakeGen(scale=1e-3)                       # Monte Carlo ratios in [1, 1.07]
    ens = Overrating(KeyedPred(), KeyedPred())
    best, best_fit, n_mc, _ = sga.run_ga(gen, scene, generations=3, pop=16, opts=None,
                                         rng=rng, ens=ens, tol=0.10, top=0.25)
    # Monte Carlo value of a road is 1 + its first x / 1000; never the overrated 11+
    assert best_fit < 2.0
    assert np.isclose(best_fit, 1.0 + 1e-3 * float(best.segments[0, 0]), rtol=1e-6)
    assert n_mc == 3 * 4                          # top 25% of 16 per generation
