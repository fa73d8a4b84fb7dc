"""Surrogate-assisted valuation of GA generations with the learned MLP.

The reference's GA (RoadGA::evaluateGeneration / computeSurrogate,
include/main/RoadGA.cpp:2040, 1553) values every design by Monte Carlo, or
by local-linear grid surrogates of one or two aggregate predictors
(buildSurrogateMTECUDA / buildSurrogateROVCUDA).  Here an ensemble of two
MLPs (transportoptimiser_gb300.mlp, own tensor-core kernels) trained on
pairs the batched simulator generates screens each generation (surrogate
pre-selection): the plain Monte Carlo values the most promising designs -
the top fraction (25%) by an optimistic score, the predicted fitness plus
the members' spread - and every design whose members disagree by more than
the tolerance (10%); it stays the measure of the surrogate's error, and only
Monte Carlo values become the incumbent.

Per road the surrogate predicts:
    0 mean over species of E[end population] / initial population
    1 mean over species of P(end < 0.2 initial)
    2 min over species of E[end population] / initial population
from 16 inputs (FEATURES): road length, segments and cells, the shares of
the road's cells on each habitat, the animals on and near the road (device
features, to_road_features), and what the reference's own surrogates look
up - each species' initial animals at risk (SpeciesRoadPatches::
computeInitialAAR) at full flow, their mean at half flow, and the animals
left off the road - from a species-model pass with no Monte Carlo.
"""
from __future__ import annotations

import time

import numpy as np

from . import synth
from .generation import Generation, pack_segments
from .mlp import MLPSurrogate

OUTPUTS = ("mean_end_ratio", "p_below", "min_end_ratio")
FEATURES = ("length / W", "segments / 64", "road cells / W", "share of road cells on code 2",
            "on code 3", "on code 5", "share of species 0's animals on road cells",
            "within 3 cells", "within 6 cells", "within 12 cells", "sinuosity / 10",
            "initial animals at risk, species 0, full flow", "species 1, full flow",
            "species 2, full flow", "mean over species, half flow",
            "initial animals, mean over species / 10^5")
# the device features kept (to_road_features slots)
_GEOM = (0, 1, 2, 5, 6, 7, 8, 9, 10, 11, 15)
SEM = 1


def road_features(gen: Generation, packed: dict) -> np.ndarray:
    """[R][16] surrogate inputs (FEATURES) of the roads in `packed`
    (segments): device features plus one species-model pass per road."""
    f = gen.features(packed)
    res = gen.evaluate_segments(packed, gen.opts(32, 0, sem=SEM))
    C = gen.scene.n_controls
    S = res.shape[1]
    iar_full = res[:, :, 16 + C - 1]
    cols = [f[:, i] for i in _GEOM]
    for s in range(3):
        cols.append(iar_full[:, s] if s < S else iar_full.mean(1))
    cols.append(res[:, :, 16 + C // 2].mean(1))
    cols.append(res[:, :, 6].mean(1) / 1e5)
    return np.stack(cols, 1).astype(np.float32)


def targets(results: np.ndarray) -> np.ndarray:
    """[R][3] surrogate targets from to_evaluate_roads result blocks."""
    init = results[:, :, 6]
    ratio = results[:, :, 2] / np.where(init > 0, init, 1.0)
    return np.stack([ratio.mean(1), results[:, :, 5].mean(1), ratio.min(1)], 1)


def fitness(y: np.ndarray, feats: np.ndarray) -> np.ndarray:
    """GA objective (higher is better): the weakest species' expected end
    population ratio, less a road-length cost."""
    return y[:, 2] - 0.05 * feats[:, 0]


def _road(pts):
    pts = pts[np.argsort(pts[:, 0])]
    segs = np.column_stack([pts[:-1], pts[1:]])
    keep = np.hypot(segs[:, 2] - segs[:, 0], segs[:, 3] - segs[:, 1]) > 1e-9
    return synth.Road(points=pts, segments=segs[keep])


def random_roads(scene, n, rng, lo=8, hi=64):
    return [synth.random_road(scene.W, scene.H, int(rng.integers(lo, hi + 1)), rng)
            for _ in range(n)]


def mutate(road, scene, rng, scale=6.0):
    """Jitter the control points; sometimes add or drop one (8..64 points)."""
    pts = road.points + rng.normal(0.0, scale, road.points.shape)
    if rng.random() < 0.2 and len(pts) < 64:
        pts = np.vstack([pts, rng.uniform(0, scene.W - 1, (1, 2))])
    elif rng.random() < 0.2 and len(pts) > 8:
        pts = np.delete(pts, int(rng.integers(len(pts))), axis=0)
    return _road(np.clip(pts, 0.0, scene.W - 1.0))


def crossover(a, b, rng):
    """Control points of a left of a random x, of b right of it."""
    x = rng.uniform(0.0, max(a.points[:, 0].max(), 1.0))
    pts = np.vstack([a.points[a.points[:, 0] <= x], b.points[b.points[:, 0] > x]])
    if len(pts) < 8:
        pts = np.vstack([pts, b.points[: 8 - len(pts)]])
    return _road(pts[:64])


def generate_dataset(gen: Generation, scene, n_samples: int, paths: int, rng,
                     batch: int | None = None, years: int = 50, seed: int = 0):
    """(features [n][16], targets [n][3]) of random roads valued by Monte Carlo."""
    batch = batch or gen.max_roads
    X, Y = [], []
    done = 0
    while done < n_samples:
        m = min(batch, n_samples - done)
        packed = pack_segments(random_roads(scene, m, rng))
        X.append(road_features(gen, packed))
        Y.append(targets(gen.evaluate_segments(packed, gen.opts(paths, years, seed=seed,
                                                                road0=done, sem=SEM))))
        done += m
    return np.concatenate(X), np.concatenate(Y).astype(np.float32)


class Ensemble:
    """Members with different initialisations; their spread is the surrogate's
    error estimate."""

    def __init__(self, n: int = 2, seed: int = 0):
        self.members = [MLPSurrogate(seed + 17 * i) for i in range(n)]

    def fit(self, X, Y, epochs=150, batch=512, lr=2e-3, ctx=None):
        for m in self.members:
            m.fit(X, Y, epochs=epochs, batch=batch, lr=lr, ctx=ctx)
        return self

    def predict(self, X, ctx=None):
        P = np.stack([m.predict(X, ctx) for m in self.members])
        mean = P.mean(0)
        spread = np.abs(P - mean).max(0) / np.maximum(np.abs(mean), 1e-6)
        return mean, spread


def screened_values(gen: Generation, ens: Ensemble, roads, opts, tol=0.10, top=0.25):
    """Values of a generation with surrogate screening.  Returns (y [R][3],
    fitness [R], mask of the designs re-valued by Monte Carlo, features)."""
    packed = pack_segments(roads)
    feats = road_features(gen, packed)
    y, spread = ens.predict(feats, gen.ctx)
    # optimistic: the predicted fitness plus the members' relative spread
    # on the fitness term, so uncertain designs get a chance
    score = fitness(y, feats) + spread[:, 2] * np.abs(y[:, 2])
    sel = (spread[:, 0] > tol) | (spread[:, 2] > tol)
    k = max(1, int(round(top * len(roads))))
    sel[np.argsort(-score)[:k]] = True
    idx = np.flatnonzero(sel)
    if idx.size:
        res = gen.evaluate_segments(pack_segments([roads[i] for i in idx]), opts)
        y[idx] = targets(res)
    return y, fitness(y, feats), sel, feats


def run_ga(gen: Generation, scene, generations: int, pop: int, opts, rng, ens: Ensemble | None,
           tol=0.10, top=0.25, timings: dict | None = None):
    """A small GA (tournament selection, crossover, mutation, elitism).  With
    an ensemble the generation is screened; without, every design is valued
    by Monte Carlo.  Returns (best road, its fitness by Monte Carlo, number of
    Monte Carlo valuations, seconds).  `timings`, when given, receives the
    seconds spent valuing generations (features, network, Monte Carlo) and
    in the host-side GA operators."""
    roads = random_roads(scene, pop, rng)
    n_mc = 0
    t0 = time.perf_counter()
    t_val = 0.0
    best, best_fit = None, -np.inf
    for _ in range(generations):
        tv = time.perf_counter()
        if ens is None:
            packed = pack_segments(roads)
            feats = road_features(gen, packed)
            y = targets(gen.evaluate_segments(packed, opts))
            fit = fitness(y, feats)
            mc = np.ones(len(roads), bool)
        else:
            y, fit, mc, feats = screened_values(gen, ens, roads, opts, tol, top)
        t_val += time.perf_counter() - tv
        n_mc += int(mc.sum())
        # only Monte Carlo values may become the incumbent
        cand = np.flatnonzero(mc)
        i = cand[np.argmax(fit[cand])]
        if fit[i] > best_fit:
            best, best_fit = roads[i], float(fit[i])
        order = np.argsort(-fit)
        children = [roads[j] for j in order[: max(1, pop // 10)]]
        while len(children) < pop:
            a = roads[max(rng.integers(pop, size=2), key=lambda j: fit[j])]
            b = roads[max(rng.integers(pop, size=2), key=lambda j: fit[j])]
            child = crossover(a, b, rng) if rng.random() < 0.5 else a
            children.append(mutate(child, scene, rng))
        roads = children
    total = time.perf_counter() - t0
    if timings is not None:
        timings["valuation_s"] = t_val
        timings["ga_ops_s"] = total - t_val
    return best, best_fit, n_mc, total
