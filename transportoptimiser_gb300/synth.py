"""Seeded synthetic road-evaluation workloads.

There is no public dataset for this path; these generators stand in for the
reference's region CSVs (habitat map, initial-population map) and its GA
road genomes, with the shapes of the benchmark configurations:

* ``mte_road``    - 64 x 64 grid, 4 habitat types drawn i.i.d. (0.4 / 0.3 /
  0.2 / 0.1, the last one CLEAR) on coarse habitat tiles, ~40 patches, a road
  through 10 random control points, one species, 2000 paths x 50 years.
* ``rov_road``    - the same dynamics on 128 x 128 (~120 patches), 2 species,
  3 mean-reverting exogenous processes, 3 flow controls, 10^4 paths.
* ``generation``  - 256 roads of 8-64 control points on 200 x 200 with 5
  habitat types (~300 patches) and 3 species.

Habitat codes follow the reference's HabitatType enum
(include/ecology/HabitatType.h:16-20): PRIMARY 0, MARGINAL 1, OTHER 2,
CLEAR 3, ROAD 4.  Grids are stored column-major like the reference's Eigen
matrices: cell (x, y) is element x + y*W.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

PRIMARY, MARGINAL, OTHER, CLEAR, ROAD = 0, 1, 2, 3, 4
SURVIVAL_PER_CROSSING = 0.7          # crossing mortality 0.3 at full flow


@dataclass
class HabitatSpec:
    type: int
    max_pop: float
    pref_mean: float
    pref_sd: float = 0.0


@dataclass
class SpeciesSpec:
    habitats: list
    params: np.ndarray                # float32[8], SimulateGPU.cu:3694-3714 layout
    hazard: np.ndarray                # float64[C]
    lambda_mean: float = 0.2          # exponential migration scale 5 cells
    lambda_sd: float = 0.0
    lambda_mult: float = 0.0
    hab_pref_mult: float = 0.0
    density: float = 25.0             # initial animals per habitable cell


@dataclass
class Road:
    points: np.ndarray                # (n, 2) control points
    segments: np.ndarray              # (G, 4) rows x1, y1, x2, y2

    @property
    def G(self) -> int:
        return int(self.segments.shape[0])

    def colmajor(self) -> np.ndarray:
        """G x 4 column-major (x1 | y1 | x2 | y2) as the reference passes."""
        return np.ascontiguousarray(self.segments.T.reshape(-1)).astype(np.float64)


@dataclass
class Scene:
    W: int
    H: int
    res: int
    base_map: np.ndarray              # int32[W*H] habitat codes (no road)
    species: list
    n_controls: int
    flows: np.ndarray
    seed: int
    roads: list = field(default_factory=list)

    def hab_map(self, road: Road) -> np.ndarray:
        m = self.base_map.copy()
        for (x, y) in road_cells(road, self.W, self.H):
            m[x + y * self.W] = ROAD
        return m

    def pop_map(self, sp: SpeciesSpec, hab: np.ndarray) -> np.ndarray:
        habitable = np.isin(hab, [h.type for h in sp.habitats if h.type not in (CLEAR, ROAD)])
        return np.where(habitable, sp.density, 0.0).astype(np.float64)


def _span_points(x0, y0, x1, y1, xs, ys, sem):
    """The grid-line crossings of one span, sorted as RoadCells sorts them."""
    f = np.float64
    x0, y0, x1, y1, xs, ys = f(x0), f(y0), f(x1), f(y1), f(xs), f(ys)
    h = int(x1 / xs) - int(x0 / xs)
    v = int(y1 / ys) - int(y0 / ys)
    with np.errstate(divide="ignore", invalid="ignore"):
        m = (y1 - y0) / (x1 - x0)
        b = y0 - x0 * m
        m2 = (x1 - x0) / (y1 - y0)
        b2 = x0 - y0 * m2
    pts = []
    for q in range(abs(h)):
        if h > 0:
            px = xs * (f(math.floor(x0 / xs)) + f(q + 1))
        elif math.fmod(x0, xs) == 0.0:
            px = xs * (f(math.ceil(x0 / xs)) - f(q))
        else:
            px = xs * (f(math.ceil(x0 / xs)) - f(q + 1))
        pts.append([px, m * px + b if np.isfinite(m) else y0])
    vy = []
    for q in range(abs(v)):
        if v > 0:
            vy.append(ys * (f(math.floor(y0 / ys)) + f(q + 1)))
        elif math.fmod(y0, ys) == 0.0:
            vy.append(ys * (f(math.ceil(y0 / ys)) - f(q)))
        else:
            vy.append(ys * (f(math.ceil(y0 / ys)) - f(q + 1)))
    ycol = [p[1] for p in pts] + vy           # column 1 of the crossing list
    for q in range(abs(v)):
        src = ycol[q] if sem == 0 else vy[q]
        if np.isfinite(m):
            px = (src - b) / m
        elif np.isfinite(m2):
            px = b2 + m2 * src
        else:
            px = x0
        pts.append([px, vy[q]])
    pts.sort(key=lambda p: (p[0], p[1]), reverse=not (x1 >= x0))
    return pts


def road_cells(road: Road, W: int, H: int, sem: int = 1, xs: float = 1.0,
               ys: float = 1.0) -> list:
    """Cells of a road as RoadCells::computeRoadCells (include/road/
    RoadCells.cpp:10-272) finds them: each span is cut at its crossings of
    the grid lines x = k xs and y = k ys (sorted by (x, y), ascending when
    the span runs towards larger x, else descending), consecutive equal
    points are dropped, and each piece lies in the cell (ceil(mid_x / xs),
    ceil(mid_y / ys)) of its midpoint.  sem 0 keeps the reference's x of a
    vertical-line crossing, computed from the y of the crossing list's row
    q (RoadCells.cpp:189-194); sem 1 uses the crossing's own y.  Returns
    the sorted (x, y) cells inside the grid."""
    cells = set()
    for x1, y1, x2, y2 in road.segments:
        seq = [[np.float64(x1), np.float64(y1)]] + _span_points(x1, y1, x2, y2, xs, ys, sem) + \
              [[np.float64(x2), np.float64(y2)]]
        for a, b in zip(seq[:-1], seq[1:]):
            if a[0] == b[0] and a[1] == b[1]:
                continue
            cx = int(math.ceil((np.float64(0.5) * (a[0] + b[0]) - np.float64(0.0)) / np.float64(xs)))
            cy = int(math.ceil((np.float64(0.5) * (a[1] + b[1]) - np.float64(0.0)) / np.float64(ys)))
            if 0 <= cx < W and 0 <= cy < H:
                cells.add((cx, cy))
    return sorted(cells, key=lambda c: c[0] + c[1] * W)


def _rng(seed: int) -> np.random.Generator:
    return np.random.Generator(np.random.Philox(seed))


def habitat_map(W: int, H: int, tile: int, probs, types, rng) -> np.ndarray:
    tw, th = -(-W // tile), -(-H // tile)
    tiles = rng.choice(np.asarray(types), size=(th, tw), p=np.asarray(probs))
    m = np.repeat(np.repeat(tiles, tile, axis=0), tile, axis=1)[:H, :W]
    return np.ascontiguousarray(m.reshape(-1)).astype(np.int32)   # [y][x] -> x + y*W


def random_road(W: int, H: int, n_points: int, rng) -> Road:
    pts = np.column_stack([rng.uniform(0, W - 1, n_points), rng.uniform(0, H - 1, n_points)])
    pts = pts[np.argsort(pts[:, 0])]
    segs = np.column_stack([pts[:-1], pts[1:]])
    keep = np.hypot(segs[:, 2] - segs[:, 0], segs[:, 3] - segs[:, 1]) > 1e-9
    return Road(points=pts, segments=segs[keep])


def default_species(n_controls: int, flows, habitat_types, threshold: float,
                    local_var: float = 0.4) -> SpeciesSpec:
    h_max = -math.log(SURVIVAL_PER_CROSSING)
    prefs = [0.0, -0.3, -0.6, -0.9]
    habs = [HabitatSpec(t, 50.0, prefs[i % len(prefs)]) for i, t in enumerate(habitat_types)]
    habs.append(HabitatSpec(CLEAR, 0.0, 0.0))
    params = np.array([0.05, 0.05, 0.0, threshold, 0.5, 0.0, 0.0, local_var], dtype=np.float32)
    hazard = np.asarray(flows, dtype=np.float64) * h_max
    return SpeciesSpec(habitats=habs, params=params, hazard=hazard)


def mte_road(seed: int = 0, W: int = 64, tile: int = 12, res: int = 4) -> Scene:
    """64 x 64 grid, one road, one species (the plain MTE workload)."""
    rng = _rng(seed)
    base = habitat_map(W, W, tile, [0.4, 0.3, 0.2, 0.1], [PRIMARY, MARGINAL, OTHER, CLEAR], rng)
    flows = np.array([0.0, 0.5, 1.0])
    sp = default_species(3, flows, [PRIMARY, MARGINAL, OTHER], threshold=0.0)
    sc = Scene(W=W, H=W, res=res, base_map=base, species=[sp], n_controls=3,
               flows=flows, seed=seed)
    sc.roads = [random_road(W, W, 10, rng)]
    return sc


def rov_road(seed: int = 0, W: int = 128, tile: int = 24, res: int = 7,
             n_species: int = 2) -> Scene:
    """128 x 128 grid, one road, two species, three flow controls (the ROV workload)."""
    rng = _rng(seed)
    base = habitat_map(W, W, tile, [0.4, 0.3, 0.2, 0.1], [PRIMARY, MARGINAL, OTHER, CLEAR], rng)
    flows = np.array([0.0, 0.5, 1.0])
    spp = []
    for s in range(n_species):
        sp = default_species(3, flows, [PRIMARY, MARGINAL, OTHER], threshold=0.0)
        spp.append(sp)
    sc = Scene(W=W, H=W, res=res, base_map=base, species=spp, n_controls=3,
               flows=flows, seed=seed)
    sc.roads = [random_road(W, W, 10, rng)]
    return sc


def generation(seed: int = 0, n_roads: int = 256, W: int = 200, tile: int = 30,
               res: int = 10, n_species: int = 3) -> Scene:
    """200 x 200 grid, 5 habitat types, a GA generation of roads of 8-64 control points."""
    rng = _rng(seed)
    base = habitat_map(W, W, tile, [0.35, 0.25, 0.15, 0.15, 0.1],
                       [PRIMARY, MARGINAL, OTHER, 5, CLEAR], rng)
    flows = np.array([0.0, 0.5, 1.0])
    spp = [default_species(3, flows, [PRIMARY, MARGINAL, OTHER, 5], threshold=0.0)
           for _ in range(n_species)]
    sc = Scene(W=W, H=W, res=res, base_map=base, species=spp, n_controls=3,
               flows=flows, seed=seed)
    # roads of 20-400 patch crossings each: a draw outside is redrawn
    lab = patch_labels(base, W, W, res)
    sc.roads = []
    while len(sc.roads) < n_roads:
        rd = random_road(W, W, int(rng.integers(8, 65)), rng)
        if 20 <= patch_crossings(rd, lab, W, W) <= 400:
            sc.roads.append(rd)
    return sc


def type_components(base: np.ndarray, W: int, H: int) -> np.ndarray:
    """[H][W] labels of the 4-connected regions of equal habitat code (the
    smallest cell index of the region), by min-label propagation."""
    g = base.reshape(H, W)
    lab = np.arange(W * H, dtype=np.int64).reshape(H, W)
    pairs = [((slice(None), slice(1, None)), (slice(None), slice(None, -1))),
             ((slice(None), slice(None, -1)), (slice(None), slice(1, None))),
             ((slice(1, None), slice(None)), (slice(None, -1), slice(None))),
             ((slice(None, -1), slice(None)), (slice(1, None), slice(None)))]
    while True:
        new = lab.copy()
        for a, b in pairs:
            same = g[a] == g[b]
            new[a] = np.where(same, np.minimum(new[a], lab[b]), new[a])
        if np.array_equal(new, lab):
            return lab
        lab = new


def patch_labels(base: np.ndarray, W: int, H: int, block: int) -> np.ndarray:
    """[H][W] patch ids as the species models cut them: a region of equal
    habitat code within one block x block square of cells."""
    lab = type_components(base, W, H)
    yy, xx = np.mgrid[0:H, 0:W]
    nb = ((W + block - 1) // block) * ((H + block - 1) // block)
    return lab * nb + (yy // block) * ((W + block - 1) // block) + xx // block


def patch_crossings(road: Road, lab: np.ndarray, W: int, H: int) -> int:
    """How often the road's path passes from one patch into another (ids
    from patch_labels), sampled at quarter-cell steps."""
    xs, ys = [], []
    for x1, y1, x2, y2 in road.segments:
        n = max(2, int(math.hypot(x2 - x1, y2 - y1) * 4))
        t = np.linspace(0.0, 1.0, n)
        xs.append(x1 + t * (x2 - x1))
        ys.append(y1 + t * (y2 - y1))
    x = np.clip(np.concatenate(xs).astype(np.int64), 0, W - 1)
    y = np.clip(np.concatenate(ys).astype(np.int64), 0, H - 1)
    seq = lab[y, x]
    return int((seq[1:] != seq[:-1]).sum())
