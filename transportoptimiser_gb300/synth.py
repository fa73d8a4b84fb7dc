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


def road_cells(road: Road, W: int, H: int) -> list:
    """Cells a polyline passes through (sampled every 0.25 cells)."""
    cells = set()
    for x1, y1, x2, y2 in road.segments:
        n = max(2, int(math.ceil(4.0 * math.hypot(x2 - x1, y2 - y1))) + 1)
        for s in np.linspace(0.0, 1.0, n):
            x = int(round(x1 + s * (x2 - x1)))
            y = int(round(y1 + s * (y2 - y1)))
            if 0 <= x < W and 0 <= y < H:
                cells.add((x, y))
    return sorted(cells)


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
    sc.roads = [random_road(W, W, int(rng.integers(8, 65)), rng) for _ in range(n_roads)]
    return sc
