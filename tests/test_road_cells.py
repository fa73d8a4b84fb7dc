"""RoadCells::computeRoadCells (include/road/RoadCells.cpp:10-272): the host
restatement the synthetic scenes use (synth.road_cells) against the C
oracle's, in both semantics, on random roads and on the spans whose
arithmetic has special cases (vertical, horizontal, endpoints on grid
lines and corners, spans running towards smaller x, zero-length spans)."""
import numpy as np
import pytest

from oracle import pyoracle as po
from transportoptimiser_gb300 import synth


def _polyline(road):
    return np.vstack([road.segments[:1, :2], road.segments[:, 2:4]])


def _host(road, W, H, sem):
    return np.array([x + y * W for (x, y) in synth.road_cells(road, W, H, sem=sem)], np.int32)


@pytest.mark.parametrize("sem", [0, 1])
def test_random_roads_match_oracle(sem):
    rng = np.random.Generator(np.random.Philox(3))
    for i in range(60):
        W = int(rng.integers(20, 220))
        rd = synth.random_road(W, W, int(rng.integers(2, 65)), rng)
        assert np.array_equal(_host(rd, W, W, sem), po.road_cells(_polyline(rd), W, W, sem)), i


@pytest.mark.parametrize("sem", [0, 1])
def test_special_spans_match_oracle(sem):
    W = H = 40
    cases = [
        [(3.5, 4.5), (3.5, 20.2)],            # vertical, upwards
        [(3.5, 20.2), (3.5, 4.5)],            # vertical, downwards
        [(2.2, 7.0), (30.9, 7.0)],            # horizontal on a grid line
        [(30.9, 7.3), (2.2, 7.3)],            # horizontal, towards smaller x
        [(5.0, 5.0), (9.0, 13.0)],            # endpoints on grid corners
        [(9.0, 13.0), (5.0, 5.0), (1.0, 2.0)],
        [(4.0, 3.3), (12.7, 8.0), (12.7, 8.0), (20.1, 2.0)],   # a zero-length span
        [(0.0, 0.0), (39.0, 39.0)],           # the diagonal through every corner
        [(38.5, 1.5), (1.5, 38.5)],
    ]
    for pts in cases:
        segs = np.array([[*a, *b] for a, b in zip(pts[:-1], pts[1:])], np.float64)
        rd = synth.Road(points=np.array(pts), segments=segs)
        assert np.array_equal(_host(rd, W, H, sem), po.road_cells(np.array(pts), W, H, sem)), pts


def test_cells_follow_the_road_in_corrected_semantics():
    """sem 1: every piece's midpoint lies on the road, so each cell is within
    one cell of the polyline; consecutive cells along a span are 4-connected
    up to corner passes."""
    rng = np.random.Generator(np.random.Philox(8))
    for _ in range(20):
        rd = synth.random_road(100, 100, 12, rng)
        for x, y in synth.road_cells(rd, 100, 100, sem=1):
            d = min(_dist_to_segment(x, y, s) for s in rd.segments)
            assert d <= 1.5, (x, y, d)


def _dist_to_segment(x, y, s):
    # cell (x, y) covers (x-1, x] x (y-1, y]: distance from its centre
    px, py = x - 0.5, y - 0.5
    x1, y1, x2, y2 = s
    dx, dy = x2 - x1, y2 - y1
    t = 0.0 if dx == dy == 0 else max(0.0, min(1.0, ((px - x1) * dx + (py - y1) * dy) /
                                                 (dx * dx + dy * dy)))
    return float(np.hypot(px - (x1 + t * dx), py - (y1 + t * dy)))
