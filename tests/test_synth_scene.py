"""The batched-generation scene has the stated shapes: 256 roads of 8-64
control points and 20-400 patch crossings each on a 200 x 200 grid, patches
cut as the species models cut them (a region of one habitat code within a
block of res x res cells)."""
import numpy as np
import pytest

from transportoptimiser_gb300 import synth


def test_type_components_match_scipy_labels():
    ndimage = pytest.importorskip("scipy.ndimage")
    rng = np.random.default_rng(3)
    W, H = 37, 29
    base = rng.integers(0, 4, W * H).astype(np.int32)
    lab = synth.type_components(base, W, H)
    g = base.reshape(H, W)
    n = 0
    for t in np.unique(g):
        ref, k = ndimage.label(g == t)          # 4-connectivity
        n += k
        for r in range(1, k + 1):
            ids = np.unique(lab[ref == r])
            assert len(ids) == 1                # one region, one id
            # the id is the region's smallest cell index
            assert ids[0] == np.flatnonzero((ref == r).reshape(-1)).min()
    assert len(np.unique(lab)) == n


def test_patch_crossings_counts_boundaries():
    W = 20
    base = np.zeros(W * W, np.int32)
    base.reshape(W, W)[:, 10:] = 1              # two regions, split at x = 10
    lab = synth.patch_labels(base, W, W, 5)     # 4 x 4 blocks of 5 cells
    road = synth.Road(points=np.array([[0.5, 2.5], [19.5, 2.5]]),
                      segments=np.array([[0.5, 2.5, 19.5, 2.5]]))
    # x = 5, 10, 15: three block edges, the type edge on one of them
    assert synth.patch_crossings(road, lab, W, W) == 3


def test_generation_scene_shapes():
    sc = synth.generation(0)
    assert (sc.W, sc.H) == (200, 200) and len(sc.roads) == 256
    lab = synth.patch_labels(sc.base_map, sc.W, sc.H, sc.res)
    pts = np.array([len(r.points) for r in sc.roads])
    cr = np.array([synth.patch_crossings(r, lab, sc.W, sc.H) for r in sc.roads])
    assert pts.min() >= 8 and pts.max() <= 64
    assert cr.min() >= 20 and cr.max() <= 400
    assert len(np.unique(sc.base_map)) == 5
