"""GA sample selection (RoadGA::generateSample): oracle properties on the CPU,
device against the oracle."""
import numpy as np
import pytest

from oracle import pyoracle as po


def _cands(n, d, seed):
    return np.random.default_rng(seed).uniform(0, 10, size=(n, d))


def test_oracle_first_pair_is_most_distant_in_projection():
    c = _cands(60, 3, 1)
    s = po.select_samples(None, c, 2)
    cn = (c - c.min(0)) / (c.max(0) - c.min(0))
    proj = np.abs(cn[:, None, :] - cn[None, :, :]).min(2)
    assert np.isclose(proj[s[0], s[1]], proj.max())


def test_oracle_selection_spreads_out():
    c = _cands(400, 2, 2)
    s = po.select_samples(None, c, 20)
    assert len(set(s.tolist())) == 20
    # the chosen set covers the space better than the same number of random points
    cn = (c - c.min(0)) / (c.max(0) - c.min(0))
    def fill(idx):
        return np.sqrt(((cn[:, None, :] - cn[None, idx, :]) ** 2).sum(2)).min(1).max()
    rnd = np.mean([fill(np.random.default_rng(k).choice(400, 20, replace=False)) for k in range(20)])
    assert fill(s) < rnd


@pytest.mark.gpu
@pytest.mark.parametrize("d,n_cur", [(1, 0), (3, 0), (5, 7), (16, 12)])
def test_gpu_matches_oracle(ctx, d, n_cur):
    from transportoptimiser_gb300 import simulate_gpu as sg
    c = _cands(3000, d, 3 + d)
    cur = _cands(n_cur, d, 40 + d) if n_cur else None
    got = sg.generateSample(cur, c, 25, ctx=ctx)
    ref = po.select_samples(cur, c, 25)
    assert np.array_equal(got, ref)
