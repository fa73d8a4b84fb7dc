"""Batched surrogate evaluation: the oracle pinned to the reference's kernel
(mode 0) and to scipy's multilinear interpolation (mode 1); the GPU against
the oracle."""
import numpy as np
import pytest

from oracle import pyoracle as po


def _surrogate(R, d, seed, uniform=True):
    """Evenly spaced axes, as the surrogate builders produce them."""
    rng = np.random.default_rng(seed)
    if uniform:
        axes = [np.linspace(rng.uniform(-2, 0), rng.uniform(1, 3), R) for _ in range(d)]
    else:
        axes = [np.sort(rng.uniform(-1.0, 3.0, R)) for _ in range(d)]
    vals = rng.normal(size=R ** d)
    return np.concatenate(axes + [vals]), axes, vals


def _points(axes, n, seed):
    rng = np.random.default_rng(seed)
    return np.stack([rng.uniform(a[0] - 0.2, a[-1] + 0.2, n) for a in axes], 1)


@pytest.mark.parametrize("d", [1, 2, 3])
def test_oracle_mode0_equals_reference_kernel(d):
    if not po.ref_available():
        pytest.skip("reference pin not built")
    S, axes, _ = _surrogate(8, d, d)
    P = _points(axes, 200, 10 + d)
    ours = po.interpolate_surrogate(S, P, 8, d, 0)
    ref = po.ref_interpolate_multi(S, P, 8, d).astype(np.float64)
    assert np.array_equal(ours, ref)


@pytest.mark.parametrize("uniform", [True, False])
@pytest.mark.parametrize("d", [1, 2, 3])
def test_oracle_mode1_is_multilinear(d, uniform):
    scipy = pytest.importorskip("scipy.interpolate")
    S, axes, vals = _surrogate(7, d, 20 + d, uniform)
    P = _points(axes, 300, 30 + d)
    P = np.stack([np.clip(P[:, j], axes[j][0], axes[j][-1]) for j in range(d)], 1)
    f = scipy.RegularGridInterpolator(axes, vals.reshape([7] * d))
    np.testing.assert_allclose(po.interpolate_surrogate(S, P, 7, d, 1), f(P), rtol=1e-12, atol=1e-12)


def test_oracle_mode2_is_linear_in_one_dimension():
    S, axes, vals = _surrogate(9, 1, 5)
    P = np.clip(_points(axes, 100, 6), axes[0][0], axes[0][-1])
    np.testing.assert_allclose(po.interpolate_surrogate(S, P, 9, 1, 2),
                               np.interp(P[:, 0], axes[0], vals), rtol=1e-12, atol=1e-12)


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [0, 1, 2])
@pytest.mark.parametrize("d", [1, 3, 4])
def test_gpu_matches_oracle(ctx, mode, d):
    from transportoptimiser_gb300 import simulate_gpu as sg
    S, axes, _ = _surrogate(6, d, 40 + d)
    P = _points(axes, 1000, 50 + d)
    got = sg.interpolateSurrogateMulti(S, P, 6, d, mode=mode, ctx=ctx)
    ref = po.interpolate_surrogate(S, P, 6, d, mode)
    if mode == 0:
        assert np.array_equal(got, ref)
    else:
        np.testing.assert_allclose(got, ref, rtol=1e-12, atol=1e-12)
