"""GPU surrogate builders against the oracle (bit-exact) and against the
reference's golden output."""
import numpy as np
import pytest

from oracle import pyoracle as po
from transportoptimiser_gb300 import simulate_gpu as sg

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n,R", [(30, 20), (300, 50), (1200, 64)])
def test_mte_surrogate_bit_exact(ctx, n, R):
    rng = np.random.default_rng(n)
    x = rng.random(n).astype(np.float32).astype(np.float64) * 0.4
    y = (1.0 - x * 1.7 + 0.05 * rng.standard_normal(n)).astype(np.float32).astype(np.float64)
    ysd = np.abs(0.1 * rng.standard_normal(n)).astype(np.float32).astype(np.float64)
    m, s = sg.buildSurrogateMTECUDA(x, y, ysd, R, ctx=ctx)
    om = po.build_surrogate_1d(x, y, R)
    osd = po.build_surrogate_1d(x, ysd, R)
    assert np.array_equal(m.astype(np.float32), om)
    assert np.array_equal(s.astype(np.float32), osd)


@pytest.mark.parametrize("sem", [0, 1])
def test_rov_surrogate_bit_exact_and_golden(ctx, golden, sem):
    g = golden["surrogate_rov"]
    R = int(g["R"])
    pred = g["pred"].astype(np.float64)
    y = g["y"].astype(np.float64)
    m, s = sg.buildSurrogateROVCUDA(pred, y, np.abs(y) * 0.1, R, sem=sem, ctx=ctx)
    om = po.build_surrogate_nd(g["pred"], g["y"], R, sem=sem, clip=1)
    assert np.array_equal(m.astype(np.float32), om)
    if sem == 0:
        assert np.abs(m - g["mean"]).max() <= 1e-5 * np.abs(g["mean"]).max()
