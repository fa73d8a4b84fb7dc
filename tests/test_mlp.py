"""Learned surrogate (MLP 16->128->128->3): oracle pins on the CPU, tensor-core
forward/backward parity with the oracle and training on the GPU."""
import numpy as np
import pytest

from oracle import pyoracle as po
from transportoptimiser_gb300 import mlp

IN, OUT = mlp.IN, mlp.OUT


_W = np.random.default_rng(99).normal(size=(IN, OUT)).astype(np.float32) / 2


def _data(n, seed):
    """Samples of one fixed smooth, non-linear function of 16 inputs."""
    rng = np.random.default_rng(seed)
    x = rng.normal(size=(n, IN)).astype(np.float32)
    t = (np.tanh(x @ _W) + 0.5 * np.sin(x[:, :OUT] * 2) * np.cos(x[:, OUT:2 * OUT]))
    return x, t.astype(np.float32)


def test_oracle_bf16_rounding_matches_torch():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(0)
    v = np.concatenate([rng.normal(size=4000) * 10.0 ** rng.integers(-30, 30, 4000),
                        [0.0, -0.0, 1.0, 65504.0, 3.0e38, 1e-40]]).astype(np.float32)
    ours = np.array([po.oracle().or_bf16(float(a)) for a in v], np.float32)
    ref = torch.from_numpy(v).to(torch.bfloat16).float().numpy()
    assert np.array_equal(ours.view(np.uint32), ref.view(np.uint32))


def test_oracle_backward_matches_autograd_without_rounding():
    torch = pytest.importorskip("torch")
    p = mlp.init_params(3)
    p[mlp.OFF_B1:mlp.OFF_W2] = 0.05
    x, t = _data(37, 1)
    g, loss = po.mlp_grad(p, x, t, rounding=False)
    P = torch.tensor(p.astype(np.float64), requires_grad=True)
    X, T = torch.tensor(x.astype(np.float64)), torch.tensor(t.astype(np.float64))
    W1 = P[mlp.OFF_W1:mlp.OFF_B1].view(128, 16)
    b1 = P[mlp.OFF_B1:mlp.OFF_W2]
    W2 = P[mlp.OFF_W2:mlp.OFF_B2].view(128, 128)
    b2 = P[mlp.OFF_B2:mlp.OFF_W3]
    W3 = P[mlp.OFF_W3:mlp.OFF_B3].view(3, 128)
    b3 = P[mlp.OFF_B3:]
    y = torch.relu(torch.relu(X @ W1.T + b1) @ W2.T + b2) @ W3.T + b3
    L = ((y - T) ** 2).mean()
    L.backward()
    ref = P.grad.numpy()
    assert abs(loss - L.item()) <= 1e-5 * abs(L.item())
    assert np.linalg.norm(g - ref) <= 1e-5 * np.linalg.norm(ref)


def _block_errors(g, ref):
    blocks = {"W1": (mlp.OFF_W1, mlp.OFF_B1), "b1": (mlp.OFF_B1, mlp.OFF_W2),
              "W2": (mlp.OFF_W2, mlp.OFF_B2), "b2": (mlp.OFF_B2, mlp.OFF_W3),
              "W3": (mlp.OFF_W3, mlp.OFF_B3), "b3": (mlp.OFF_B3, mlp.NPARAM)}
    return {k: np.linalg.norm(g[a:b] - ref[a:b]) / max(np.linalg.norm(ref[a:b]), 1e-30)
            for k, (a, b) in blocks.items()}


@pytest.mark.gpu
@pytest.mark.parametrize("n", [1, 100, 128, 1000])
def test_gpu_forward_matches_oracle(ctx, n):
    p = mlp.init_params(5)
    x, _ = _data(n, 2)
    y = mlp.predict_raw(p, x, ctx)
    ref = po.mlp_forward(p, x)
    # BF16 activations: a tie-breaking flip moves an output by ~1e-3 relative
    assert np.allclose(y, ref, rtol=1e-2, atol=2e-3), np.abs(y - ref).max()


@pytest.mark.gpu
@pytest.mark.parametrize("n", [64, 128, 777])
def test_gpu_gradient_matches_oracle(ctx, n):
    p = mlp.init_params(7)
    p[mlp.OFF_B1:mlp.OFF_W2] = 0.02
    x, t = _data(n, 3)
    g, loss = mlp.grad(p, x, t, ctx)
    ref, rloss = po.mlp_grad(p, x, t)
    assert abs(loss - rloss) <= 1e-3 * rloss
    errs = _block_errors(g.astype(np.float64), ref)
    # tolerance: FP32 tensor-core sums vs FP64, plus rare BF16 rounding flips
    assert all(e < 2e-2 for e in errs.values()), errs


@pytest.mark.gpu
def test_gpu_training_reduces_loss_and_beats_linear_fit(ctx):
    x, t = _data(6000, 4)
    xt, tt = _data(2000, 5)
    p0 = mlp.init_params(1)
    p, curve = mlp.train_raw(p0, x, t, epochs=60, batch=512, lr=2e-3, seed=3, ctx=ctx)
    assert np.all(np.isfinite(curve)) and curve[-1] < 0.2 * curve[0]
    mse = float(((mlp.predict_raw(p, xt, ctx) - tt) ** 2).mean())
    A = np.c_[x, np.ones(len(x))]
    coef, *_ = np.linalg.lstsq(A, t, rcond=None)
    lin = float(((np.c_[xt, np.ones(len(xt))] @ coef - tt) ** 2).mean())
    assert mse < 0.5 * lin, (mse, lin)
    # deterministic: same seed, same parameters
    p2, _ = mlp.train_raw(p0, x, t, epochs=60, batch=512, lr=2e-3, seed=3, ctx=ctx)
    assert np.array_equal(p, p2)
