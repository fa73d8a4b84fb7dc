"""Adjoint (pathwise sensitivities with the exercise policy frozen) against
FP64 central finite differences of the oracle at common random numbers."""
import numpy as np
import pytest

from oracle import pyoracle as po
from transportoptimiser_gb300 import synth
from transportoptimiser_gb300.adjoint import theta_from_problem
from transportoptimiser_gb300.rov import rov_problem_from_models

REL_STEP = 1e-4


def _problem(P=600, Y=30, seed=3):
    sc = synth.rov_road(0, n_species=2)
    models = [po.species_model(sc, sc.species[s], sc.roads[0], sem=1) for s in range(2)]
    rp = rov_problem_from_models(models, sc, n_paths=P, n_years=Y, dim_res=8, sem=1,
                                 n_processes=3, demand=True, seed=seed)
    hz = np.asarray(sc.species[0].hazard, np.float64)
    assert all(np.array_equal(hz, s.hazard) for s in sc.species)
    cross = [m["crossings"] for m in models]
    return rp, cross, hz


def _fd_jacobian(rp, ctl, cross, hz, theta):
    cols = []
    for i in range(theta.size):
        h = REL_STEP * max(abs(theta[i]), 1.0)
        tp, tm = theta.copy(), theta.copy()
        tp[i] += h
        tm[i] -= h
        cols.append((po.adjoint_forward(rp, ctl, cross, hz, tp) -
                     po.adjoint_forward(rp, ctl, cross, hz, tm)) / (2 * h))
    return np.stack(cols, axis=1)


def test_oracle_finite_differences_converge():
    rp, cross, hz = _problem(P=200, Y=20)
    rng = np.random.default_rng(0)
    ctl = rng.integers(0, 3, size=(rp["n_years"], rp["n_paths"])).astype(np.int32)
    th = theta_from_problem(rp, hz)
    for i in (0, 4, 6, 9, 12):
        d = []
        for h in (1e-3, 5e-4):
            step = h * max(abs(th[i]), 1.0)
            tp, tm = th.copy(), th.copy()
            tp[i] += step
            tm[i] -= step
            d.append((po.adjoint_forward(rp, ctl, cross, hz, tp) -
                      po.adjoint_forward(rp, ctl, cross, hz, tm)) / (2 * step))
        scale = np.abs(d[1]).max() + 1e-12
        assert np.abs(d[0] - d[1]).max() <= 1e-4 * scale, (i, d)


@pytest.mark.gpu
def test_gpu_forward_matches_fp64_oracle(ctx):
    from transportoptimiser_gb300.adjoint import FrozenPolicy
    rp, cross, hz = _problem()
    rng = np.random.default_rng(1)
    ctl = rng.integers(0, 3, size=(rp["n_years"], rp["n_paths"])).astype(np.int32)
    th = theta_from_problem(rp, hz)
    fp = FrozenPolicy(rp, ctl, cross, hz, ctx)
    out, tape = fp.forward(th)
    fp.free(tape)
    ref = po.adjoint_forward(rp, ctl, cross, hz, th)
    np.testing.assert_allclose(out, ref, rtol=1e-4)


@pytest.mark.gpu
def test_gpu_adjoint_matches_fp64_finite_differences(ctx):
    from transportoptimiser_gb300 import simulate_gpu as sg
    from transportoptimiser_gb300.adjoint import FrozenPolicy
    rp, cross, hz = _problem()
    # the exercise policy of a forward LSM valuation, frozen
    rov = sg.simulateROVCUDA(rp, want=("opt_cont",), ctx=ctx)
    ctl = rov["opt_cont"].reshape(rp["n_years"], rp["n_paths"]).astype(np.int32)
    th = theta_from_problem(rp, hz)
    fp = FrozenPolicy(rp, ctl, cross, hz, ctx)
    out, J = fp.jacobian(th)
    Jfd = _fd_jacobian(rp, ctl, cross, hz, th)
    assert J.shape == (3, 13)
    for r in range(3):
        scale = np.abs(Jfd[r]).max()
        assert scale > 0
        err = np.abs(J[r] - Jfd[r])
        assert np.all(err <= 2e-3 * np.abs(Jfd[r]) + 1e-3 * scale), (r, J[r], Jfd[r])


@pytest.mark.gpu
def test_autograd_function_backward_is_the_adjoint(ctx):
    torch = pytest.importorskip("torch")
    from transportoptimiser_gb300.adjoint import FrozenPolicy, autograd_function
    rp, cross, hz = _problem(P=300, Y=20)
    rng = np.random.default_rng(2)
    ctl = rng.integers(0, 3, size=(rp["n_years"], rp["n_paths"])).astype(np.int32)
    th = theta_from_problem(rp, hz)
    fp = FrozenPolicy(rp, ctl, cross, hz, ctx)
    f = autograd_function()
    theta = torch.tensor(th, requires_grad=True)
    out = f.apply(theta, fp)
    w = torch.tensor([0.3, -1.0, 2.0], dtype=torch.float64)
    (out * w).sum().backward()
    o2, tape = fp.forward(th)
    g = fp.backward(tape, w.numpy())
    fp.free(tape)
    np.testing.assert_allclose(out.detach().numpy(), o2, rtol=1e-12)
    np.testing.assert_allclose(theta.grad.numpy(), g, rtol=1e-12, atol=0)
