"""Pathwise sensitivities of the controlled road valuation with the
exercise policy frozen (``to_adjoint_forward`` / ``to_adjoint_backward``,
include/transopt.h), and a ``torch.autograd.Function`` over them.

Parameters theta (2U + 2S + C), in order: OU reversion theta_u, OU
volatility sigma_u, growth-rate mean mu_s (species params[1]), growth
variability v_s (species params[7]), crossing hazard h_c.  Outputs
(1 + S): expected PV of the controlled flow's unit profits and the
expected end population of each species.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _capi
from ._capi import Context, ptr
from .simulate_gpu import context, rov_ctypes


class AdjointProblem(C.Structure):
    _fields_ = [("rov", C.POINTER(_capi.RovProblem)), ("controls", C.POINTER(C.c_int)),
                ("crossings", C.POINTER(C.POINTER(C.c_int))), ("hazard", C.POINTER(C.c_double))]


def theta_from_problem(problem: dict, hazard) -> np.ndarray:
    """theta at the problem's own values."""
    unc = np.asarray(problem["uncert"], np.float64).reshape(-1, 6)
    sp = [np.asarray(s["params"], np.float64) for s in problem["species"]]
    return np.concatenate([unc[:, 3], unc[:, 2], [p[1] for p in sp], [p[7] for p in sp],
                           np.asarray(hazard, np.float64)])


class FrozenPolicy:
    """A frozen-policy valuation bound to a problem, controls and crossings."""

    def __init__(self, problem: dict, controls: np.ndarray, crossings, hazard,
                 ctx: Context | None = None):
        self.ctx = ctx or context()
        self.S = len(problem["species"])
        self.C = len(problem["flows"])
        self.U = len(problem["uncert"]) // 6
        self.ntheta = 2 * self.U + 2 * self.S + self.C
        self._pr, self._keep = rov_ctypes(problem)
        self._ctl = np.ascontiguousarray(controls, np.int32).reshape(-1)
        self._cross = [np.ascontiguousarray(x, np.int32) for x in crossings]
        self._xp = (C.POINTER(C.c_int) * self.S)(*[ptr(x, C.c_int) for x in self._cross])
        self._hz = np.ascontiguousarray(hazard, np.float64)
        self._adj = AdjointProblem(C.pointer(self._pr), ptr(self._ctl, C.c_int), self._xp,
                                   ptr(self._hz, C.c_double))

    def forward(self, theta, keep_tape=True):
        th = np.ascontiguousarray(theta, np.float64)
        out = np.zeros(1 + self.S)
        tape = C.c_void_p()
        self.ctx.check(self.ctx.lib.to_adjoint_forward(
            self.ctx.handle, C.byref(self._adj), ptr(th, C.c_double), ptr(out, C.c_double),
            C.byref(tape) if keep_tape else None), "to_adjoint_forward")
        return out, (tape if keep_tape else None)

    def backward(self, tape, grad_out) -> np.ndarray:
        go = np.ascontiguousarray(grad_out, np.float64)
        g = np.zeros(self.ntheta)
        self.ctx.check(self.ctx.lib.to_adjoint_backward(self.ctx.handle, tape, ptr(go, C.c_double),
                                                        ptr(g, C.c_double)), "to_adjoint_backward")
        return g

    def free(self, tape) -> None:
        if tape:
            self.ctx.lib.to_tape_destroy(tape)

    def jacobian(self, theta) -> tuple[np.ndarray, np.ndarray]:
        out, tape = self.forward(theta)
        try:
            J = np.stack([self.backward(tape, np.eye(1 + self.S)[i]) for i in range(1 + self.S)])
        finally:
            self.free(tape)
        return out, J


def autograd_function():
    """torch.autograd.Function over a FrozenPolicy (torch imported lazily)."""
    import torch

    class FrozenPolicyValue(torch.autograd.Function):
        @staticmethod
        def forward(fctx, theta, model: FrozenPolicy):
            out, tape = model.forward(theta.detach().cpu().double().numpy())
            fctx.model, fctx.tape = model, tape
            return torch.from_numpy(out)

        @staticmethod
        def backward(fctx, grad_out):
            g = fctx.model.backward(fctx.tape, grad_out.detach().cpu().double().numpy())
            fctx.model.free(fctx.tape)
            fctx.tape = None
            return torch.from_numpy(g), None

    return FrozenPolicyValue
