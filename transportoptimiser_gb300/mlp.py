"""Learned surrogate of the road-evaluation outputs: an MLP 16 -> 128 -> 128
-> 3 whose GEMMs run on the GB300's tensor cores (BF16 operands, FP32
accumulation) in this library's own forward and backward kernels
(``to_mlp_*`` in include/transopt.h).

The reference's GA fitness uses local-linear grid surrogates
(SimulateGPU.cu:5533-5917, ``buildSurrogate*CUDA``); it has no learned
model.  Here the MLP screens designs, and the plain Monte Carlo stays the
fallback and the measure of its error.

Parameter vector layout (FP32, ``NPARAM``): W1[128][16], b1[128],
W2[128][128], b2[128], W3[3][128], b3[3].
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._capi import Context, ptr
from .simulate_gpu import context

IN, HID, OUT = 16, 128, 3
NPARAM = HID * IN + HID + HID * HID + HID + OUT * HID + OUT
OFF_W1, OFF_B1 = 0, HID * IN
OFF_W2 = OFF_B1 + HID
OFF_B2 = OFF_W2 + HID * HID
OFF_W3 = OFF_B2 + HID
OFF_B3 = OFF_W3 + OUT * HID


def init_params(seed: int = 0) -> np.ndarray:
    """He-uniform weights, zero biases (seeded)."""
    rng = np.random.default_rng(seed)
    p = np.zeros(NPARAM, np.float32)

    def he(n_out, n_in):
        lim = np.sqrt(6.0 / n_in)
        return rng.uniform(-lim, lim, size=n_out * n_in).astype(np.float32)

    p[OFF_W1:OFF_B1] = he(HID, IN)
    p[OFF_W2:OFF_B2] = he(HID, HID)
    p[OFF_W3:OFF_B3] = he(OUT, HID) * 0.5
    return p


def _f32(a, shape1):
    a = np.ascontiguousarray(a, np.float32)
    if a.ndim != 2 or a.shape[1] != shape1:
        raise ValueError(f"expected rows of {shape1} floats, got {a.shape}")
    return a


def predict_raw(params: np.ndarray, x: np.ndarray, ctx: Context | None = None) -> np.ndarray:
    """y = f(x) on the GPU for raw (already scaled) inputs."""
    ctx = ctx or context()
    p = np.ascontiguousarray(params, np.float32)
    x = _f32(x, IN)
    y = np.zeros((x.shape[0], OUT), np.float32)
    ctx.check(ctx.lib.to_mlp_predict(ctx.handle, ptr(p, C.c_float), x.shape[0], ptr(x, C.c_float),
                                     ptr(y, C.c_float)), "to_mlp_predict")
    return y


def grad(params: np.ndarray, x: np.ndarray, t: np.ndarray, ctx: Context | None = None):
    """Gradient of mean((f(x) - t)^2) and that loss, on the GPU."""
    ctx = ctx or context()
    p = np.ascontiguousarray(params, np.float32)
    x = _f32(x, IN)
    t = _f32(t, OUT)
    g = np.zeros(NPARAM, np.float32)
    loss = C.c_double(0.0)
    ctx.check(ctx.lib.to_mlp_grad(ctx.handle, ptr(p, C.c_float), x.shape[0], ptr(x, C.c_float),
                                  ptr(t, C.c_float), ptr(g, C.c_float), C.byref(loss)),
              "to_mlp_grad")
    return g, loss.value


def train_raw(params: np.ndarray, x: np.ndarray, t: np.ndarray, epochs: int = 100,
              batch: int = 512, lr: float = 1e-3, seed: int = 0,
              ctx: Context | None = None):
    """Adam training on the GPU; returns (new params, per-epoch loss)."""
    ctx = ctx or context()
    p = np.array(params, np.float32, copy=True)
    x = _f32(x, IN)
    t = _f32(t, OUT)
    curve = np.zeros(max(epochs, 1), np.float64)
    ctx.check(ctx.lib.to_mlp_train(ctx.handle, ptr(p, C.c_float), x.shape[0], ptr(x, C.c_float),
                                   ptr(t, C.c_float), epochs, batch, float(lr), seed,
                                   ptr(curve, C.c_double)), "to_mlp_train")
    return p, curve[:epochs]


class MLPSurrogate:
    """Standardises inputs and outputs, trains and predicts on the GPU."""

    def __init__(self, seed: int = 0):
        self.params = init_params(seed)
        self.seed = seed
        self.x_mu = np.zeros(IN, np.float32)
        self.x_sd = np.ones(IN, np.float32)
        self.y_mu = np.zeros(OUT, np.float32)
        self.y_sd = np.ones(OUT, np.float32)
        self.loss_curve = np.zeros(0)

    def fit(self, x, y, epochs=150, batch=512, lr=2e-3, ctx: Context | None = None):
        x = np.asarray(x, np.float32)
        y = np.asarray(y, np.float32)
        self.x_mu = x.mean(0)
        self.x_sd = np.where(x.std(0) > 1e-12, x.std(0), 1.0).astype(np.float32)
        self.y_mu = y.mean(0)
        self.y_sd = np.where(y.std(0) > 1e-12, y.std(0), 1.0).astype(np.float32)
        xs = (x - self.x_mu) / self.x_sd
        ys = (y - self.y_mu) / self.y_sd
        self.params, self.loss_curve = train_raw(self.params, xs, ys, epochs, batch, lr,
                                                 self.seed, ctx)
        return self

    def predict(self, x, ctx: Context | None = None) -> np.ndarray:
        xs = (np.asarray(x, np.float32) - self.x_mu) / self.x_sd
        return predict_raw(self.params, xs, ctx) * self.y_sd + self.y_mu
