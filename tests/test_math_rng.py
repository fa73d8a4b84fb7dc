"""Philox4x32-10 known-answer vectors and the accuracy of the shared
deterministic math (to_math.h) used by both the kernels and the oracle."""
import ctypes as C
import math

import numpy as np

from oracle import pyoracle as po

# Known-answer vectors published with Random123 (Salmon et al., SC'11):
# (counter, key) -> output for philox4x32 with 10 rounds.
KAT = [
    ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
    ((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2, (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
    ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
     (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
]

HELPER = r"""
#include <stdint.h>
#include "to_lsm_math.h"
void kat(const uint32_t* c, const uint32_t* k, uint32_t* o) {
  to_u32x4 r = to_philox4x32_10(c[0], c[1], c[2], c[3], k[0], k[1]);
  for (int i = 0; i < 4; ++i) o[i] = r.v[i];
}
void vlog(const float* x, float* y, int n) { for (int i = 0; i < n; ++i) y[i] = to_logf(x[i]); }
void vexp(const float* x, float* y, int n) { for (int i = 0; i < n; ++i) y[i] = to_expf(x[i]); }
void vsc(const float* x, float* s, float* c, int n) { for (int i = 0; i < n; ++i) to_sincospif(x[i], &s[i], &c[i]); }
void vlogu(const uint32_t* x, float* y, int n) { for (int i = 0; i < n; ++i) y[i] = to_log_u01(x[i]); }
void vsc2(const uint32_t* x, float* s, float* c, int n) { for (int i = 0; i < n; ++i) to_sincos2pi_u01(x[i], &s[i], &c[i]); }
void vdiv(const float* a, const float* b, float* q, int n) { for (int i = 0; i < n; ++i) q[i] = to_div_rcp(a[i], b[i], 1.0f / b[i]); }
float vsolve(int dim, const double* sums) { return to_lsm_solve_compact(dim, sums); }
void vw(const float* d, const float* h, float* w0, float* w1, int n) {
  for (int i = 0; i < n; ++i) { w0[i] = to_lsm_weight(d[i], h[i]); w1[i] = to_lsm_weight_within(d[i], h[i], 1.0f / h[i]); }
}
"""


def _helper(tmp_path_factory):
    import subprocess
    from transportoptimiser_gb300 import build
    d = tmp_path_factory.mktemp("mathhelper")
    src = d / "h.c"
    src.write_text(HELPER)
    so = d / "h.so"
    subprocess.run(["gcc", "-O2", "-ffp-contract=off", "-shared", "-fPIC",
                    "-I", str(build.CSRC), str(src), "-o", str(so), "-lm"], check=True)
    return C.CDLL(str(so))


def test_philox_known_answers(tmp_path_factory):
    h = _helper(tmp_path_factory)
    for ctr, key, want in KAT:
        c = (C.c_uint32 * 4)(*ctr)
        k = (C.c_uint32 * 2)(*key)
        o = (C.c_uint32 * 4)()
        h.kat(c, k, o)
        assert tuple(o) == want


def test_math_accuracy(tmp_path_factory):
    h = _helper(tmp_path_factory)
    fp = C.POINTER(C.c_float)
    x = np.linspace(1e-6, 1.0, 200001, dtype=np.float32)
    y = np.zeros_like(x)
    h.vlog(x.ctypes.data_as(fp), y.ctypes.data_as(fp), len(x))
    ref = np.log(x.astype(np.float64))
    assert np.max(np.abs(y - ref) / np.maximum(np.abs(ref), 1e-30)) < 4e-7
    x = np.linspace(-87.0, 88.0, 200001, dtype=np.float32)
    h.vexp(x.ctypes.data_as(fp), y.ctypes.data_as(fp), len(x))
    ref = np.exp(x.astype(np.float64))
    assert np.max(np.abs(y - ref) / ref) < 2.5e-7
    x = np.linspace(0.0, 2.0, 200001, dtype=np.float32)
    s = np.zeros_like(x); c = np.zeros_like(x)
    h.vsc(x.ctypes.data_as(fp), s.ctypes.data_as(fp), c.ctypes.data_as(fp), len(x))
    assert np.max(np.abs(s - np.sin(math.pi * x.astype(np.float64)))) < 2e-7
    assert np.max(np.abs(c - np.cos(math.pi * x.astype(np.float64)))) < 2e-7


def test_normal_stream_moments():
    z = po.fill_stream(0, po.STREAM["GROWTH"], 0, 1, 200, 50, 40)
    assert abs(z.mean()) < 0.01 and abs(z.std() - 1.0) < 0.01
    u = po.fill_stream(0, po.STREAM["SP_JUMP"], 0, 0, 200, 50, 40)
    assert u.min() >= 0.0 and u.max() < 1.0 and abs(u.mean() - 0.5) < 0.01
    # distinct streams / roads are not the same numbers
    z2 = po.fill_stream(0, po.STREAM["GROWTH"], 1, 1, 200, 50, 40)
    assert abs(np.corrcoef(z, z2)[0, 1]) < 0.02


def test_box_muller_log_and_sincos_accuracy(tmp_path_factory):
    """The table-assisted log and sine/cosine of Box-Muller against double
    precision, over every 24-bit uniform the log sees near 0 and 1 and a
    dense sample between, and every table entry of the angle."""
    h = _helper(tmp_path_factory)
    up = C.POINTER(C.c_uint32)
    fp = C.POINTER(C.c_float)
    rng = np.random.default_rng(1)
    hi = np.arange(1 << 24, dtype=np.uint32)
    words = np.concatenate([hi[:1 << 16], hi[-(1 << 16):], rng.integers(0, 1 << 24, 1 << 20,
                                                                           dtype=np.uint32)])
    x = (words << 8).astype(np.uint32) | rng.integers(0, 256, len(words), dtype=np.uint32)
    y = np.zeros(len(x), np.float32)
    h.vlogu(x.ctypes.data_as(up), y.ctypes.data_as(fp), len(x))
    # the uniform as to_u01_open forms it in float ((x >> 8) + 1/2 rounds
    # above 2^23), then its log in double
    u = ((x >> 8).astype(np.float32) + np.float32(0.5)) * np.float32(2.0 ** -24)
    ref = np.log(u.astype(np.float64))
    # absolute error below 2e-9 near u = 1, relative below 3e-7 elsewhere
    assert np.all(np.abs(y - ref) <= 3e-7 * np.abs(ref) + 2e-9)
    s = np.zeros(len(x), np.float32)
    c = np.zeros(len(x), np.float32)
    h.vsc2(x.ctypes.data_as(up), s.ctypes.data_as(fp), c.ctypes.data_as(fp), len(x))
    ang = 2.0 * math.pi * (x >> 8).astype(np.float64) * 2.0 ** -24
    assert np.max(np.abs(s - np.sin(ang))) < 2.5e-7
    assert np.max(np.abs(c - np.cos(ang))) < 2.5e-7


def test_division_from_reciprocal_is_correctly_rounded(tmp_path_factory):
    """to_div_rcp (Markstein's quotient from the rounded reciprocal) against
    IEEE float division, bit for bit: random significands over the growth
    step's ranges and well beyond them, and divisors with all-ones, all-zero
    and single-bit significands."""
    h = _helper(tmp_path_factory)
    fp = C.POINTER(C.c_float)
    rng = np.random.default_rng(7)
    n = 1 << 22

    def floats(emin, emax, m):
        sig = rng.integers(0, 1 << 23, m, dtype=np.uint32)
        exp = rng.integers(127 + emin, 127 + emax + 1, m, dtype=np.uint32)
        sign = rng.integers(0, 2, m, dtype=np.uint32) << 31
        return (sign | (exp << 23) | sig).view(np.float32)

    a = np.concatenate([floats(-30, 30, n), (rng.standard_normal(n) * 1e4).astype(np.float32)])
    b = np.concatenate([np.abs(floats(-30, 30, n)), rng.uniform(1.0, 1e5, n).astype(np.float32)])
    special = np.array([0x3F7FFFFF, 0x3F800000, 0x3F800001, 0x42C80000, 0x4B7FFFFF, 0x3FFFFFFF],
                       np.uint32).view(np.float32)
    b[:len(special) * 1000] = np.repeat(special, 1000)
    q = np.zeros_like(a)
    h.vdiv(a.ctypes.data_as(fp), b.ctypes.data_as(fp), q.ctypes.data_as(fp), len(a))
    want = a / b
    assert np.array_equal(q.view(np.uint32), want.view(np.uint32))


def test_kernel_weight_within_the_bandwidth_equals_the_general_form(tmp_path_factory):
    """to_lsm_weight_within (the kNN kernel's form: reciprocal of the
    bandwidth once per query, the exponential on [-1/2, 0]) gives the bits of
    to_lsm_weight (the oracle's form) for every distance 0 <= d <= h: the
    kernel's case, d and h square roots of float squared distances with h the
    largest, over the whole float range of such keys, and the edges d = 0,
    d = h and d one ulp below h."""
    h = _helper(tmp_path_factory)
    fp = C.POINTER(C.c_float)
    rng = np.random.default_rng(11)
    n = 1 << 21
    # squared distances: log-uniform over the positive floats a key can take
    kmax = np.exp(rng.uniform(np.log(1e-44), np.log(1e30), n)).astype(np.float32)
    kmax = np.maximum(kmax, np.float32(1.4e-45))
    key = (kmax * rng.uniform(0.0, 1.0, n).astype(np.float32)).astype(np.float32)
    hh = np.sqrt(kmax).astype(np.float32)
    dd = np.sqrt(np.minimum(key, kmax)).astype(np.float32)
    m = n // 8
    dd[:m] = 0.0
    dd[m:2 * m] = hh[m:2 * m]
    dd[2 * m:3 * m] = np.nextafter(hh[2 * m:3 * m], np.float32(0.0))
    # the bench's scale: normalised coordinates, bandwidths 1e-3 .. 1
    hh[3 * m:4 * m] = rng.uniform(1e-3, 1.0, m).astype(np.float32)
    dd[3 * m:4 * m] = (hh[3 * m:4 * m] * rng.uniform(0.0, 1.0, m)).astype(np.float32)
    assert np.all(dd <= hh) and np.all(hh > 0)
    w0 = np.zeros(n, np.float32)
    w1 = np.zeros(n, np.float32)
    h.vw(dd.ctypes.data_as(fp), hh.ctypes.data_as(fp), w0.ctypes.data_as(fp),
         w1.ctypes.data_as(fp), n)
    assert np.array_equal(w0.view(np.uint32), w1.view(np.uint32))


def _compact_sums(dx, y, z):
    """The normal-equation sums of a weighted local linear fit in the solve's
    compact order: B (sum y w_i z, w = [1, dx]), then the upper triangle of
    A (sum w_i w_j z) row by row."""
    w = np.concatenate([np.ones((len(y), 1)), dx], axis=1)
    m = w.shape[1]
    B = (w * (y * z)[:, None]).sum(0)
    A = (w * z[:, None]).T @ w
    return np.concatenate([B, [A[i, j] for i in range(m) for j in range(i, m)]])


def test_regression_solve_matches_weighted_least_squares(tmp_path_factory):
    """to_lsm_solve_compact (FP64 square-root-free Cholesky, intercept last,
    every update one fused multiply-add) returns the intercept of the
    weighted least-squares fit, against numpy's float64 solution, for local
    fits of 3 and 4 state dimensions; a state dimension constant over the
    neighbours is dropped and the fit of the others returned."""
    h = _helper(tmp_path_factory)
    h.vsolve.restype = C.c_float
    h.vsolve.argtypes = [C.c_int, C.POINTER(C.c_double)]
    rng = np.random.default_rng(5)
    for case in range(400):
        d = 3 + case % 2
        n = 65
        dx = rng.normal(0.0, 0.1, (n, d))
        coef = rng.normal(0.0, 1.0, d + 1)
        y = coef[0] + dx @ coef[1:] + rng.normal(0.0, 0.05, n)
        z = np.exp(-rng.uniform(0.0, 0.5, n)) * 0.3989422804
        if case % 5 == 4:
            dx[:, case % d] = 0.0          # a direction the neighbours do not span
        sums = _compact_sums(dx, y, z)
        got = h.vsolve(d, sums.ctypes.data_as(C.POINTER(C.c_double)))
        keep = [j for j in range(d) if np.any(dx[:, j] != 0.0)]
        w = np.concatenate([np.ones((n, 1)), dx[:, keep]], axis=1)
        sw = np.sqrt(z)
        want = np.linalg.lstsq(w * sw[:, None], y * sw, rcond=None)[0][0]
        assert abs(got - want) <= 1e-6 * max(1.0, abs(want)), (case, got, want)
