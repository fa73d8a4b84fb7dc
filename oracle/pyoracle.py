"""ctypes front end of the CPU oracle (oracle/oracle.c) and of the
reference-on-CPU pin library (oracle/_ref/libtoref.so).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg as the checker; the product never imports it.
"""
from __future__ import annotations

import ctypes as C
import math
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ORACLE_LIB = HERE / "_build" / "liboracle.so"
REF_LIB = HERE / "_ref" / "libtoref.so"

c_int_p = C.POINTER(C.c_int)
c_double_p = C.POINTER(C.c_double)
c_float_p = C.POINTER(C.c_float)


def _p(a, t):
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data_as(C.POINTER(t))


class OrHabitat(C.Structure):
    _fields_ = [("type", C.c_int), ("max_pop", C.c_double),
                ("pref_mean", C.c_double), ("pref_sd", C.c_double)]


class OrSpeciesIn(C.Structure):
    _fields_ = [("W", C.c_int), ("H", C.c_int), ("res", C.c_int),
                ("xspacing", C.c_double), ("yspacing", C.c_double),
                ("x0", C.c_double), ("y0", C.c_double),
                ("n_hab", C.c_int), ("habs", C.POINTER(OrHabitat)),
                ("hab_map", c_int_p), ("pop_map", c_double_p),
                ("G", C.c_int), ("road", c_double_p),
                ("lambda_mean", C.c_double), ("lambda_sd", C.c_double),
                ("lambda_mult", C.c_double), ("hab_pref_mult", C.c_double),
                ("n_controls", C.c_int), ("hazard", c_double_p), ("sem", C.c_int)]


class OrSpeciesOut(C.Structure):
    _fields_ = [("max_patches", C.c_int), ("n_patches", C.c_int),
                ("area", c_double_p), ("cap", c_double_p), ("pop", c_double_p),
                ("cx", c_double_p), ("cy", c_double_p), ("type", c_int_p),
                ("dists", c_double_p), ("crossings", c_int_p), ("trans", c_double_p),
                ("surv", c_double_p), ("mmm", c_float_p), ("n_transitions", C.c_int)]


_oracle = None
_ref = None


def build_oracle() -> Path:
    from transportoptimiser_gb300 import build as b
    return b.build_oracle()


def oracle() -> C.CDLL:
    global _oracle
    if _oracle is None:
        build_oracle()
        _oracle = C.CDLL(str(ORACLE_LIB))
        _oracle.or_normal.restype = C.c_float
        _oracle.or_normal.argtypes = [C.c_uint64, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]
        _oracle.or_uniform.restype = C.c_float
        _oracle.or_uniform.argtypes = [C.c_uint64, C.c_int, C.c_int, C.c_int, C.c_int, C.c_int]
        _oracle.or_simulate_mte.argtypes = [C.c_int, C.c_int, C.c_int, C.c_float, c_float_p,
                                            c_float_p, c_float_p, c_float_p, C.c_uint64,
                                            C.c_int, C.c_int, C.c_int, C.c_int, c_float_p]
        _oracle.or_exp_pv.argtypes = [C.c_int, C.c_int, c_float_p, C.c_uint64, C.c_int,
                                      C.c_int, c_float_p, c_double_p, c_double_p]
        _oracle.or_fill_stream.argtypes = [C.c_uint64, C.c_int, C.c_int, C.c_int, C.c_int,
                                           C.c_int, C.c_int, C.c_int, c_float_p]
        _oracle.or_fill_pv_stream.argtypes = [C.c_uint64, C.c_int, C.c_int, C.c_int,
                                              C.c_long, c_float_p]
        _oracle.or_species_model.argtypes = [C.POINTER(OrSpeciesIn), C.POINTER(OrSpeciesOut)]
    return _oracle


def ref_available() -> bool:
    return REF_LIB.exists()


def ref() -> C.CDLL:
    """The reference's own kernels compiled for the CPU (only where the
    reference tree is mounted)."""
    global _ref
    if _ref is None:
        if not REF_LIB.exists():
            script = HERE / "build_ref.sh"
            subprocess.run(["sh", str(script)], check=True, capture_output=True)
        if not REF_LIB.exists():
            raise FileNotFoundError("reference pin library not built")
        _ref = C.CDLL(str(REF_LIB))
        _ref.ref_simulate_mte.argtypes = [C.c_int, C.c_int, C.c_int, C.c_float] + [c_float_p] * 9
        _ref.ref_exp_pv.argtypes = [C.c_int, C.c_int] + [c_float_p] * 5 + [c_double_p] * 2
        _ref.ref_build_patches.argtypes = [C.c_int] * 7 + [C.c_double] * 4 + [
            c_int_p, c_double_p] + [c_double_p] * 5 + [c_int_p]
        _ref.ref_line_segment_intersect.argtypes = [C.c_int, c_double_p, C.c_int, c_double_p, c_int_p]
        _ref.ref_label_image.argtypes = [C.c_int, C.c_int, c_int_p, c_int_p]
    return _ref


# ---------------------------------------------------------------------------
# wrappers
# ---------------------------------------------------------------------------
def label_image(W, H, inp, lib=None):
    lib = lib or oracle()
    inp = np.ascontiguousarray(inp, dtype=np.int32)
    out = np.zeros(W * H, dtype=np.int32)
    fn = lib.or_label_image if hasattr(lib, "or_label_image") else lib.ref_label_image
    n = fn(W, H, _p(inp, C.c_int), _p(out, C.c_int))
    return out, n


def build_patches(W, H, skpx, skpy, xres, yres, nreg, xs, ys, spa, maxpop, labels,
                  pops, use_ref=False):
    lib = ref() if use_ref else oracle()
    fn = lib.ref_build_patches if use_ref else lib.or_build_patches
    if not use_ref:
        fn.argtypes = [C.c_int] * 7 + [C.c_double] * 4 + [c_int_p, c_double_p] + [c_double_p] * 5 + [c_int_p]
    cap = xres * yres * max(nreg, 1)
    arrs = [np.zeros(cap) for _ in range(5)]
    n = C.c_int(0)
    labels = np.ascontiguousarray(labels, dtype=np.int32)
    pops = np.ascontiguousarray(pops, dtype=np.float64)
    fn(W, H, skpx, skpy, xres, yres, nreg, xs, ys, spa, maxpop, _p(labels, C.c_int),
       _p(pops, C.c_double), *[_p(a, C.c_double) for a in arrs], C.byref(n))
    k = n.value
    return {"area": arrs[0][:k], "cap": arrs[1][:k], "pop": arrs[2][:k],
            "cx": arrs[3][:k], "cy": arrs[4][:k]}


def line_segment_intersect(xy1_cm, T, xy2_cm, G, use_ref=False):
    lib = ref() if use_ref else oracle()
    fn = lib.ref_line_segment_intersect if use_ref else lib.or_line_segment_intersect
    fn.argtypes = [C.c_int, c_double_p, C.c_int, c_double_p, c_int_p]
    out = np.zeros(T, dtype=np.int32)
    fn(T, _p(np.ascontiguousarray(xy1_cm, np.float64), C.c_double), G,
       _p(np.ascontiguousarray(xy2_cm, np.float64), C.c_double), _p(out, C.c_int))
    return out


def species_model(scene, sp, road, sem=0, max_patches=2048):
    lib = oracle()
    hab = scene.hab_map(road)
    popm = scene.pop_map(sp, hab)
    habs = (OrHabitat * len(sp.habitats))(*[OrHabitat(h.type, h.max_pop, h.pref_mean, h.pref_sd)
                                             for h in sp.habitats])
    segs = road.colmajor()
    hz = np.ascontiguousarray(sp.hazard, dtype=np.float64)
    inp = OrSpeciesIn(scene.W, scene.H, scene.res, 1.0, 1.0, 0.0, 0.0, len(sp.habitats),
                      habs, _p(hab, C.c_int), _p(popm, C.c_double), road.G,
                      _p(segs, C.c_double), sp.lambda_mean, sp.lambda_sd, sp.lambda_mult,
                      sp.hab_pref_mult, len(hz), _p(hz, C.c_double), sem)
    NM = max_patches
    Cn = len(hz)
    bufs = dict(area=np.zeros(NM), cap=np.zeros(NM), pop=np.zeros(NM), cx=np.zeros(NM),
                cy=np.zeros(NM), type=np.zeros(NM, np.int32))
    out = OrSpeciesOut()
    out.max_patches = NM
    for k in ("area", "cap", "pop", "cx", "cy"):
        setattr(out, k, _p(bufs[k], C.c_double))
    out.type = _p(bufs["type"], C.c_int)
    # first pass to learn N is avoided by sizing the N*N arrays for NM
    big = dict(dists=np.zeros(NM * NM), crossings=np.zeros(NM * NM, np.int32),
               trans=np.zeros(NM * NM), surv=np.zeros(Cn * NM * NM),
               mmm=np.zeros(Cn * NM * NM, np.float32))
    out.dists = _p(big["dists"], C.c_double)
    out.crossings = _p(big["crossings"], C.c_int)
    out.trans = _p(big["trans"], C.c_double)
    out.surv = _p(big["surv"], C.c_double)
    out.mmm = _p(big["mmm"], C.c_float)
    N = lib.or_species_model(C.byref(inp), C.byref(out))
    if N < 0:
        raise RuntimeError("oracle: patch capacity exceeded")
    res = {k: v[:N].copy() for k, v in bufs.items()}
    res["N"] = N
    res["n_transitions"] = out.n_transitions
    res["crossings"] = big["crossings"][:N * N].reshape(N, N).copy()
    res["dists"] = big["dists"][:N * N].reshape(N, N).copy()
    res["trans"] = big["trans"][:N * N].reshape(N, N).copy()
    res["surv"] = big["surv"][:Cn * N * N].reshape(Cn, N, N).copy()
    res["mmm"] = big["mmm"][:Cn * N * N].reshape(Cn, N, N).copy()
    res["init_pops"] = res["pop"].astype(np.float32)
    res["caps"] = res["cap"].astype(np.float32)
    return res


def simulate_mte(P, Y, N, dt, params, init, caps, mmm, seed, road, species, sem, threads=1):
    lib = oracle()
    out = np.zeros(P, dtype=np.float32)
    params = np.ascontiguousarray(params, np.float32)
    init = np.ascontiguousarray(init, np.float32)
    caps = np.ascontiguousarray(caps, np.float32)
    mmm = np.ascontiguousarray(mmm, np.float32)
    lib.or_simulate_mte(P, Y, N, dt, _p(params, C.c_float), _p(init, C.c_float),
                        _p(caps, C.c_float), _p(mmm, C.c_float), seed, road, species,
                        sem, threads, _p(out, C.c_float))
    return out


def exp_pv(P, Y, prm9, seed, road, sem):
    lib = oracle()
    vals = np.zeros(P, np.float32)
    m, s = C.c_double(), C.c_double()
    prm = np.ascontiguousarray(prm9, np.float32)
    lib.or_exp_pv(P, Y, _p(prm, C.c_float), seed, road, sem, _p(vals, C.c_float),
                  C.byref(m), C.byref(s))
    return vals, m.value, s.value


def fill_stream(seed, stream, road, normal, P, Y, L, lane_offset=0):
    out = np.zeros(P * Y * L, np.float32)
    oracle().or_fill_stream(seed, stream, road, int(normal), P, Y, L, lane_offset,
                            _p(out, C.c_float))
    return out


def fill_pv_stream(seed, stream, road, normal, n):
    out = np.zeros(n, np.float32)
    oracle().or_fill_pv_stream(seed, stream, road, int(normal), n, _p(out, C.c_float))
    return out


# stream ids (to_math.h)
STREAM = dict(GROWTH=1, SP_BROWNIAN=2, SP_JUMPSIZE=3, SP_JUMP=4, CONTROL=5,
              EX_BROWNIAN=6, EX_JUMPSIZE=7, EX_JUMP=8, ORE=9, PV_BROWNIAN=10,
              PV_JUMPSIZE=11, PV_JUMP=12)


def ref_simulate_mte(P, Y, N, dt, params, init, caps, mmm, seed, road, species):
    """The reference mteKernel on the CPU, fed the same Philox streams."""
    lib = ref()
    N4 = (N + 3) & ~3
    rgr = fill_stream(seed, STREAM["GROWTH"], road, 1, P, Y, N, species * N4)
    br = fill_stream(seed, STREAM["SP_BROWNIAN"], road, 1, P, Y, 1, species)
    js = fill_stream(seed, STREAM["SP_JUMPSIZE"], road, 1, P, Y, 1, species)
    jp = fill_stream(seed, STREAM["SP_JUMP"], road, 0, P, Y, 1, species)
    out = np.zeros(P, np.float32)
    arrs = [np.ascontiguousarray(a, np.float32) for a in (params, init, caps, mmm)]
    lib.ref_simulate_mte(P, Y, N, dt, *[_p(a, C.c_float) for a in arrs],
                         _p(rgr, C.c_float), _p(br, C.c_float), _p(js, C.c_float),
                         _p(jp, C.c_float), _p(out, C.c_float))
    return out


def ref_exp_pv(P, Y, prm9, seed, road):
    """The reference expPVPath on the CPU (overlapping windows, Q11)."""
    lib = ref()
    n = P * Y
    gr, meanP, ts, rrr, cur, rev, jp, nsd, pj = [float(x) for x in prm9]
    zb = fill_pv_stream(seed, STREAM["PV_BROWNIAN"], road, 1, n)
    zj = fill_pv_stream(seed, STREAM["PV_JUMPSIZE"], road, 1, n)
    uj = fill_pv_stream(seed, STREAM["PV_JUMP"], road, 0, n)
    br = (zb * np.float32(nsd)).astype(np.float32)
    pj2 = np.float32(pj) * np.float32(pj)
    js = (zj * pj2 + (-pj2 / np.float32(2.0))).astype(np.float32)
    prm = np.array([gr, meanP, ts, rrr, cur, rev, jp], np.float32)
    vals = np.zeros(P, np.float32)
    m, s = C.c_double(), C.c_double()
    lib.ref_exp_pv(P, Y, _p(prm, C.c_float), _p(br, C.c_float), _p(js, C.c_float),
                   _p(uj, C.c_float), _p(vals, C.c_float), C.byref(m), C.byref(s))
    return vals, m.value, s.value
