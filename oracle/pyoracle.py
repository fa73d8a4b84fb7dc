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
                ("surv", c_double_p), ("mmm", c_float_p), ("n_transitions", C.c_int),
                ("iar", c_double_p)]


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
        _oracle.or_knn.argtypes = [c_float_p, C.c_int, c_float_p, C.c_int, C.c_int, C.c_int,
                                   c_float_p, c_int_p]
        _oracle.or_build_surrogate_1d.argtypes = [C.c_int, c_float_p, c_float_p, C.c_int,
                                                  c_float_p]
        _oracle.or_build_surrogate_nd.argtypes = [C.c_int, C.c_int, c_float_p, c_float_p,
                                                  C.c_int, C.c_int, C.c_int, c_float_p]
        _oracle.or_bf16.restype = C.c_float
        _oracle.or_bf16.argtypes = [C.c_float]
        _oracle.or_mlp_set_rounding.argtypes = [C.c_int]
        _oracle.or_mlp_forward.argtypes = [c_float_p, C.c_int, c_float_p, c_float_p]
        _oracle.or_mlp_grad.argtypes = [c_float_p, C.c_int, c_float_p, c_float_p, c_double_p,
                                        c_double_p]
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
        _ref.ref_knn.argtypes = [c_float_p, C.c_int, c_float_p, C.c_int, C.c_int, C.c_int,
                                 c_float_p, c_int_p]
        _ref.ref_build_surrogate_rov.argtypes = [C.c_int, C.c_int, c_float_p, c_float_p,
                                                 C.c_int, C.c_int, c_float_p]
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


def species_model(scene, sp, road, sem=0, max_patches=2048, hab=None):
    """or_species_model on a synthetic scene's road; hab: the road's habitat
    map (scene.hab_map(road)) when the caller has it already."""
    lib = oracle()
    hab = scene.hab_map(road) if hab is None else hab
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
    iar = np.zeros(Cn)
    out.iar = _p(iar, C.c_double)
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
    res["iar"] = iar
    return res


def road_cells(points, W, H, sem=1, xs=1.0, ys=1.0):
    """or_road_cells: RoadCells::computeRoadCells of a polyline (n x 2)."""
    lib = oracle()
    lib.or_road_cells.restype = C.c_int
    lib.or_road_cells.argtypes = [C.c_int, c_double_p, c_double_p, C.c_int, C.c_int,
                                  C.c_double, C.c_double, C.c_int, c_int_p, C.c_int]
    pts = np.asarray(points, np.float64)
    x = np.ascontiguousarray(pts[:, 0])
    y = np.ascontiguousarray(pts[:, 1])
    cap = 4 * W * H if W * H < 1 << 20 else 1 << 22
    out = np.zeros(cap, np.int32)
    n = lib.or_road_cells(len(x), _p(x, C.c_double), _p(y, C.c_double), W, H, xs, ys, sem,
                          _p(out, C.c_int), cap)
    return out[:n].copy()


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


# ---------------------------------------------------------------------------
# ROV (oracle_rov.c) and the reference ALGO4 on the CPU
# ---------------------------------------------------------------------------
class OrRovProblem(C.Structure):
    _fields_ = [("n_paths", C.c_int), ("n_years", C.c_int), ("n_species", C.c_int),
                ("n_controls", C.c_int), ("n_uncertainties", C.c_int), ("dim_res", C.c_int),
                ("n_patches", c_int_p), ("params", C.POINTER(c_float_p)),
                ("params_flat", c_float_p), ("init_pops", C.POINTER(c_float_p)),
                ("caps", C.POINTER(c_float_p)), ("mmm", C.POINTER(c_float_p)),
                ("flows", c_float_p), ("uncert", c_float_p), ("n_fuels", C.c_int),
                ("fuel_costs", c_float_p), ("fuel_idx", c_int_p), ("n_commodities", C.c_int),
                ("ore_content", c_float_p), ("ore_sd", c_float_p), ("unit_cost", C.c_float),
                ("unit_revenue", C.c_float), ("dt", C.c_float), ("rrr", C.c_float),
                ("scaling", C.c_float), ("demand_idx", C.c_int), ("seed", C.c_uint64),
                ("road", C.c_int), ("sem", C.c_int), ("n_threads", C.c_int),
                ("algo", C.c_int)]


class OrRovResult(C.Structure):
    _fields_ = [("cond_exp", c_float_p), ("opt_cont", c_int_p), ("unit_profits", c_float_p),
                ("adj_pops", c_float_p), ("regression", c_float_p), ("controls", c_int_p),
                ("total_pops", c_float_p), ("aars", c_float_p), ("u_results", c_float_p),
                ("stats", C.c_double * 3), ("value_se", C.c_double), ("n_best", C.c_int)]


def rov_problem_arrays(rp):
    """Normalise a ROV problem dict (see transportoptimiser_gb300.rov) into
    contiguous arrays; returns (arrays dict)."""
    S = len(rp["species"])
    out = dict(S=S)
    out["N"] = np.array([sp["N"] for sp in rp["species"]], np.int32)
    out["params"] = [np.ascontiguousarray(sp["params"], np.float32) for sp in rp["species"]]
    out["init"] = [np.ascontiguousarray(sp["init_pops"], np.float32) for sp in rp["species"]]
    out["caps"] = [np.ascontiguousarray(sp["caps"], np.float32) for sp in rp["species"]]
    out["mmm"] = [np.ascontiguousarray(sp["mmm"], np.float32) for sp in rp["species"]]
    out["flat"] = np.ascontiguousarray(np.concatenate(out["params"]), np.float32)
    for k in ("flows", "uncert", "fuel_costs", "ore_content", "ore_sd"):
        out[k] = np.ascontiguousarray(rp[k], np.float32)
    out["fuel_idx"] = np.ascontiguousarray(rp["fuel_idx"], np.int32)
    return out


def simulate_rov(rp, threads=1, want_paths=False):
    lib = oracle()
    lib.or_simulate_rov.argtypes = [C.POINTER(OrRovProblem), C.POINTER(OrRovResult)]
    a = rov_problem_arrays(rp)
    S, P, Y, C_, R = a["S"], rp["n_paths"], rp["n_years"], len(rp["flows"]), rp["dim_res"]
    U = len(rp["uncert"]) // 6
    fp = lambda arrs: (c_float_p * len(arrs))(*[_p(x, C.c_float) for x in arrs])
    pr = OrRovProblem(P, Y, S, C_, U, R, _p(a["N"], C.c_int), fp(a["params"]),
                      _p(a["flat"], C.c_float), fp(a["init"]), fp(a["caps"]), fp(a["mmm"]),
                      _p(a["flows"], C.c_float), _p(a["uncert"], C.c_float),
                      len(a["fuel_costs"]), _p(a["fuel_costs"], C.c_float),
                      _p(a["fuel_idx"], C.c_int), len(a["ore_content"]),
                      _p(a["ore_content"], C.c_float), _p(a["ore_sd"], C.c_float),
                      rp["unit_cost"], rp["unit_revenue"], rp["dt"], rp["rrr"], 2.0,
                      rp.get("demand_idx", -1), rp["seed"], rp["road"], rp["sem"], threads,
                      int(rp.get("algo", 4)))
    d = S + 1
    blk = R * d + 2 * R ** d
    res = dict(cond_exp=np.zeros(P * Y, np.float32), opt_cont=np.zeros(P * Y, np.int32),
               unit_profits=np.zeros(P * Y, np.float32), adj_pops=np.zeros(Y * S * P, np.float32),
               regression=np.zeros(Y * C_ * blk, np.float32))
    extra = {}
    if want_paths:
        extra = dict(controls=np.zeros(P * Y, np.int32),
                     total_pops=np.zeros(P * (Y + 1) * S, np.float32),
                     aars=np.zeros(P * (Y + 1) * S * C_, np.float32),
                     u_results=np.zeros(P * (Y + 1) * U, np.float32))
    r = OrRovResult()
    r.cond_exp = _p(res["cond_exp"], C.c_float)
    r.opt_cont = _p(res["opt_cont"], C.c_int)
    r.unit_profits = _p(res["unit_profits"], C.c_float)
    r.adj_pops = _p(res["adj_pops"], C.c_float)
    r.regression = _p(res["regression"], C.c_float)
    for k, v in extra.items():
        setattr(r, k, _p(v, C.c_int if v.dtype == np.int32 else C.c_float))
    assert lib.or_simulate_rov(C.byref(pr), C.byref(r)) == 0
    res.update(extra)
    res["stats"] = np.array(list(r.stats))
    res["value_se"] = r.value_se
    res["n_best"] = r.n_best
    return res


def ref_simulate_rov(rp):
    """The reference's ALGO4 (one species) on the CPU, fed the same streams."""
    lib = ref()
    assert len(rp["species"]) == 1
    sp = rp["species"][0]
    P, Y, R = rp["n_paths"], rp["n_years"], rp["dim_res"]
    N = int(sp["N"])
    C_ = len(rp["flows"])
    U = len(rp["uncert"]) // 6
    Cm = len(rp["ore_content"])
    seed, road = rp["seed"], rp["road"]
    N4 = (N + 3) & ~3
    rand_cont = fill_stream(seed, STREAM["CONTROL"], road, 0, P, Y, 1, 0)
    rgr = fill_stream(seed, STREAM["GROWTH"], road, 1, P, Y, N, 0)
    sp_br = fill_stream(seed, STREAM["SP_BROWNIAN"], road, 1, P, Y, 1, 0)
    sp_js = fill_stream(seed, STREAM["SP_JUMPSIZE"], road, 1, P, Y, 1, 0)
    sp_jp = fill_stream(seed, STREAM["SP_JUMP"], road, 0, P, Y, 1, 0)
    ex_br = fill_stream(seed, STREAM["EX_BROWNIAN"], road, 1, P, Y, U, 0)
    ex_js = fill_stream(seed, STREAM["EX_JUMPSIZE"], road, 1, P, Y, U, 0)
    ex_jp = fill_stream(seed, STREAM["EX_JUMP"], road, 0, P, Y, U, 0)
    zore = fill_pv_stream(seed, STREAM["ORE"], road, 1, P * Y * max(Cm, 1))
    ucomp = np.zeros(P * Y * max(Cm, 1), np.float32)
    for c in range(Cm):
        sl = slice(c * P * Y, (c + 1) * P * Y)
        ucomp[sl] = np.float32(rp["ore_content"][c]) + np.float32(rp["ore_sd"][c]) * zore[sl]
    d = 2
    blk = R * d + 2 * R ** d
    out = dict(cond_exp=np.zeros(P * Y, np.float32), opt_cont=np.zeros(P * Y, np.int32),
               unit_profits=np.zeros(P * Y, np.float32), adj_pops=np.zeros(Y * P, np.float32),
               regression=np.zeros(Y * C_ * blk, np.float32), stats=np.zeros(3, np.float32))
    f32 = lambda x: np.ascontiguousarray(x, np.float32)
    args = [P, Y, N, C_, U, R, C.c_float(rp["dt"]), f32(sp["params"]), f32(sp["init_pops"]),
            f32(sp["caps"]), f32(sp["mmm"]), f32(rp["flows"]), f32(rp["uncert"]),
            len(rp["fuel_costs"]), f32(rp["fuel_costs"]),
            np.ascontiguousarray(rp["fuel_idx"], np.int32), Cm,
            C.c_float(rp["unit_cost"]), C.c_float(rp["unit_revenue"]), C.c_float(rp["rrr"]),
            rand_cont, rgr, sp_br, sp_js, sp_jp, ex_br, ex_js, ex_jp, ucomp,
            out["cond_exp"], out["opt_cont"], out["unit_profits"], out["adj_pops"],
            out["regression"], out["stats"]]
    conv = []
    for x in args:
        if isinstance(x, np.ndarray):
            conv.append(_p(x, C.c_int if x.dtype == np.int32 else C.c_float))
        else:
            conv.append(x)
    lib.ref_simulate_rov(*conv)
    return out


def knn(ref_pts, n, query, Q, dim, k, use_ref=False):
    dist = np.zeros(k * Q, np.float32)
    ind = np.zeros(k * Q, np.int32)
    rp_ = np.ascontiguousarray(ref_pts, np.float32)
    q_ = np.ascontiguousarray(query, np.float32)
    if use_ref:
        ref().ref_knn(_p(rp_, C.c_float), n, _p(q_, C.c_float), Q, dim, k,
                      _p(dist, C.c_float), _p(ind, C.c_int))
    else:
        oracle().or_knn(_p(rp_, C.c_float), n, _p(q_, C.c_float), Q, dim, k,
                        _p(dist, C.c_float), _p(ind, C.c_int))
    return dist, ind


def build_surrogate_1d(x, y, R):
    out = np.zeros(2 * R, np.float32)
    x = np.ascontiguousarray(x, np.float32); y = np.ascontiguousarray(y, np.float32)
    oracle().or_build_surrogate_1d(len(x), _p(x, C.c_float), _p(y, C.c_float), R,
                                   _p(out, C.c_float))
    return out


def build_surrogate_nd(pred, y, R, sem=0, clip=1, use_ref=False):
    pred = np.ascontiguousarray(pred, np.float32)
    d, n = pred.shape
    y = np.ascontiguousarray(y, np.float32)
    out = np.zeros(R * d + R ** d, np.float32)
    if use_ref:
        ref().ref_build_surrogate_rov(n, d, _p(pred, C.c_float), _p(y, C.c_float), R, clip,
                                      _p(out, C.c_float))
    else:
        oracle().or_build_surrogate_nd(n, d, _p(pred, C.c_float), _p(y, C.c_float), R, sem, clip,
                                       _p(out, C.c_float))
    return out


# ---- learned surrogate (oracle_mlp.c) ----------------------------------------
def mlp_forward(params, x):
    p = np.ascontiguousarray(params, np.float32)
    x = np.ascontiguousarray(x, np.float32)
    y = np.zeros((x.shape[0], 3), np.float32)
    oracle().or_mlp_forward(_p(p, C.c_float), x.shape[0], _p(x, C.c_float), _p(y, C.c_float))
    return y


def mlp_grad(params, x, t, rounding=True):
    oracle().or_mlp_set_rounding(1 if rounding else 0)
    p = np.ascontiguousarray(params, np.float32)
    x = np.ascontiguousarray(x, np.float32)
    t = np.ascontiguousarray(t, np.float32)
    g = np.zeros(p.size, np.float64)
    loss = C.c_double(0.0)
    oracle().or_mlp_grad(_p(p, C.c_float), x.shape[0], _p(x, C.c_float), _p(t, C.c_float),
                         _p(g, C.c_double), C.byref(loss))
    oracle().or_mlp_set_rounding(1)
    return g, loss.value


# ---- frozen-policy valuation in FP64 (oracle_adjoint.c) ----------------------
class OrAdjProblem(C.Structure):
    _fields_ = [("P", C.c_int), ("Y", C.c_int), ("S", C.c_int), ("C", C.c_int), ("U", C.c_int),
                ("NP", C.c_int), ("dt", C.c_float), ("rrr", C.c_float), ("seed", C.c_uint64),
                ("road", C.c_int), ("uncert", c_float_p), ("flows", c_float_p), ("nF", C.c_int),
                ("fuel_costs", c_float_p), ("fuel_idx", c_int_p), ("Cm", C.c_int),
                ("ore_content", c_float_p), ("ore_sd", c_float_p), ("unit_cost", C.c_float),
                ("unit_revenue", C.c_float), ("demand_idx", C.c_int), ("controls", c_int_p),
                ("n_patches", c_int_p), ("params", c_float_p), ("init_pops", c_float_p),
                ("caps", c_float_p), ("mmm", c_float_p), ("cross", c_int_p),
                ("base_h", c_double_p)]


def adjoint_forward(problem, controls, crossings, hazard, theta, threads=None):
    """E[PV], E[end population_s] of the frozen-policy model in FP64."""
    lib = oracle()
    lib.or_adjoint_forward.argtypes = [C.POINTER(OrAdjProblem), c_double_p, c_double_p, C.c_int]
    sps = problem["species"]
    S, Cn = len(sps), len(problem["flows"])
    NP = max(int(s["N"]) for s in sps)
    NP = (NP + 3) & ~3
    keep = []

    def f32(a):
        a = np.ascontiguousarray(a, np.float32)
        keep.append(a)
        return _p(a, C.c_float)

    def i32(a):
        a = np.ascontiguousarray(a, np.int32)
        keep.append(a)
        return _p(a, C.c_int)

    ip = np.zeros((S, NP), np.float32)
    cp = np.ones((S, NP), np.float32)
    mm = np.zeros((S, Cn, NP, NP), np.float32)
    cr = np.zeros((S, NP, NP), np.int32)
    for s, sp in enumerate(sps):
        N = int(sp["N"])
        ip[s, :N] = sp["init_pops"]
        cp[s, :N] = sp["caps"]
        mm[s, :, :N, :N] = np.asarray(sp["mmm"], np.float32).reshape(Cn, N, N)
        cr[s, :N, :N] = crossings[s]
    hz = np.ascontiguousarray(hazard, np.float64)
    keep.append(hz)
    pr = OrAdjProblem(problem["n_paths"], problem["n_years"], S, Cn, len(problem["uncert"]) // 6,
                      NP, problem["dt"], problem["rrr"], problem["seed"], problem["road"],
                      f32(problem["uncert"]), f32(problem["flows"]), len(problem["fuel_costs"]),
                      f32(problem["fuel_costs"]), i32(problem["fuel_idx"]),
                      len(problem["ore_content"]), f32(problem["ore_content"]),
                      f32(problem["ore_sd"]), problem["unit_cost"], problem["unit_revenue"],
                      problem.get("demand_idx", -1), i32(controls),
                      i32([int(s["N"]) for s in sps]),
                      f32(np.concatenate([np.asarray(s["params"], np.float32) for s in sps])),
                      f32(ip), f32(cp), f32(mm), i32(cr), _p(hz, C.c_double))
    th = np.ascontiguousarray(theta, np.float64)
    out = np.zeros(1 + S)
    lib.or_adjoint_forward(C.byref(pr), _p(th, C.c_double), _p(out, C.c_double),
                           threads or os.cpu_count() or 1)
    return out


# ---- surrogate evaluation (oracle_interp.c, reference kernel) -----------------
def interpolate_surrogate(surrogate, predictors, R, d, mode):
    lib = oracle()
    lib.or_interpolate_surrogate.argtypes = [C.c_int, C.c_int, C.c_int, c_double_p, c_double_p,
                                             c_double_p, C.c_int, c_float_p, c_float_p]
    s = np.ascontiguousarray(surrogate, np.float64)
    p = np.ascontiguousarray(predictors, np.float64).reshape(-1, d)
    out = np.zeros(p.shape[0])
    fs = np.zeros(s.size, np.float32)
    fp = np.zeros(p.size, np.float32)
    lib.or_interpolate_surrogate(p.shape[0], d, R, _p(s, C.c_double), _p(p, C.c_double),
                                 _p(out, C.c_double), mode, _p(fs, C.c_float), _p(fp, C.c_float))
    return out


def ref_interpolate_multi(surrogate, predictors, R, d):
    lib = ref()
    lib.ref_interpolate_multi.argtypes = [C.c_int, C.c_int, C.c_int, c_float_p, c_float_p,
                                          c_float_p]
    s = np.ascontiguousarray(surrogate, np.float32)
    p = np.ascontiguousarray(predictors, np.float32).reshape(-1, d)
    out = np.zeros(p.shape[0], np.float32)
    lib.ref_interpolate_multi(p.shape[0], d, R, _p(s, C.c_float), _p(p, C.c_float),
                              _p(out, C.c_float))
    return out


# ---- GA sample selection (oracle_sample.c) ------------------------------------
def select_samples(current, candidates, n):
    lib = oracle()
    lib.or_select_samples.argtypes = [C.c_int, c_double_p, C.c_int, c_double_p, C.c_int, C.c_int,
                                      c_int_p]
    cand = np.ascontiguousarray(candidates, np.float64)
    d = cand.shape[1]
    cur = np.ascontiguousarray(current if current is not None else np.zeros((0, d)), np.float64)
    out = np.zeros(n, np.int32)
    lib.or_select_samples(cur.shape[0], _p(cur, C.c_double) if cur.size else None, cand.shape[0],
                          _p(cand, C.c_double), d, n, _p(out, C.c_int))
    return out
