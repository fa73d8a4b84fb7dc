"""Python mirror of TransportOptimiser's ``namespace SimulateGPU``
(include/gpuCode/SimulateGPU.h:34-482) over the C ABI of libtransopt.so.

The reference's entry points take Eigen matrices and shared_ptr object
graphs; these take numpy arrays with the same layouts and return the same
quantities.  Every call runs on the GPU through ``_capi``; there is no CPU
fallback.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _capi
from ._capi import Context, ptr

_default_ctx: Context | None = None


def context(device: int = 0) -> Context:
    global _default_ctx
    if _default_ctx is None:
        _default_ctx = Context(device)
    return _default_ctx


def deviceCount() -> int:
    """SimulateGPU::deviceCount (SimulateGPU.h:44)."""
    lib = _capi.load()
    n = C.c_int(0)
    lib.to_device_count(C.byref(n))
    return n.value


def labelImage(W: int, H: int, inp: np.ndarray, ctx: Context | None = None):
    """LabelImage (include/utilities/labelmethod.cpp:34) on the GPU."""
    ctx = ctx or context()
    inp = np.ascontiguousarray(inp, dtype=np.int32).reshape(-1)
    out = np.zeros(W * H, dtype=np.int32)
    n = C.c_int(0)
    ctx.check(ctx.lib.to_label_image(ctx.handle, W, H, ptr(inp, C.c_int), ptr(out, C.c_int),
                                     C.byref(n)), "to_label_image")
    return out, n.value


def buildPatches(W, H, skpx, skpy, xres, yres, noRegions, xspacing, yspacing, subPatchArea,
                 maxPop, labelledImage, populations, max_patches=None, start=0,
                 ctx: Context | None = None):
    """SimulateGPU::buildPatches (SimulateGPU.cu:3573) for one habitat type.

    Returns (patches dict of area/cap/pop/cx/cy arrays, initPop increment)."""
    ctx = ctx or context()
    cap_n = max_patches or (start + xres * yres * max(noRegions, 1))
    arrs = [np.zeros(cap_n) for _ in range(5)]
    lab = np.ascontiguousarray(labelledImage, dtype=np.int32).reshape(-1)
    pops = np.ascontiguousarray(populations, dtype=np.float64).reshape(-1)
    n = C.c_int(start)
    ip = C.c_double(0.0)
    ctx.check(ctx.lib.to_build_patches(
        ctx.handle, W, H, skpx, skpy, xres, yres, noRegions, xspacing, yspacing, subPatchArea,
        maxPop, ptr(lab, C.c_int), ptr(pops, C.c_double), cap_n,
        *[ptr(a, C.c_double) for a in arrs], C.byref(ip), C.byref(n)), "to_build_patches")
    k = n.value
    keys = ("area", "cap", "pop", "cx", "cy")
    return {kk: a[start:k].copy() for kk, a in zip(keys, arrs)}, ip.value


def lineSegmentIntersect(XY1: np.ndarray, XY2: np.ndarray, ctx: Context | None = None):
    """SimulateGPU::lineSegmentIntersect (SimulateGPU.cu:3478).  XY1 is T x 4
    and XY2 G x 4 (rows x1, y1, x2, y2); returns the crossings per row of XY1."""
    ctx = ctx or context()
    XY1 = np.asarray(XY1, dtype=np.float64)
    XY2 = np.asarray(XY2, dtype=np.float64)
    T, G = XY1.shape[0], XY2.shape[0]
    a = np.ascontiguousarray(XY1.T.reshape(-1))
    b = np.ascontiguousarray(XY2.T.reshape(-1))
    out = np.zeros(T, dtype=np.int32)
    ctx.check(ctx.lib.to_line_segment_intersect(ctx.handle, T, ptr(a, C.c_double), G,
                                                ptr(b, C.c_double), ptr(out, C.c_int)),
              "to_line_segment_intersect")
    return out


def createSpeciesModel(hab_map, pop_map, W, H, res, habitats, road_colmajor, G, hazard,
                       lambda_mean, lambda_sd=0.0, lambda_mult=0.0, hab_pref_mult=0.0,
                       sem=0, max_patches=1024, xspacing=1.0, yspacing=1.0,
                       ctx: Context | None = None):
    """SpeciesRoadPatches::createSpeciesModel (SpeciesRoadPatches.cpp:12) on
    the GPU: patches, crossings, transition / survival probabilities and the
    per-control migration matrices."""
    ctx = ctx or context()
    hab_map = np.ascontiguousarray(hab_map, dtype=np.int32).reshape(-1)
    pop_map = np.ascontiguousarray(pop_map, dtype=np.float64).reshape(-1)
    road = np.ascontiguousarray(road_colmajor, dtype=np.float64)
    hz = np.ascontiguousarray(hazard, dtype=np.float64)
    habs = (_capi.Habitat * len(habitats))(*[_capi.Habitat(h.type, h.max_pop, h.pref_mean,
                                                           h.pref_sd) for h in habitats])
    inp = _capi.SpeciesIn(W, H, res, xspacing, yspacing, len(habitats), habs,
                          ptr(hab_map, C.c_int), ptr(pop_map, C.c_double), G,
                          ptr(road, C.c_double) if G > 0 else None, lambda_mean, lambda_sd,
                          lambda_mult, hab_pref_mult, len(hz), ptr(hz, C.c_double), sem)
    NM = max_patches
    Cn = len(hz)
    b = dict(area=np.zeros(NM), cap=np.zeros(NM), pop=np.zeros(NM), cx=np.zeros(NM),
             cy=np.zeros(NM), type=np.zeros(NM, np.int32))
    big = dict(crossings=np.zeros(NM * NM, np.int32), trans=np.zeros(NM * NM),
               surv=np.zeros(Cn * NM * NM), mmm=np.zeros(Cn * NM * NM, np.float32))
    out = _capi.SpeciesOut()
    out.max_patches = NM
    for k in ("area", "cap", "pop", "cx", "cy"):
        setattr(out, k, ptr(b[k], C.c_double))
    out.type = ptr(b["type"], C.c_int)
    out.crossings = ptr(big["crossings"], C.c_int)
    out.trans = ptr(big["trans"], C.c_double)
    out.surv = ptr(big["surv"], C.c_double)
    out.mmm = ptr(big["mmm"], C.c_float)
    iar = np.zeros(Cn)
    out.iar = ptr(iar, C.c_double)
    ctx.check(ctx.lib.to_species_model(ctx.handle, C.byref(inp), C.byref(out)),
              "to_species_model")
    N = out.n_patches
    res_ = {k: v[:N].copy() for k, v in b.items()}
    res_["N"] = N
    res_["n_transitions"] = out.n_transitions
    res_["crossings"] = big["crossings"][:N * N].reshape(N, N).copy()
    res_["trans"] = big["trans"][:N * N].reshape(N, N).copy()
    res_["surv"] = big["surv"][:Cn * N * N].reshape(Cn, N, N).copy()
    res_["mmm"] = big["mmm"][:Cn * N * N].reshape(Cn, N, N).copy()
    res_["init_pops"] = res_["pop"].astype(np.float32)
    res_["caps"] = res_["cap"].astype(np.float32)
    res_["iar"] = iar
    return res_


def simulateMTECUDA(species_models, params, n_paths, n_years, dt=1.0, seed=0, road=0, sem=0,
                    migration=_capi.MIG_AUTO, control=-1, ctx: Context | None = None):
    """SimulateGPU::simulateMTECUDA (SimulateGPU.cu:3650).

    species_models: list of dicts with N, init_pops, caps, mmm (C x N x N,
    destination-major); params: list of float32[8].  Uses the highest-flow
    control's matrix as the reference does.  Returns (endPops P x S, stats)."""
    ctx = ctx or context()
    S = len(species_models)
    keep = []
    sps = (_capi.MteSpecies * S)()
    for s, m in enumerate(species_models):
        prm = np.ascontiguousarray(params[s], np.float32)
        ip = np.ascontiguousarray(m["init_pops"], np.float32)
        cp = np.ascontiguousarray(m["caps"], np.float32)
        mm = np.ascontiguousarray(m["mmm"][control], np.float32)
        keep += [prm, ip, cp, mm]
        sps[s] = _capi.MteSpecies(int(m["N"]), ptr(prm, C.c_float), ptr(ip, C.c_float),
                                  ptr(cp, C.c_float), ptr(mm, C.c_float))
    prob = _capi.MteProblem(S, n_paths, n_years, dt, seed, road, sem, migration, sps)
    end = np.zeros(S * n_paths, np.float64)
    st = (_capi.MteStats * S)()
    ctx.check(ctx.lib.to_simulate_mte(ctx.handle, C.byref(prob), ptr(end, C.c_double), st),
              "to_simulate_mte")
    stats = [dict(mean=x.mean, sd=x.sd, se=x.se, p_below=x.p_below, init_total=x.init_total)
             for x in st]
    return end.reshape(S, n_paths).T.copy(), stats


def expPV(gr, mean, time_step, rrr, current, reversion, jump_prob, noise_sd, jump_sd,
          n_paths, n_years, seed=0, road=0, sem=0, return_values=False,
          ctx: Context | None = None):
    """SimulateGPU::expPV (SimulateGPU.cu:3163): (expPV, expPVSD)."""
    ctx = ctx or context()
    prm = _capi.ExpPvParams(gr, mean, time_step, rrr, current, reversion, jump_prob,
                            noise_sd, jump_sd)
    vals = np.zeros(n_paths, np.float32)
    m, s = C.c_double(), C.c_double()
    ctx.check(ctx.lib.to_exp_pv(ctx.handle, C.byref(prm), n_paths, n_years, seed, road, sem,
                                ptr(vals, C.c_float), C.byref(m), C.byref(s)), "to_exp_pv")
    if return_values:
        return m.value, s.value, vals
    return m.value, s.value


def rov_ctypes(problem: dict, migration=_capi.MIG_AUTO):
    """to_rov_problem for a problem dict (transportoptimiser_gb300.rov);
    returns (struct, arrays that must stay alive while it is used)."""
    S = len(problem["species"])
    P, Y, R = problem["n_paths"], problem["n_years"], problem["dim_res"]
    Cn = len(problem["flows"])
    keep = []
    sps = (_capi.RovSpecies * S)()
    for s, sp in enumerate(problem["species"]):
        arrs = [np.ascontiguousarray(sp[k], np.float32) for k in ("params", "init_pops", "caps", "mmm")]
        keep += arrs
        sps[s] = _capi.RovSpecies(int(sp["N"]), *[ptr(a_, C.c_float) for a_ in arrs])
    keep.append(sps)
    f32 = lambda k: np.ascontiguousarray(problem[k], np.float32)
    flows, unc, fc, oc, osd = (f32(k) for k in ("flows", "uncert", "fuel_costs", "ore_content",
                                                  "ore_sd"))
    fi = np.ascontiguousarray(problem["fuel_idx"], np.int32)
    keep += [flows, unc, fc, oc, osd, fi]
    pr = _capi.RovProblem(S, P, Y, Cn, R, sps, ptr(flows, C.c_float), len(unc) // 6,
                          ptr(unc, C.c_float), len(fc), ptr(fc, C.c_float), ptr(fi, C.c_int),
                          len(oc), ptr(oc, C.c_float), ptr(osd, C.c_float),
                          problem["unit_cost"], problem["unit_revenue"], problem["dt"],
                          problem["rrr"], problem.get("demand_idx", -1), problem["seed"],
                          problem["road"], problem["sem"], migration,
                          int(problem.get("algo", 4)))
    return pr, keep


def simulateROVCUDA(problem: dict, want=("cond_exp", "opt_cont", "unit_profits", "adj_pops",
                                        "regression"), migration=_capi.MIG_AUTO,
                    ctx: Context | None = None) -> dict:
    """SimulateGPU::simulateROVCUDA, ALGO4 (SimulateGPU.cu:3870-5003).

    ``problem`` follows transportoptimiser_gb300.rov.  Returns condExp,
    optCont, unitProfits ([Y][P]), adjPops ([Y][S][P]), the regression
    surfaces and the stats (value, control, sd) plus the Monte Carlo SE."""
    ctx = ctx or context()
    S = len(problem["species"])
    P, Y, R = problem["n_paths"], problem["n_years"], problem["dim_res"]
    Cn = len(problem["flows"])
    pr, keep = rov_ctypes(problem, migration)
    d = S + 1
    out = {}
    if "cond_exp" in want: out["cond_exp"] = np.zeros(Y * P)
    if "opt_cont" in want: out["opt_cont"] = np.zeros(Y * P, np.int32)
    if "unit_profits" in want: out["unit_profits"] = np.zeros(Y * P)
    if "adj_pops" in want: out["adj_pops"] = np.zeros(Y * S * P)
    if "regression" in want: out["regression"] = np.zeros(Y * Cn * (R * d + 2 * R ** d))
    r = _capi.RovResult()
    r.cond_exp = ptr(out.get("cond_exp"), C.c_double)
    r.opt_cont = ptr(out.get("opt_cont"), C.c_int)
    r.unit_profits = ptr(out.get("unit_profits"), C.c_double)
    r.adj_pops = ptr(out.get("adj_pops"), C.c_double)
    r.regression = ptr(out.get("regression"), C.c_double)
    ctx.check(ctx.lib.to_simulate_rov(ctx.handle, C.byref(pr), C.byref(r)), "to_simulate_rov")
    out["stats"] = np.array([r.value, r.control, r.sd])
    out["value_se"] = r.se
    out["n_best"] = r.n_best
    return out


def simulateROVCUDA_batch(problems, want=("cond_exp", "opt_cont", "regression"),
                          migration=_capi.MIG_AUTO, ctx: Context | None = None) -> list:
    """Several roads valued in one batch (to_simulate_rov_batch): problems
    with the same dimensions, processes, costs, seed and species parameters,
    each with its own species models and road id.  Returns one dict per road,
    as simulateROVCUDA does."""
    ctx = ctx or context()
    n = len(problems)
    prs = (_capi.RovProblem * n)()
    ress = (_capi.RovResult * n)()
    keep, outs = [], []
    for i, problem in enumerate(problems):
        S = len(problem["species"])
        P, Y, R = problem["n_paths"], problem["n_years"], problem["dim_res"]
        Cn = len(problem["flows"])
        pr, k = rov_ctypes(problem, migration)
        keep.append(k)
        prs[i] = pr
        d = S + 1
        out = {}
        if "cond_exp" in want: out["cond_exp"] = np.zeros(Y * P)
        if "opt_cont" in want: out["opt_cont"] = np.zeros(Y * P, np.int32)
        if "unit_profits" in want: out["unit_profits"] = np.zeros(Y * P)
        if "adj_pops" in want: out["adj_pops"] = np.zeros(Y * S * P)
        if "regression" in want: out["regression"] = np.zeros(Y * Cn * (R * d + 2 * R ** d))
        r = ress[i]
        r.cond_exp = ptr(out.get("cond_exp"), C.c_double)
        r.opt_cont = ptr(out.get("opt_cont"), C.c_int)
        r.unit_profits = ptr(out.get("unit_profits"), C.c_double)
        r.adj_pops = ptr(out.get("adj_pops"), C.c_double)
        r.regression = ptr(out.get("regression"), C.c_double)
        outs.append(out)
    ctx.check(ctx.lib.to_simulate_rov_batch(ctx.handle, n, prs, ress), "to_simulate_rov_batch")
    for i, out in enumerate(outs):
        r = ress[i]
        out["stats"] = np.array([r.value, r.control, r.sd])
        out["value_se"] = r.se
        out["n_best"] = r.n_best
    return outs


def knn(ref_pts: np.ndarray, query: np.ndarray, k: int, ctx: Context | None = None):
    """knn_cuda_with_indexes::knn: ref (dim x n), query (dim x Q), dim-major.
    Returns dist, ind (k x Q, ind 1-based)."""
    ctx = ctx or context()
    ref_pts = np.ascontiguousarray(ref_pts, np.float32)
    query = np.ascontiguousarray(query, np.float32)
    dim, n = ref_pts.shape
    Q = query.shape[1]
    dist = np.zeros(k * Q, np.float32)
    ind = np.zeros(k * Q, np.int32)
    ctx.check(ctx.lib.to_knn(ctx.handle, ptr(ref_pts, C.c_float), n, ptr(query, C.c_float), Q,
                             dim, k, ptr(dist, C.c_float), ptr(ind, C.c_int)), "to_knn")
    return dist.reshape(k, Q), ind.reshape(k, Q)


def buildSurrogateMTECUDA(iars, pops_mean, pops_sd, dim_res, ctx: Context | None = None):
    """SimulateGPU::buildSurrogateMTECUDA (SimulateGPU.cu:5533) for one
    species: returns the (mean, sd) surrogate vectors [R x | R y]."""
    ctx = ctx or context()
    x = np.ascontiguousarray(iars, np.float64)
    m = np.ascontiguousarray(pops_mean, np.float64)
    sd = np.ascontiguousarray(pops_sd, np.float64)
    om, osd = np.zeros(2 * dim_res), np.zeros(2 * dim_res)
    ctx.check(ctx.lib.to_build_surrogate_mte(ctx.handle, len(x), ptr(x, C.c_double),
                                             ptr(m, C.c_double), ptr(sd, C.c_double), dim_res,
                                             ptr(om, C.c_double), ptr(osd, C.c_double)),
              "to_build_surrogate_mte")
    return om, osd


def interpolateSurrogateMulti(surrogate, predictors, dim_res, n_dims, mode=0,
                              ctx: Context | None = None):
    """SimulateGPU::interpolateSurrogateMulti (SimulateGPU.cu:5919) batched:
    predictors [n][n_dims].  mode 0 the reference kernel's float arithmetic,
    1 multilinear in double, 2 Utility::interpolateSurrogate (Utility.cpp:253)."""
    ctx = ctx or context()
    s = np.ascontiguousarray(surrogate, np.float64)
    p = np.ascontiguousarray(predictors, np.float64).reshape(-1, n_dims)
    out = np.zeros(p.shape[0])
    ctx.check(ctx.lib.to_interpolate_surrogate(ctx.handle, p.shape[0], n_dims, dim_res,
                                               ptr(s, C.c_double), ptr(p, C.c_double),
                                               ptr(out, C.c_double), mode),
              "to_interpolate_surrogate")
    return out


def generateSample(current, candidates, n, ctx: Context | None = None) -> np.ndarray:
    """RoadGA::generateSample (RoadGA.cpp:3288) on the device: indices of n
    candidates chosen by the reference's max-min rule."""
    ctx = ctx or context()
    cand = np.ascontiguousarray(candidates, np.float64)
    d = cand.shape[1]
    cur = np.ascontiguousarray(current if current is not None else np.zeros((0, d)), np.float64)
    out = np.zeros(n, np.int32)
    ctx.check(ctx.lib.to_select_samples(ctx.handle, cur.shape[0], ptr(cur, C.c_double) if cur.size else None,
                                        cand.shape[0], ptr(cand, C.c_double), d, n,
                                        ptr(out, C.c_int)), "to_select_samples")
    return out


def buildSurrogateROVCUDA(predictors, values, values_sd, dim_res, sem=0,
                          ctx: Context | None = None):
    """SimulateGPU::buildSurrogateROVCUDA (SimulateGPU.cu:5694): predictors
    d x n (IARs, unit use).  Returns the (mean, sd) surrogate vectors."""
    ctx = ctx or context()
    pr = np.ascontiguousarray(predictors, np.float64)
    d, n = pr.shape
    v = np.ascontiguousarray(values, np.float64)
    vs = np.ascontiguousarray(values_sd, np.float64)
    size = dim_res * d + dim_res ** d
    om, osd = np.zeros(size), np.zeros(size)
    ctx.check(ctx.lib.to_build_surrogate_rov(ctx.handle, n, d, ptr(pr, C.c_double),
                                             ptr(v, C.c_double), ptr(vs, C.c_double), dim_res,
                                             sem, ptr(om, C.c_double), ptr(osd, C.c_double)),
              "to_build_surrogate_rov")
    return om, osd
