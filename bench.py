#!/usr/bin/env python3
"""Road designs valued per second at +-1% Monte Carlo standard error.

Workload (the batched GA generation): 256 roads (8-64 control points, 20-400
patch crossings) on a 200 x 200 habitat grid with 5 habitat types (200-345
patches per species model) and 3 species, 50 yearly steps (synthetic,
seeded).  A "step" values
every road of the generation in both of the reference's modes: the
species-road model (patches, crossings, transition and survival matrices,
initial animals at risk), the MTE population Monte Carlo at N*_mte paths and
the ROV real-options valuation (ALGO4, 3 controls, 3 exogenous processes,
regressions on 8 bins per state dimension) at N*_rov paths, all in one
captured CUDA graph.  N* = ceil((sigma / (0.01 * mu))^2) per road comes from
untimed pilots at the configuration's 2000 MTE and 5000 ROV paths (the
largest over roads is used for the batch).

    value  - batched path, road inputs already resident in HBM
    e2e    - same through the public C ABI with pinned host inputs, H2D and
             D2H inside the timed region
    plain  - the reference-style path: one road per call through the host
             entry points (species models, simulate MTE, simulate ROV), with
             the habitat maps rasterised beforehand, and its GPU-kernel share
    --impl reference - the CPU restatement of the reference (oracle/) on all
             host cores, one road per core, bounded sample of the same work
             at the same N* (SCENE_N_STAR)

One JSON line on stdout (rank 0).
"""
from __future__ import annotations

import argparse
import concurrent.futures as cf
import json
import math
import os
import statistics
import subprocess
import sys
import time
from pathlib import Path

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "road designs valued/sec at ±1% MC error: batched/surrogate vs plain, 1 GB300"
WORKLOAD = ("GA generation: 256 roads (8-64 control points), 200x200 grid, 5 habitat types, "
            "~300 patches, 3 species, each road valued by MTE and ROV at N* paths "
            "(pilots 2000 MTE / 5000 ROV paths), 50 years")
N_ROADS = 256
PILOT_PATHS = 2000
ROV_PILOT_PATHS = 5000
ROV_DIM_RES = 8
ROV_SEED = 17
SEM = 1
REF_SECONDS = 90          # the reference arm's sample window
# N* of the bench scene (synth.generation(0), 256 roads): the largest per-road
# N* of the 2000-path MTE and 5000-path ROV pilots, as this arm's pilots
# compute it on the GPU.  The reference arm values the same workload at these
# path counts (its CPU cannot run the pilots of all 256 roads in its window).
SCENE_N_STAR = (64, 768)
YEARS = 50


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--roads", type=int, default=N_ROADS)
    ap.add_argument("--plain-roads", type=int, default=8)
    ap.add_argument("--rov-dim-res", type=int, default=ROV_DIM_RES)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--profile-only", action="store_true",
                    help="pilots + one step, for profiler launch lists")
    ap.add_argument("--profile-mte-only", action="store_true",
                    help="pilot + one MTE-only generation step, for profilers")
    ap.add_argument("--profile-rov", action="store_true",
                    help="one ROV valuation of a one-road scene (2 species, ~115 "
                         "patches, 3 controls, 16 bins per dimension), for profilers")
    ap.add_argument("--profile-rov-batch", type=int, default=0, metavar="PATHS",
                    help="one batched ROV valuation of 256 roads at PATHS paths each, for "
                         "profilers")
    ap.add_argument("--rov-paths", type=int, default=10000)
    ap.add_argument("--surrogate-samples", type=int, default=50000,
                    help="training pairs for the learned surrogate (0: skip that leg)")
    ap.add_argument("--ga-generations", type=int, default=64)
    ap.add_argument("--no-rov-leg", dest="rov_leg", action="store_false",
                    help="skip the one-road ROV, batched-ROV and adjoint timings")
    return ap.parse_args()


# --------------------------------------------------------------------------
def clocks_start():
    try:
        f = open("/tmp/to_bench_clocks.csv", "w")
        p = subprocess.Popen(
            ["nvidia-smi", "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,"
             "clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap", "--format=csv,noheader,nounits", "-lms", "200"],
            stdout=f, stderr=subprocess.DEVNULL)
        return p, f
    except Exception:
        return None, None


def clocks_stop(h, device_index=0):
    p, f = h
    if p is None:
        return None
    p.terminate()
    try:
        p.wait(timeout=5)
    except Exception:
        p.kill()
    f.close()
    sm, mx, reasons = [], None, set()
    names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
    for line in open("/tmp/to_bench_clocks.csv"):
        parts = [x.strip() for x in line.split(",")]
        if len(parts) < 9 or parts[0] != str(device_index):
            continue
        try:
            sm.append(float(parts[1]))
            mx = float(parts[2])
        except ValueError:
            continue
        for n, v in zip(names, parts[5:9]):
            if v.lower() == "active":
                reasons.add(n)
    if not sm:
        return None
    return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons),
            "samples": len(sm)}


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return d.get("bf16_tflops", 1900.0), d.get("hbm_gbs", 6800.0), "measured"
    return 1900.0, 6800.0, "fallback"


# --------------------------------------------------------------------------
def n_star(results, floor=64):
    """Paths needed per road for a 1% relative standard error of the MTE end
    population (max over species), from a pilot at PILOT_PATHS."""
    need = []
    for r in range(results.shape[0]):
        nr = 0
        for s in range(results.shape[1]):
            mean, se = results[r, s, 2], results[r, s, 4]
            sigma = se * math.sqrt(PILOT_PATHS)
            if mean > 0:
                nr = max(nr, math.ceil((sigma / (0.01 * abs(mean))) ** 2))
        need.append(max(floor, nr))
    return need


def rov_n_star(results, pilot, floor=128):
    """Paths needed per road for a 1% relative standard error of the ROV
    value (result slots 10 and 13), from a pilot at `pilot` paths."""
    need = []
    for r in range(results.shape[0]):
        v, se = results[r, 0, 10], results[r, 0, 13]
        n = floor
        if v != 0.0 and math.isfinite(v) and math.isfinite(se):
            n = max(floor, math.ceil((se * math.sqrt(pilot) / (0.01 * abs(v))) ** 2))
        need.append(n)
    return need


def rov_template(models, scene, P, dim_res, road=0):
    from transportoptimiser_gb300.rov import rov_problem_from_models
    return rov_problem_from_models(models, scene, n_paths=P, n_years=YEARS, dim_res=dim_res,
                                   sem=1, n_processes=3, demand=True, seed=ROV_SEED, road=road)


def oracle_road(scene, r, rd, hab, P_mte, P_rov, dim_res, road0=0):
    """The reference's work for one road on one core (oracle/): the species
    model of every species, the MTE at P_mte paths and the ROV at P_rov."""
    from oracle import pyoracle as po
    models = []
    for s, sp in enumerate(scene.species):
        m = po.species_model(scene, sp, rd, sem=SEM, max_patches=1024, hab=hab)
        models.append(m)
        po.simulate_mte(P_mte, YEARS, m["N"], 1.0, sp.params, m["init_pops"], m["caps"],
                        m["mmm"][-1], 0, road0 + r, s, SEM, 1)
    if P_rov > 0:
        po.simulate_rov(rov_template(models, scene, P_rov, dim_res, road=road0 + r), threads=1)
    return r


def oracle_generation(scene, habs, P_mte, P_rov, dim_res, seconds, threads=None, start=0):
    """Roads valued by the oracle in parallel, one road per host core (the
    oracle's ctypes calls release the GIL), for about `seconds`; returns
    (designs/s, threads, roads)."""
    threads = threads or os.cpu_count() or 1
    R = len(scene.roads)
    t0 = time.perf_counter()
    done = 0
    nxt = start
    with cf.ThreadPoolExecutor(max_workers=threads) as ex:
        running = set()
        while True:
            while len(running) < threads and time.perf_counter() - t0 < seconds:
                r = nxt % R
                nxt += 1
                running.add(ex.submit(oracle_road, scene, r, scene.roads[r], habs[r], P_mte,
                                      P_rov, dim_res))
            if not running:
                break
            fin, running = cf.wait(running, return_when=cf.FIRST_COMPLETED)
            for f in fin:
                f.result()
                done += 1
    dt = time.perf_counter() - t0
    return done / dt, threads, done


def reference_n_star(scene, habs, roads, dim_res, threads=None):
    """N* by the GPU arm's rule from CPU pilots (MTE at PILOT_PATHS, ROV at
    a quarter of ROV_PILOT_PATHS to bound the time) on the given roads."""
    import numpy as np
    from oracle import pyoracle as po
    threads = threads or os.cpu_count() or 1
    need_m, need_r = 64, 128
    rp = ROV_PILOT_PATHS // 4
    for r in roads:
        rd = scene.roads[r]
        models = []
        for s, sp in enumerate(scene.species):
            m = po.species_model(scene, sp, rd, sem=SEM, max_patches=1024, hab=habs[r])
            models.append(m)
            e = po.simulate_mte(PILOT_PATHS, YEARS, m["N"], 1.0, sp.params, m["init_pops"],
                                m["caps"], m["mmm"][-1], 1, r, s, SEM, threads).astype(np.float64)
            if e.mean() > 0:
                need_m = max(need_m, math.ceil((e.std(ddof=1) / (0.01 * e.mean())) ** 2))
        o = po.simulate_rov(rov_template(models, scene, rp, dim_res, road=r), threads=threads)
        v = o["stats"][0]
        if v != 0.0:
            need_r = max(need_r, math.ceil((o["value_se"] * math.sqrt(rp) / (0.01 * abs(v))) ** 2))
    P_mte = int(min(math.ceil(need_m / 64.0) * 64, 16384))
    P_rov = int(min(math.ceil(need_r / 128.0) * 128, 16384))
    return P_mte, P_rov


# --------------------------------------------------------------------------
def run_reference(args):
    """--impl reference: the CPU port of the reference on the host cores,
    one road per core.  A road takes seconds on one core, so the K steps
    share one continuous sample: the pool values roads for REF_SECONDS (then
    finishes the roads in flight) and the line reports designs per second
    over that whole window."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return 0
    from transportoptimiser_gb300 import synth
    from transportoptimiser_gb300 import build as b
    b.build_oracle()
    scene = synth.generation(0, n_roads=args.roads)
    habs = [scene.hab_map(rd) for rd in scene.roads]       # rasterised outside the timing
    if args.roads == N_ROADS:
        P_mte, P_rov = SCENE_N_STAR
        nstar = "N* of the GPU arm's pilots for this scene (SCENE_N_STAR)"
    else:
        P_mte, P_rov = reference_n_star(scene, habs, [0, 1], args.rov_dim_res)
        nstar = ("N* from CPU pilots (MTE %d paths, ROV %d paths) on 2 roads"
                 % (PILOT_PATHS, ROV_PILOT_PATHS // 4))
    for _ in range(args.warmup):
        oracle_road(scene, 0, scene.roads[0], habs[0], 64, 0, args.rov_dim_res)
    value, cores, n = oracle_generation(scene, habs, P_mte, P_rov, args.rov_dim_res,
                                        seconds=REF_SECONDS)
    sample = ("%d roads valued by a pool of %d workers, one road per core, over %d s (the "
              "roads in flight then finished); each road: 3 species models, MTE at %d paths, "
              "ROV at %d paths (%d bins per state dimension), 50 years"
              % (n, cores, REF_SECONDS, P_mte, P_rov, args.rov_dim_res))
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": "designs/s",
            "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": 1000.0 / value, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f32", "data": "synthetic",
            "config": {"workload": WORKLOAD, "roads": args.roads,
                       "species": len(scene.species),
                       "mte_paths_per_road": P_mte, "rov_paths_per_road": P_rov,
                       "pilot_paths": {"mte": PILOT_PATHS, "rov": ROV_PILOT_PATHS},
                       "years": YEARS, "rov_bins_per_dim": args.rov_dim_res,
                       "semantics": "corrected",
                       "note": "the steps share one continuous sample; " + nstar},
            "cpu_baseline": {"value": value, "unit": "designs/s", "cores": cores,
                             "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "designs/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)
    return 0


# --------------------------------------------------------------------------
def surrogate_leg(args, gen, scene, P, ctx):
    """Learned surrogate: an ensemble of two MLPs (own BF16 tensor-core
    kernels) trained on pairs the batched simulator generates, then a GA of
    args.ga_generations x 256 roads valued with screening (Monte Carlo on
    designs whose members disagree by > 1% and on the top 10%) against the
    same GA valued by Monte Carlo throughout."""
    import numpy as np
    from transportoptimiser_gb300 import surrogate_ga as sga
    t0 = time.perf_counter()
    X, Y = sga.generate_dataset(gen, scene, args.surrogate_samples, paths=128,
                                rng=np.random.default_rng(101), seed=77)
    t_data = time.perf_counter() - t0
    t0 = time.perf_counter()
    ens = sga.Ensemble(2).fit(X, Y, epochs=60, batch=512, lr=2e-3, ctx=ctx)
    t_fit = time.perf_counter() - t0
    Xt, Yt = sga.generate_dataset(gen, scene, 1024, paths=1024, rng=np.random.default_rng(202),
                                  seed=88)
    pred, _ = ens.predict(Xt, ctx)
    err = np.abs(pred[:, 0] - Yt[:, 0]) / Yt[:, 0]
    opts = gen.opts(P, YEARS, seed=5, sem=SEM)
    pop = args.roads
    out = {}
    # config 4's own rule (Monte Carlo where the predicted error is above 1%,
    # and on the top 10%), then wider tolerances, then Monte Carlo throughout
    for name, e, tol, top in (("rule_1pct_top10", ens, 0.01, 0.10),
                              ("screened_tol10", ens, 0.10, 0.25),
                              ("screened_tol20", ens, 0.20, 0.25),
                              ("plain_mc", None, 0.0, 0.25)):
        tm = {}
        _, best, n_mc, secs = sga.run_ga(gen, scene, args.ga_generations, pop, opts,
                                         np.random.default_rng(7), e, tol, top=top, timings=tm)
        designs = args.ga_generations * pop
        out[name] = {"designs_per_s": designs / secs, "mc_valuations": n_mc,
                     "designs": designs, "best_fitness_mc": best, "seconds": secs,
                     "valuation_s": tm["valuation_s"], "ga_operators_s": tm["ga_ops_s"],
                     "valuation_designs_per_s": designs / tm["valuation_s"]}
    return {"model": "MLP 16-128-128-3, ensemble of 2, BF16 tcgen05 GEMMs",
            "train_pairs": int(len(X)), "train_paths": 128, "data_s": t_data, "fit_s": t_fit,
            "final_loss": float(ens.members[0].loss_curve[-1]),
            "heldout_median_rel_err_mean_end_ratio": float(np.median(err)),
            "ga": out, "ga_generations": args.ga_generations, "ga_population": pop,
            "screen_rule": "MC on the top fraction (10% for rule_1pct_top10, else 25%) by "
                           "predicted fitness plus the members' spread, and where the members "
                           "disagree by > tol (1%, 10%, 20%)",
            "features": list(sga.FEATURES),
            "designs_per_s_ratio_rule_1pct_vs_mc":
                out["rule_1pct_top10"]["designs_per_s"] / out["plain_mc"]["designs_per_s"],
            "designs_per_s_ratio_screened_tol10_vs_mc":
                out["screened_tol10"]["designs_per_s"] / out["plain_mc"]["designs_per_s"],
            "designs_per_s_ratio_screened_tol20_vs_mc":
                out["screened_tol20"]["designs_per_s"] / out["plain_mc"]["designs_per_s"],
            "valuation_ratio_screened_tol10_vs_mc":
                out["screened_tol10"]["valuation_designs_per_s"] /
                out["plain_mc"]["valuation_designs_per_s"],
            "valuation_ratio_screened_tol20_vs_mc":
                out["screened_tol20"]["valuation_designs_per_s"] /
                out["plain_mc"]["valuation_designs_per_s"],
            "note": "designs_per_s includes the host-side GA operators (Python), "
                    "valuation_designs_per_s only the valuation of each generation"}


def rov_adjoint_leg(ctx, rov_paths=10000, adj_paths=20000, reps=3):
    """One-road ROV (2 species, ~115 patches, 3 controls, 3 exogenous
    processes, 16 bins per dimension, 50 years) timed through the public
    entry point, then the adjoint of its frozen optimal policy (13
    parameters) at adj_paths paths: forward and one backward per output."""
    import numpy as np
    from transportoptimiser_gb300 import synth
    from transportoptimiser_gb300 import simulate_gpu as sg
    from transportoptimiser_gb300.rov import rov_problem_from_models
    from transportoptimiser_gb300.adjoint import FrozenPolicy, theta_from_problem
    sc = synth.rov_road(0, n_species=2)
    models = []
    for s in range(2):
        sp = sc.species[s]
        hab = sc.hab_map(sc.roads[0])
        models.append(sg.createSpeciesModel(hab, sc.pop_map(sp, hab), sc.W, sc.H, sc.res,
                                            sp.habitats, sc.roads[0].colmajor(), sc.roads[0].G,
                                            sp.hazard, sp.lambda_mean, sem=1, max_patches=512,
                                            ctx=ctx))
    rp = rov_problem_from_models(models, sc, n_paths=rov_paths, n_years=YEARS, dim_res=16,
                                 sem=1, n_processes=3, demand=True)
    out = sg.simulateROVCUDA(rp, want=(), ctx=ctx)
    ts = []
    for _ in range(reps):
        t0 = time.perf_counter()
        out = sg.simulateROVCUDA(rp, want=(), ctx=ctx)
        ts.append(time.perf_counter() - t0)
    rov = {"paths": rov_paths, "ms_per_valuation": 1000.0 * statistics.median(ts),
           "value": float(out["stats"][0]), "se": float(out["value_se"]),
           "patches": [int(m["N"]) for m in models]}
    # ALGO6: each year's value from paths re-simulated under the optimal policy
    r6 = rov_problem_from_models(models, sc, n_paths=rov_paths, n_years=YEARS, dim_res=16,
                                 sem=1, n_processes=3, demand=True, algo=6)
    out6 = sg.simulateROVCUDA(r6, want=(), ctx=ctx)
    ts6 = []
    for _ in range(reps):
        t0 = time.perf_counter()
        out6 = sg.simulateROVCUDA(r6, want=(), ctx=ctx)
        ts6.append(time.perf_counter() - t0)
    rov["algo6_ms_per_valuation"] = 1000.0 * statistics.median(ts6)
    rov["algo6_value"] = float(out6["stats"][0])
    rov["algo6_se"] = float(out6["value_se"])
    ra = rov_problem_from_models(models, sc, n_paths=adj_paths, n_years=YEARS, dim_res=16,
                                 sem=1, n_processes=3, demand=True)
    pol = sg.simulateROVCUDA(ra, want=("opt_cont",), ctx=ctx)
    ctl = pol["opt_cont"].reshape(YEARS, adj_paths).astype(np.int32)
    hz = np.asarray(sc.species[0].hazard, np.float64)
    fp = FrozenPolicy(ra, ctl, [m["crossings"] for m in models], hz, ctx)
    th = theta_from_problem(ra, hz)
    o, tape = fp.forward(th)
    fp.free(tape)
    t0 = time.perf_counter()
    o, tape = fp.forward(th)
    t_fwd = time.perf_counter() - t0
    t0 = time.perf_counter()
    J = [fp.backward(tape, np.eye(3)[i]) for i in range(3)]
    t_bwd = (time.perf_counter() - t0) / 3
    fp.free(tape)
    adj = {"paths": adj_paths, "parameters": int(th.size), "forward_ms": 1000.0 * t_fwd,
           "backward_ms_per_output": 1000.0 * t_bwd, "outputs": [float(x) for x in o],
           "dPV_dtheta_fuel": float(J[0][0]), "checkpoint_years": 10}
    return {"rov": rov, "adjoint": adj}


def rov_generation_leg(ctx, n_roads=256, reps=3, plain_roads=16, paths=None):
    """ROV valuation of a GA generation of roads in one batch
    (to_simulate_rov_batch) at N* paths per road from a 512-path pilot, next
    to one road per call (the reference's way)."""
    import numpy as np
    from transportoptimiser_gb300 import synth
    from transportoptimiser_gb300 import simulate_gpu as sg
    from transportoptimiser_gb300.rov import rov_problem_from_models
    sc = synth.rov_road(0, n_species=2)
    rng = np.random.Generator(np.random.Philox(11))
    roads = [sc.roads[0]] + [synth.random_road(sc.W, sc.H, int(rng.integers(8, 65)), rng)
                             for _ in range(n_roads - 1)]
    models = []
    for rd in roads:
        hab = sc.hab_map(rd)
        models.append([sg.createSpeciesModel(hab, sc.pop_map(sp, hab), sc.W, sc.H, sc.res,
                                             sp.habitats, rd.colmajor(), rd.G, sp.hazard,
                                             sp.lambda_mean, sem=1, max_patches=512, ctx=ctx)
                       for sp in sc.species])

    def problems(P):
        return [rov_problem_from_models(m, sc, n_paths=P, n_years=YEARS, dim_res=16, sem=1,
                                        n_processes=3, demand=True, road=i)
                for i, m in enumerate(models)]
    if paths is None:
        pilot = sg.simulateROVCUDA_batch(problems(512), want=(), ctx=ctx)
        need = max((o["value_se"] * math.sqrt(512) / (0.01 * abs(o["stats"][0]))) ** 2
                   for o in pilot if o["stats"][0] != 0.0)
        P = int(min(max(128, math.ceil(need / 128.0) * 128), 4096))
    else:
        P = paths
    probs = problems(P)
    sg.simulateROVCUDA_batch(probs, want=(), ctx=ctx)
    if reps == 0:
        return {"roads": n_roads, "paths_per_road": P}
    ts = []
    for _ in range(reps):
        t0 = time.perf_counter()
        sg.simulateROVCUDA_batch(probs, want=(), ctx=ctx)
        ts.append(time.perf_counter() - t0)
    tb = statistics.median(ts)
    t0 = time.perf_counter()
    for p in probs[:plain_roads]:
        sg.simulateROVCUDA(p, want=(), ctx=ctx)
    t1 = (time.perf_counter() - t0) / max(plain_roads, 1)
    return {"roads": n_roads, "paths_per_road": P, "pilot_paths": 512, "years": YEARS,
            "batch_ms": 1000.0 * tb, "designs_per_s": n_roads / tb,
            "plain_ms_per_road": 1000.0 * t1, "plain_designs_per_s": 1.0 / t1,
            "note": "2 species, 3 controls, 16^3 regression grid; batch = to_simulate_rov_batch"}


def profile_rov(args):
    """One ROV valuation (ALGO4) of a 128 x 128 one-road scene with 2 species on the GPU."""
    from transportoptimiser_gb300 import synth
    from transportoptimiser_gb300 import simulate_gpu as sg
    from transportoptimiser_gb300.rov import rov_problem_from_models
    sc = synth.rov_road(0, n_species=2)
    models = []
    for s in range(2):
        sp = sc.species[s]
        hab = sc.hab_map(sc.roads[0])
        models.append(sg.createSpeciesModel(hab, sc.pop_map(sp, hab), sc.W, sc.H, sc.res,
                                            sp.habitats, sc.roads[0].colmajor(), sc.roads[0].G,
                                            sp.hazard, sp.lambda_mean, sem=1, max_patches=512))
    rp = rov_problem_from_models(models, sc, n_paths=args.rov_paths, n_years=YEARS, dim_res=16,
                                 sem=1, n_processes=3, demand=True)
    out = sg.simulateROVCUDA(rp, want=())
    print(json.dumps({"rov_value": out["stats"][0], "se": out["value_se"]}))
    return 0


def kernel_split(ctx, names):
    """{name: (ms per launch, launches)} from the context's event timing."""
    out = {}
    for n in names:
        ms, k = ctx.kernel_time(n)
        if k:
            out[n] = (ms, k)
    return out


def main():
    args = parse()
    if args.impl == "reference":
        return run_reference(args)
    if args.profile_rov:
        return profile_rov(args)
    if args.profile_rov_batch:
        from transportoptimiser_gb300._capi import Context
        print(json.dumps(rov_generation_leg(Context(0), reps=0, plain_roads=0,
                                            paths=args.profile_rov_batch)))
        return 0

    import numpy as np
    import torch

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)

    from transportoptimiser_gb300 import synth
    from transportoptimiser_gb300._capi import MIG_AUTO, MIG_SPARSE_FP32, RESULT_STRIDE, Context
    from transportoptimiser_gb300.generation import Generation, pack_roads
    from transportoptimiser_gb300 import simulate_gpu as sg
    from transportoptimiser_gb300 import shard

    scene = synth.generation(0, n_roads=args.roads)
    if rank > 0:
        # each rank values its own generation of roads (weak scaling)
        scene.roads = shard.rank_roads(scene, args.roads, rank)
    S = len(scene.species)
    ctx = Context(local)
    stream = torch.cuda.Stream()
    ctx.set_stream(stream.cuda_stream)
    gen = Generation(scene, max_roads=args.roads, max_patches=512, ctx=ctx)
    packed = pack_roads(scene, scene.roads)
    road0 = shard.road0(rank)
    R_dim = args.rov_dim_res

    # pilots (untimed): N* per road for the MTE (2000 paths) and the ROV (5000)
    pilot = gen.evaluate(packed, gen.opts(PILOT_PATHS, YEARS, seed=1, road0=road0, sem=SEM,
                                          migration=MIG_SPARSE_FP32))
    P = min(int(math.ceil(max(n_star(pilot)) / 64.0) * 64), 16384)
    Ns = pilot[:, :, 0].astype(int)
    if args.profile_mte_only:
        o = gen.opts(P, YEARS, seed=0, road0=road0, sem=SEM, migration=MIG_SPARSE_FP32)
        gen.evaluate(packed, o)
        gen.evaluate(packed, o)
        return 0
    tmpl_models = [gen.species_model(0, s) for s in range(S)]
    gen.set_rov(rov_template(tmpl_models, scene, ROV_PILOT_PATHS, R_dim))
    rpilot = gen.evaluate(packed, gen.opts(64, YEARS, seed=1, road0=road0, sem=SEM))
    P_rov = min(int(math.ceil(max(rov_n_star(rpilot, ROV_PILOT_PATHS)) / 128.0) * 128), 16384)
    gen.set_rov(rov_template(tmpl_models, scene, P_rov, R_dim))
    # the whole generation is captured once as a CUDA graph and replayed
    opts = gen.opts(P, YEARS, seed=0, road0=road0, sem=SEM, migration=MIG_AUTO, graph=True)

    dev = {k: torch.from_numpy(v).cuda() for k, v in packed.items()}
    d_res = torch.zeros(args.roads * S * RESULT_STRIDE, dtype=torch.float64, device="cuda")
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def step_device(o=opts):
        gen.evaluate_device(args.roads, dev["cell_off"].data_ptr(), dev["cells"].data_ptr(),
                            dev["seg_off"].data_ptr(), dev["segs"].data_ptr(), o,
                            d_res.data_ptr())

    def timed(fn, steps):
        evs = []
        for _ in range(steps):
            flush.zero_()
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            evs.append((e0, e1))
        torch.cuda.synchronize()
        return [a.elapsed_time(b) for a, b in evs]

    with torch.cuda.stream(stream):
        for _ in range(args.warmup):
            step_device()
            flush.zero_()
        torch.cuda.synchronize()
        if args.profile_only:
            step_device()
            torch.cuda.synchronize()
            r = d_res.cpu().numpy().reshape(args.roads, S, RESULT_STRIDE)
            C = len(scene.flows)
            print(json.dumps({"profile_step": {
                "roads": args.roads, "rov_paths": P_rov, "mte_paths": P, "species": S,
                "years": YEARS, "fitted_queries": float(r[:, 0, 15].sum()) * (YEARS - 2) * C *
                R_dim ** (S + 1),
                "forward_units": args.roads * math.ceil(P_rov / 32) * S * YEARS}}), flush=True)
            return 0
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        clk = clocks_start()
        l0 = ctx.launches
        t_wall0 = time.perf_counter()
        step_ms = timed(step_device, args.steps)
        t_wall = time.perf_counter() - t_wall0
        launches = (ctx.launches - l0) // args.steps
        clocks = clocks_stop(clk, local)
        # per-kernel times: the same step launched directly (not from the
        # graph) with CUDA events around each kernel on this stream
        o_prof = gen.opts(P, YEARS, seed=0, road0=road0, sem=SEM, migration=MIG_SPARSE_FP32)
        step_device(o_prof)
        ctx.profile(True)
        for _ in range(args.steps):
            flush.zero_()
            step_device(o_prof)
        torch.cuda.synchronize()
        names = ["species_labels", "species_patches", "species_links", "mte_sparse",
                 "rov_exog", "rov_forward_sparse", "lsm_prepare", "knn_grid", "knn",
                 "knn_solve", "rov_backward"]
        split = {k: (v[0] / args.steps, v[1] // args.steps)
                 for k, v in kernel_split(ctx, names).items()}
        ctx.profile(False)
    ms = shard.max_over_ranks(sum(step_ms) / len(step_ms))
    value = args.roads * world / (ms / 1000.0)
    res = d_res.cpu().numpy().reshape(args.roads, S, RESULT_STRIDE)

    # e2e: public host-pointer entry point, pinned inputs, copies inside
    pinned = {k: torch.from_numpy(v).pin_memory() for k, v in packed.items()}
    pnp = {k: v.numpy() for k, v in pinned.items()}
    h2d = sum(v.nbytes for v in pnp.values())
    d2h = args.roads * S * RESULT_STRIDE * 8
    gen.evaluate(pnp, opts)
    torch.cuda.synchronize()
    e2e_ms = []
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        gen.evaluate(pnp, opts)
        e2e_ms.append((time.perf_counter() - t0) * 1000.0)
    e2e_value = args.roads * world / (statistics.mean(e2e_ms) / 1000.0)

    # the MTE-only generation (the step without the ROV), for comparison
    gen.set_rov(None)
    with torch.cuda.stream(stream):
        step_device(opts)
        torch.cuda.synchronize()
        mte_only_ms = statistics.mean(timed(step_device, args.steps))

    # plain: one road per call through the host entry points (the
    # reference's way), habitat maps rasterised beforehand as for the
    # batched arm; the share of that time the GPU kernels take
    plain = None
    if rank == 0 and args.plain_roads > 0:
        habs = [scene.hab_map(scene.roads[r]) for r in range(args.plain_roads)]
        pops = [[scene.pop_map(sp, habs[r]) for sp in scene.species]
                for r in range(args.plain_roads)]

        def plain_road(r):
            rd = scene.roads[r]
            models = [sg.createSpeciesModel(habs[r], pops[r][s], scene.W, scene.H, scene.res,
                                            sp.habitats, rd.colmajor(), rd.G, sp.hazard,
                                            sp.lambda_mean, sp.lambda_sd, sp.lambda_mult,
                                            sp.hab_pref_mult, sem=SEM, max_patches=512, ctx=ctx)
                      for s, sp in enumerate(scene.species)]
            sg.simulateMTECUDA(models, [sp.params for sp in scene.species], P, YEARS, seed=0,
                               road=road0 + r, sem=SEM, migration=MIG_AUTO, ctx=ctx)
            sg.simulateROVCUDA(rov_template(models, scene, P_rov, R_dim, road=road0 + r),
                               want=(), ctx=ctx)
        plain_road(0)
        ctx.profile(True)
        t0 = time.perf_counter()
        for r in range(args.plain_roads):
            plain_road(r)
        t_plain = time.perf_counter() - t0
        kern_ms = sum(v[0] for v in kernel_split(ctx, ctx.kernel_names()).values())
        ctx.profile(False)
        plain = {"value": args.plain_roads / t_plain, "unit": "designs/s",
                 "roads": args.plain_roads, "ms_per_road": 1000.0 * t_plain / args.plain_roads,
                 "gpu_kernel_ms_per_road": kern_ms / args.plain_roads,
                 "note": "one road per call: 3 species models, MTE, ROV through the host entry "
                         "points; habitat maps rasterised beforehand; the rest of each "
                         "road's time is host work and copies"}

    # roofline: the kernel that dominates the step
    bf16_peak, hbm_peak, peak_kind = measured_peaks()
    top = max(split.items(), key=lambda kv: kv[1][0]) if split else ("n/a", (0.0, 0))
    nnz = res[:, :, 7].astype(np.float64)
    mte_ms = split.get("mte_sparse", (0.0, 0))[0]
    mte_flops = 2.0 * P * float((Ns.astype(np.float64) ** 2).sum()) * YEARS
    mte_useful = 2.0 * P * float(nnz.sum()) * YEARS if (nnz >= 0).all() else None
    # units of work of the two issue-bound kernels in this step
    Q_rov = R_dim ** (S + 1)
    units = {"rov_forward_sparse": args.roads * math.ceil(P_rov / 32) * S * YEARS,
             "knn": float(res[:, 0, 15].sum()) * (YEARS - 2) * len(scene.flows) * Q_rov}
    clock_mhz = (clocks or {}).get("sm_mhz") or 2070.0
    roofline = roofline_line(top, split, units, clock_mhz, mte_flops, mte_useful, bf16_peak,
                             hbm_peak, peak_kind)

    rov_adj = rov_adjoint_leg(ctx) if rank == 0 and args.rov_leg else None
    rov_gen = rov_generation_leg(ctx) if rank == 0 and args.rov_leg else None

    surrogate = None
    if rank == 0 and args.surrogate_samples > 0:
        surrogate = surrogate_leg(args, gen, scene, P, ctx)

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        from transportoptimiser_gb300 import build as b
        b.build_oracle()
        habs = [scene.hab_map(rd) for rd in scene.roads]
        v, cores, n = oracle_generation(scene, habs, P, P_rov, R_dim, seconds=20.0)
        cpu = {"value": v, "unit": "designs/s", "cores": cores, "kind": "port",
               "sample": "%d road(s) in 20 s, one road per core, each: 3 species models, MTE "
                         "at %d paths, ROV at %d paths, 50 years" % (n, P, P_rov)}

    if rank == 0:
        line = {
            "metric": METRIC, "value": value, "unit": "designs/s", "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32", "data": "synthetic (seeded; no public dataset for this path)",
            "config": {"workload": WORKLOAD, "roads": args.roads, "species": S,
                       "mte_paths_per_road": P, "rov_paths_per_road": P_rov,
                       "pilot_paths": {"mte": PILOT_PATHS, "rov": ROV_PILOT_PATHS},
                       "years": YEARS, "rov_bins_per_dim": R_dim, "semantics": "corrected",
                       "n_star_as_reference_arm": (P, P_rov) == SCENE_N_STAR,
                       "patches_min_max": [int(Ns.min()), int(Ns.max())],
                       "graph": "whole generation (species models, MTE, ROV, results) "
                                "captured once, replayed per step",
                       "l2": "flushed (256 MB write) between steps",
                       "wall_s_timed": t_wall, "ms_steps": [round(x, 3) for x in step_ms]},
            "e2e": {"value": e2e_value, "unit": "designs/s", "h2d_bytes_per_step": h2d,
                    "ms_steps": [round(x, 3) for x in e2e_ms],
                    "d2h_bytes_per_step": d2h},
            "plain": plain,
            "batched_vs_plain": (value / plain["value"]) if plain else None,
            "mte_only": {"value": args.roads * world / (mte_only_ms / 1000.0),
                         "unit": "designs/s", "ms_per_step": mte_only_ms,
                         "note": "the same generation valued by MTE alone"},
            "kernel_ms_per_step": {k: round(v[0], 4) for k, v in split.items()},
            "rov_grid_share_fitted": float(res[:, 0, 15].mean()),
            "roofline": roofline,
            "surrogate": surrogate,
            "rov_one_road": rov_adj["rov"] if rov_adj else None,
            "rov_generation": rov_gen,
            "adjoint": rov_adj["adjoint"] if rov_adj else None,
            "cpu_baseline": cpu,
            "gpu_launches": int(launches),
            "clocks": clocks,
        }
        print(json.dumps(line), flush=True)
    gen.close()
    ctx.close()
    if world > 1:
        torch.distributed.destroy_process_group()
    return 0


# Per unit of work, from one ncu capture of this bench's own replayed step at
# 64 roads (640 ROV paths a road, 192,000 forward units, 6,180,003 fitted
# queries over the step's 48 kNN launches):
#   ncu --metrics smsp__inst_executed.sum,dram__bytes_read.sum,
#       dram__bytes_write.sum,gpu__time_duration.sum --clock-control none
#       -k "regex:k_knn_rov|k_rov_forward_union" -s 98 -c 49 --csv
#       python bench.py --profile-only --roads 64 --no-rov-leg
#       --surrogate-samples 0 --no-cpu-baseline --warmup 1
# warp instructions executed and DRAM bytes (read + write) divided by the
# units that step processed.
#   k_rov_forward_union: unit = one 32-path tile of a road, one species, one year
#   k_knn_rov: unit = one fitted regression query (k nearest points and the
#              local normal equations)
ROOF = {
    "rov_forward_sparse": {"kernel": "k_rov_forward_union", "inst_per_unit": 46845.0,
                           "bytes_per_unit": 280.0,
                           "unit": "(32-path tile, species, year)"},
    "knn": {"kernel": "k_knn_rov", "inst_per_unit": 1588.3, "bytes_per_unit": 22.8,
            "unit": "fitted regression query"},
}
SMS, SCHEDULERS = 152, 4


def roofline_line(top, split, units, clock_mhz, mte_flops, mte_useful, bf16_peak, hbm_peak,
                  peak_kind):
    """Roofline of the step's dominant kernel.  The ROV's forward pass and
    its kNN + regression kernel are both bound by instruction issue: their
    data stay in shared memory and L1/L2 (DRAM idle), and the migration
    matrices are 2.3-5% non-zero (a dense tensor-core contraction would do
    20-40x the work).  `achieved` is warp instructions per second (ncu's
    count per unit of work x the units this step processed / the kernel's
    CUDA-event time), `peak` the issue slots per second of 152 SMs x 4
    schedulers at the SM clock sampled during the timed steps."""
    peak = SMS * SCHEDULERS * clock_mhz * 1e6 / 1e9

    def issue_line(name, ms, n):
        ref = ROOF.get(name)
        line = {"kernel": ref["kernel"] if ref else "k_" + name, "kernel_ms": ms,
                "launches_per_step": n, "bound": "issue", "unit": "Gwarp-inst/s",
                "peak_kind": "issue slots: %d SMs x %d schedulers x %.0f MHz (sampled)"
                             % (SMS, SCHEDULERS, clock_mhz)}
        if ref and ref["inst_per_unit"] and ms > 0 and units.get(name):
            u = units[name]
            ach = ref["inst_per_unit"] * u / (ms / 1e3) / 1e9
            traffic = ref["bytes_per_unit"] * u / max(n, 1)
            line.update({"achieved": ach, "peak": peak, "frac": ach / peak,
                         "traffic": traffic, "traffic_unit": "bytes per launch",
                         "units_per_step": u, "unit_of_work": ref["unit"],
                         "inst_per_unit": ref["inst_per_unit"],
                         "dram_frac": (traffic * max(n, 1) / (ms / 1e3) / 1e9) / hbm_peak})
        else:
            line.update({"achieved": None, "peak": peak, "frac": None, "traffic": None})
        return line

    name, (ms, n) = top
    out = issue_line(name, ms, n)
    # the other issue-bound kernel of the step
    out["others"] = [issue_line(k, *split[k]) for k in ROOF if k != name and k in split]
    mte_ms = split.get("mte_sparse", (0.0, 0))[0]
    out["mte_sparse"] = {"ms": mte_ms, "dense_equiv_tflops": (mte_flops / (mte_ms / 1e3) / 1e12)
                         if mte_ms > 0 else None,
                         "useful_tflops": (mte_useful / (mte_ms / 1e3) / 1e12)
                         if (mte_ms > 0 and mte_useful) else None,
                         "frac_of_bf16_peak": (mte_flops / (mte_ms / 1e3) / 1e12 / bf16_peak)
                         if mte_ms > 0 else None,
                         "bf16_peak_kind": peak_kind}
    return out


if __name__ == "__main__":
    sys.exit(main())
