"""Generates tests/golden/*.npz from the reference's own kernels.

Runs the reference kernels compiled for the CPU (oracle/build_ref.sh, only
where the reference tree is mounted) on small seeded synthetic inputs and
stores inputs and outputs, so that tests on any machine can pin the oracle
(and through it the GPU path) to the reference's arithmetic.

    python tests/golden/make_golden.py
"""
from __future__ import annotations

import math
import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from oracle import pyoracle as po  # noqa: E402
from transportoptimiser_gb300 import synth  # noqa: E402

OUT = Path(__file__).resolve().parent


def patches_case(seed: int, scene=None, types=(0, 1, 2)):
    sc = scene if scene is not None else synth.mte_road(seed)
    sp, road = sc.species[0], sc.roads[0]
    hab = sc.hab_map(road)
    W = H = sc.W
    res = sc.res
    xres = res if W % res == 0 else res + 1
    skp = (W - 1) // res
    popm = sc.pop_map(sp, hab)
    labels, nregs, area, cap, pop, cx, cy = [], [], [], [], [], [], []
    for typ in types:
        lab, nr = po.label_image(W, H, (hab == typ).astype(np.int32), lib=po.ref())
        labels.append(lab)
        nregs.append(nr)
        r = po.build_patches(W, H, skp, skp, xres, xres, nr, 1.0, 1.0, 1.0, 50.0, lab, popm,
                             use_ref=True)
        area.append(r["area"]); cap.append(r["cap"]); pop.append(r["pop"])
        cx.append(r["cx"]); cy.append(r["cy"])
    cat = lambda v: np.concatenate(v)
    cxa, cya = cat(cx), cat(cy)
    N = len(cxa)
    md = math.log(0.05) / (-sp.lambda_mean)
    pairs = [(i, j) for i in range(N) for j in range(i + 1, N)
             if math.hypot(cxa[i] - cxa[j], cya[i] - cya[j]) <= md][:-1]
    xy1 = np.array([[cxa[i], cya[i], cxa[j], cya[j]] for i, j in pairs]).T.reshape(-1)
    cr = po.line_segment_intersect(xy1, len(pairs), road.colmajor(), road.G, use_ref=True)
    return dict(hab=hab, pop_map=popm, W=W, res=res, road=road.colmajor(), G=road.G,
                types=np.array(types, np.int32),
                labels=np.stack(labels), nregs=np.array(nregs), area=cat(area), cap=cat(cap),
                pop=cat(pop), cx=cxa, cy=cya, pairs=np.array(pairs, np.int32), xy1=xy1,
                pair_crossings=cr)


def mte_case(seed: int, P=64, Y=30, scene=None):
    sc = scene if scene is not None else synth.mte_road(seed)
    sp, road = sc.species[0], sc.roads[0]
    m = po.species_model(sc, sp, road, sem=0, max_patches=1024)
    end = po.ref_simulate_mte(P, Y, m["N"], 1.0, sp.params, m["init_pops"], m["caps"],
                              m["mmm"][2], seed, 0, 0)
    return dict(P=P, Y=Y, N=m["N"], params=sp.params, init=m["init_pops"], caps=m["caps"],
                mmm=m["mmm"][2], seed=seed, end=end)


def exppv_case(seed: int):
    prm = np.array([0.02, 1.0, 1.0, 0.07, 1.0, 0.3, 0.1, 0.1, 0.2], np.float32)
    vals, mean, sd = po.ref_exp_pv(200, 40, prm, seed, 0)
    return dict(prm=prm, P=200, Y=40, seed=seed, values=vals, mean=mean, sd=sd)


def rov_problem(seed: int, P=600, Y=12, R=8, scene=None):
    from transportoptimiser_gb300.rov import rov_problem_from_models
    sc = scene if scene is not None else synth.mte_road(seed)
    m = po.species_model(sc, sc.species[0], sc.roads[0], sem=0)
    return rov_problem_from_models([m], sc, n_paths=P, n_years=Y, dim_res=R, n_processes=2,
                                   seed=seed)


def rov_case(seed: int, **kw):
    rp = rov_problem(seed, **kw)
    out = po.ref_simulate_rov(rp)
    sp = rp["species"][0]
    flat = {k: v for k, v in rp.items() if k != "species"}
    flat.update({"sp_" + k: np.asarray(v) for k, v in sp.items()})
    flat.update({"out_" + k: v for k, v in out.items()})
    return flat


def knn_case(seed: int):
    rng = np.random.default_rng(seed)
    n, Q, dim, k = 500, 200, 3, 30
    ref_pts = rng.random((dim, n)).astype(np.float32)
    ref_pts[:, 10] = ref_pts[:, 3]          # an exact duplicate: tie on distance
    q = rng.random((dim, Q)).astype(np.float32)
    dist, ind = po.knn(ref_pts, n, q, Q, dim, k, use_ref=True)
    return dict(ref=ref_pts, query=q, k=k, dist=dist, ind=ind)


def surrogate_case(seed: int):
    rng = np.random.default_rng(seed)
    n, d, R = 300, 2, 8
    pred = rng.random((d, n)).astype(np.float32) * np.array([[2.0], [50.0]], np.float32)
    y = (-(pred[0] ** 2) * 10 - pred[1]).astype(np.float32)
    mean = po.build_surrogate_nd(pred, y, R, clip=1, use_ref=True)
    return dict(pred=pred, y=y, R=R, mean=mean)


def main():
    if not po.ref_available():
        po.ref()
    np.savez_compressed(OUT / "patches_crossings.npz", **patches_case(0))
    np.savez_compressed(OUT / "mte.npz", **mte_case(0))
    np.savez_compressed(OUT / "exppv.npz", **exppv_case(0))
    np.savez_compressed(OUT / "rov.npz", **rov_case(0))
    np.savez_compressed(OUT / "knn.npz", **knn_case(0))
    np.savez_compressed(OUT / "surrogate_rov.npz", **surrogate_case(0))
    # at the benchmark shapes: the 200 x 200 generation grid (patches and
    # crossings of its first road, 4 habitable types), the plain MTE at 2000
    # paths x 50 years, the MTE of a generation road (~300 patches) over 50
    # years, and the one-species ROV (the reference's multi-species ROV is
    # not defined) at 2000 paths x 50 years with 16 bins per dimension
    gen = synth.generation(0, n_roads=1)
    np.savez_compressed(OUT / "patches_crossings_gen.npz",
                        **patches_case(0, scene=gen, types=(0, 1, 2, 5)))
    np.savez_compressed(OUT / "mte_y50.npz", **mte_case(0, P=2000, Y=50))
    np.savez_compressed(OUT / "mte_gen.npz", **mte_case(0, P=256, Y=50, scene=gen))
    np.savez_compressed(OUT / "rov_y50.npz", **rov_case(0, P=2000, Y=50, R=16))
    print("golden fixtures written to", OUT)


if __name__ == "__main__":
    main()
