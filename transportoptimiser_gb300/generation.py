"""Batched valuation of a GA generation of roads (C ABI to_scene_* /
to_evaluate_roads*).  The scene is uploaded once and stays resident; each
call streams in only the road geometry."""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _capi
from ._capi import Context, ptr
from .synth import Scene as SynthScene
from .synth import road_cells


def pack_roads(scene: SynthScene, roads, sem: int = 1) -> dict:
    """CSR arrays (cell offsets, cells, segment offsets, segments); the road
    cells by RoadCells::computeRoadCells' rule (sem 0 keeps its quirk)."""
    cell_off, cells, seg_off, segs = [0], [], [0], []
    for rd in roads:
        cs = [x + y * scene.W for (x, y) in road_cells(rd, scene.W, scene.H, sem=sem)]
        cells.extend(cs)
        cell_off.append(len(cells))
        segs.append(np.asarray(rd.segments, np.float64).reshape(-1))
        seg_off.append(seg_off[-1] + rd.G)
    return dict(cell_off=np.asarray(cell_off, np.int32), cells=np.asarray(cells, np.int32),
                seg_off=np.asarray(seg_off, np.int32),
                segs=np.ascontiguousarray(np.concatenate(segs) if segs else np.zeros(4)))


def pack_segments(roads) -> dict:
    """Segment CSR only (the device computes the road cells)."""
    seg_off = np.zeros(len(roads) + 1, np.int32)
    segs = []
    for r, rd in enumerate(roads):
        segs.append(np.asarray(rd.segments, np.float64).reshape(-1))
        seg_off[r + 1] = seg_off[r] + rd.G
    return dict(seg_off=seg_off,
                segs=np.ascontiguousarray(np.concatenate(segs) if segs else np.zeros(4)))


class Generation:
    """Resident scene + per-generation evaluation."""

    def __init__(self, scene: SynthScene, max_roads: int, max_patches: int = 512,
                 max_cells: int | None = None, max_segments: int | None = None,
                 ctx: Context | None = None):
        from .simulate_gpu import context
        self.ctx = ctx or context()
        self.scene = scene
        self.S = len(scene.species)
        self._keep = []
        descs = (_capi.SpeciesDesc * self.S)()
        base = np.ascontiguousarray(scene.base_map, np.int32)
        self._keep.append(base)
        for s, sp in enumerate(scene.species):
            habs = (_capi.Habitat * len(sp.habitats))(
                *[_capi.Habitat(h.type, h.max_pop, h.pref_mean, h.pref_sd) for h in sp.habitats])
            popm = np.ascontiguousarray(scene.pop_map(sp, scene.base_map), np.float64)
            hz = np.ascontiguousarray(sp.hazard, np.float64)
            prm = np.ascontiguousarray(sp.params, np.float32)
            self._keep += [habs, popm, hz, prm]
            descs[s] = _capi.SpeciesDesc(len(sp.habitats), habs, ptr(popm, C.c_double),
                                         ptr(hz, C.c_double), ptr(prm, C.c_float),
                                         sp.lambda_mean, sp.lambda_sd, sp.lambda_mult,
                                         sp.hab_pref_mult)
        self._keep.append(descs)
        sc = _capi.Scene(scene.W, scene.H, scene.res, 1.0, 1.0, ptr(base, C.c_int), self.S,
                         descs, scene.n_controls, max_patches, max_roads,
                         max_cells or 64 * max_roads * scene.W, max_segments or 128 * max_roads)
        h = C.c_void_p()
        self.ctx.check(self.ctx.lib.to_scene_create(self.ctx.handle, C.byref(sc), C.byref(h)),
                       "to_scene_create")
        self.handle = h
        self.max_roads = max_roads

    def opts(self, mte_paths, n_years=50, dt=1.0, seed=0, road0=0, sem=0,
             migration=_capi.MIG_AUTO, graph=False):
        return _capi.EvalOpts(mte_paths, n_years, dt, seed, road0, sem, migration, int(graph))

    def evaluate(self, packed: dict, opts) -> np.ndarray:
        """Host-pointer entry point; returns [R][S][RESULT_STRIDE]."""
        R = len(packed["cell_off"]) - 1
        out = np.zeros(R * self.S * _capi.RESULT_STRIDE, np.float64)
        self.ctx.check(self.ctx.lib.to_evaluate_roads(
            self.ctx.handle, self.handle, R, ptr(packed["cell_off"], C.c_int),
            ptr(packed["cells"], C.c_int) if len(packed["cells"]) else None,
            ptr(packed["seg_off"], C.c_int), ptr(packed["segs"], C.c_double),
            C.byref(opts), ptr(out, C.c_double)), "to_evaluate_roads")
        return out.reshape(R, self.S, _capi.RESULT_STRIDE)

    def evaluate_segments(self, packed: dict, opts) -> np.ndarray:
        """Host entry point with the road cells rasterised on the device."""
        R = len(packed["seg_off"]) - 1
        out = np.zeros(R * self.S * _capi.RESULT_STRIDE, np.float64)
        self.ctx.check(self.ctx.lib.to_evaluate_roads(
            self.ctx.handle, self.handle, R, None, None, ptr(packed["seg_off"], C.c_int),
            ptr(packed["segs"], C.c_double), C.byref(opts), ptr(out, C.c_double)),
            "to_evaluate_roads")
        return out.reshape(R, self.S, _capi.RESULT_STRIDE)

    def features(self, packed: dict) -> np.ndarray:
        """[R][16] surrogate features (to_road_features)."""
        R = len(packed["seg_off"]) - 1
        out = np.zeros((R, 16), np.float32)
        self.ctx.check(self.ctx.lib.to_road_features(
            self.ctx.handle, self.handle, R, ptr(packed["seg_off"], C.c_int),
            ptr(packed["segs"], C.c_double), ptr(out, C.c_float)), "to_road_features")
        return out

    def evaluate_device(self, R, d_cell_off, d_cells, d_seg_off, d_segs, opts, d_results):
        """Device-pointer entry point (ints are raw device addresses)."""
        self.ctx.check(self.ctx.lib.to_evaluate_roads_d(
            self.ctx.handle, self.handle, R, C.c_void_p(d_cell_off), C.c_void_p(d_cells),
            C.c_void_p(d_seg_off), C.c_void_p(d_segs), C.byref(opts),
            C.c_void_p(d_results)), "to_evaluate_roads_d")

    def set_penalty(self, confidence, threshold, init_population, cost_per_animal):
        """MTE penalty per species (to_scene_set_penalty)."""
        arrs = [np.ascontiguousarray(x, np.float64) for x in (threshold, init_population,
                                                             cost_per_animal)]
        pen = _capi.Penalty(confidence, *[ptr(a, C.c_double) for a in arrs])
        self.ctx.check(self.ctx.lib.to_scene_set_penalty(self.ctx.handle, self.handle,
                                                         C.byref(pen)), "to_scene_set_penalty")

    def set_rov(self, problem: dict | None, species_params: bool = True):
        """ROV valuation of every road in evaluate() (to_scene_set_rov).
        ``problem`` is a ROV problem dict (transportoptimiser_gb300.rov) whose
        road-independent fields apply to every road; its species' params are
        used when species_params, else the scene's.  None switches it off."""
        if problem is None:
            self.ctx.check(self.ctx.lib.to_scene_set_rov(self.ctx.handle, self.handle, None),
                           "to_scene_set_rov")
            return
        from .simulate_gpu import rov_ctypes
        pr, keep = rov_ctypes(problem)
        if not species_params:
            pr.species = None
        self.ctx.check(self.ctx.lib.to_scene_set_rov(self.ctx.handle, self.handle, C.byref(pr)),
                       "to_scene_set_rov")

    def end_pops(self, road: int, species: int, n_paths: int) -> np.ndarray:
        """Per-path end populations of (road, species) from the last call."""
        out = np.zeros(n_paths, np.float32)
        self.ctx.check(self.ctx.lib.to_gen_end_pops(self.ctx.handle, self.handle, road, species,
                                                    n_paths, ptr(out, C.c_float)),
                       "to_gen_end_pops")
        return out

    def species_model(self, road: int, species: int, max_patches: int = 1024) -> dict:
        """The species model the last call's migration kernel read: N, initial
        populations, capacities, dense destination-major matrices [C][N][N]
        and the packed non-zero counts (-1: none packed)."""
        n = C.c_int(0)
        ip = np.zeros(max_patches, np.float32)
        cp = np.zeros(max_patches, np.float32)
        Cn = self.scene.n_controls
        nnz = np.zeros(Cn, np.int32)
        self.ctx.check(self.ctx.lib.to_gen_species_model(
            self.ctx.handle, self.handle, road, species, max_patches, C.byref(n),
            ptr(ip, C.c_float), ptr(cp, C.c_float), None, ptr(nnz, C.c_int)),
            "to_gen_species_model")
        N = n.value
        mmm = np.zeros(Cn * N * N, np.float32)
        self.ctx.check(self.ctx.lib.to_gen_species_model(
            self.ctx.handle, self.handle, road, species, max_patches, C.byref(n), None, None,
            ptr(mmm, C.c_float), None), "to_gen_species_model")
        return dict(N=N, init_pops=ip[:N].copy(), caps=cp[:N].copy(),
                    mmm=mmm.reshape(Cn, N, N), nnz=nnz)

    def close(self):
        if getattr(self, "handle", None):
            self.ctx.lib.to_scene_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
