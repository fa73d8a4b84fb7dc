"""ctypes view of ``include/transopt.h``.

Loads the in-tree ``_lib/libtransopt.so`` and fails loudly when it is
missing: there is no CPU fallback in this package.
"""
from __future__ import annotations

import ctypes as C
from pathlib import Path

import numpy as np

_LIB_PATH = Path(__file__).resolve().parent / "_lib" / "libtransopt.so"

TO_OK = 0
STATUS_NAMES = {
    0: "TO_OK", 1: "TO_ERR_INVALID", 2: "TO_ERR_CUDA", 3: "TO_ERR_ALLOC",
    4: "TO_ERR_NONFINITE", 5: "TO_ERR_TIMEOUT", 6: "TO_ERR_UNSUPPORTED",
    7: "TO_ERR_NO_DEVICE",
}
SEM_REFERENCE, SEM_CORRECTED = 0, 1
MIG_AUTO, MIG_SIMT_FP32, MIG_TC_3XTF32, MIG_SPARSE_FP32 = 0, 1, 2, 3

c_int_p = C.POINTER(C.c_int)
c_double_p = C.POINTER(C.c_double)
c_float_p = C.POINTER(C.c_float)


class Habitat(C.Structure):
    _fields_ = [("type", C.c_int), ("max_pop", C.c_double),
                ("pref_mean", C.c_double), ("pref_sd", C.c_double)]


class SpeciesIn(C.Structure):
    _fields_ = [("W", C.c_int), ("H", C.c_int), ("res", C.c_int),
                ("xspacing", C.c_double), ("yspacing", C.c_double),
                ("n_hab", C.c_int), ("habs", C.POINTER(Habitat)),
                ("hab_map", c_int_p), ("pop_map", c_double_p),
                ("G", C.c_int), ("road", c_double_p),
                ("lambda_mean", C.c_double), ("lambda_sd", C.c_double),
                ("lambda_mult", C.c_double), ("hab_pref_mult", C.c_double),
                ("n_controls", C.c_int), ("hazard", c_double_p),
                ("sem", C.c_int)]


class SpeciesOut(C.Structure):
    _fields_ = [("max_patches", C.c_int), ("n_patches", C.c_int),
                ("n_transitions", C.c_int),
                ("area", c_double_p), ("cap", c_double_p), ("pop", c_double_p),
                ("cx", c_double_p), ("cy", c_double_p), ("type", c_int_p),
                ("crossings", c_int_p), ("trans", c_double_p),
                ("surv", c_double_p), ("mmm", c_float_p), ("iar", c_double_p)]


class MteSpecies(C.Structure):
    _fields_ = [("n_patches", C.c_int), ("params", c_float_p),
                ("init_pops", c_float_p), ("caps", c_float_p),
                ("mmm", c_float_p)]


class MteProblem(C.Structure):
    _fields_ = [("n_species", C.c_int), ("n_paths", C.c_int),
                ("n_years", C.c_int), ("dt", C.c_float), ("seed", C.c_uint64),
                ("road", C.c_int), ("sem", C.c_int), ("migration", C.c_int),
                ("species", C.POINTER(MteSpecies))]


class MteStats(C.Structure):
    _fields_ = [("mean", C.c_double), ("sd", C.c_double), ("se", C.c_double),
                ("p_below", C.c_double), ("init_total", C.c_double)]


class MteDeviceProblem(C.Structure):
    _fields_ = [("n_species", C.c_int), ("n_paths", C.c_int), ("n_years", C.c_int),
                ("npad", C.c_int), ("dt", C.c_float), ("seed", C.c_uint64), ("road", C.c_int),
                ("sem", C.c_int), ("n_patches", C.c_void_p), ("params", C.c_void_p),
                ("init_pops", C.c_void_p), ("caps", C.c_void_p), ("mmm", C.c_void_p)]


class Penalty(C.Structure):
    _fields_ = [("confidence", C.c_double), ("threshold", c_double_p),
                ("init_population", c_double_p), ("cost_per_animal", c_double_p)]


class ExpPvParams(C.Structure):
    _fields_ = [(n, C.c_float) for n in ("gr", "mean", "time_step", "rrr",
                                         "current", "reversion", "jump_prob",
                                         "noise_sd", "jump_sd")]


class SpeciesDesc(C.Structure):
    _fields_ = [("n_hab", C.c_int), ("habs", C.POINTER(Habitat)), ("pop_map", c_double_p),
                ("hazard", c_double_p), ("params", c_float_p),
                ("lambda_mean", C.c_double), ("lambda_sd", C.c_double),
                ("lambda_mult", C.c_double), ("hab_pref_mult", C.c_double)]


class Scene(C.Structure):
    _fields_ = [("W", C.c_int), ("H", C.c_int), ("res", C.c_int),
                ("xspacing", C.c_double), ("yspacing", C.c_double),
                ("base_map", c_int_p), ("n_species", C.c_int),
                ("species", C.POINTER(SpeciesDesc)), ("n_controls", C.c_int),
                ("max_patches", C.c_int), ("max_roads", C.c_int),
                ("max_cells", C.c_int), ("max_segments", C.c_int)]


class EvalOpts(C.Structure):
    _fields_ = [("mte_paths", C.c_int), ("n_years", C.c_int), ("dt", C.c_float),
                ("seed", C.c_uint64), ("road0", C.c_int), ("sem", C.c_int),
                ("migration", C.c_int), ("graph", C.c_int)]


RESULT_STRIDE = 24


class RovSpecies(C.Structure):
    _fields_ = [("n_patches", C.c_int), ("params", c_float_p), ("init_pops", c_float_p),
                ("caps", c_float_p), ("mmm", c_float_p)]


class RovProblem(C.Structure):
    _fields_ = [("n_species", C.c_int), ("n_paths", C.c_int), ("n_years", C.c_int),
                ("n_controls", C.c_int), ("dim_res", C.c_int),
                ("species", C.POINTER(RovSpecies)), ("flows", c_float_p),
                ("n_uncertainties", C.c_int), ("uncert", c_float_p), ("n_fuels", C.c_int),
                ("fuel_costs", c_float_p), ("fuel_idx", c_int_p), ("n_commodities", C.c_int),
                ("ore_content", c_float_p), ("ore_sd", c_float_p), ("unit_cost", C.c_float),
                ("unit_revenue", C.c_float), ("dt", C.c_float), ("rrr", C.c_float),
                ("demand_idx", C.c_int), ("seed", C.c_uint64), ("road", C.c_int),
                ("sem", C.c_int), ("migration", C.c_int), ("algo", C.c_int)]


class RovResult(C.Structure):
    _fields_ = [("cond_exp", c_double_p), ("opt_cont", c_int_p), ("unit_profits", c_double_p),
                ("adj_pops", c_double_p), ("regression", c_double_p), ("value", C.c_double),
                ("control", C.c_double), ("sd", C.c_double), ("se", C.c_double),
                ("n_best", C.c_int)]

# name -> (restype, argtypes); every symbol declared in include/transopt.h
SIGNATURES = {
    "to_device_count": (C.c_int, [c_int_p]),
    "to_ctx_create": (C.c_int, [C.c_int, C.POINTER(C.c_void_p)]),
    "to_ctx_destroy": (C.c_int, [C.c_void_p]),
    "to_ctx_set_stream": (C.c_int, [C.c_void_p, C.c_void_p]),
    "to_ctx_synchronize": (C.c_int, [C.c_void_p]),
    "to_status_string": (C.c_char_p, [C.c_int]),
    "to_last_error": (C.c_char_p, [C.c_void_p]),
    "to_ctx_launch_count": (C.c_uint64, [C.c_void_p]),
    "to_simulate_rov_batch": (C.c_int, [C.c_void_p, C.c_int, C.POINTER(RovProblem),
                                        C.POINTER(RovResult)]),
    "to_ctx_profile": (C.c_int, [C.c_void_p, C.c_int]),
    "to_ctx_inject_fault": (C.c_int, [C.c_void_p, C.c_int]),
    "to_ctx_kernel_time": (C.c_int, [C.c_void_p, C.c_char_p, c_double_p, c_int_p]),
    "to_label_image": (C.c_int, [C.c_void_p, C.c_int, C.c_int, c_int_p, c_int_p, c_int_p]),
    "to_build_patches": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_int,
                                   C.c_int, C.c_int, C.c_int, C.c_double, C.c_double,
                                   C.c_double, C.c_double, c_int_p, c_double_p,
                                   C.c_int, c_double_p, c_double_p, c_double_p,
                                   c_double_p, c_double_p, c_double_p, c_int_p]),
    "to_line_segment_intersect": (C.c_int, [C.c_void_p, C.c_int, c_double_p,
                                            C.c_int, c_double_p, c_int_p]),
    "to_species_model": (C.c_int, [C.c_void_p, C.POINTER(SpeciesIn),
                                   C.POINTER(SpeciesOut)]),
    "to_simulate_mte": (C.c_int, [C.c_void_p, C.POINTER(MteProblem), c_double_p,
                                  C.POINTER(MteStats)]),
    "to_simulate_mte_noalloc_d": (C.c_int, [C.c_void_p, C.POINTER(MteDeviceProblem),
                                            C.c_void_p]),
    "to_exp_pv": (C.c_int, [C.c_void_p, C.POINTER(ExpPvParams), C.c_int, C.c_int,
                            C.c_uint64, C.c_int, C.c_int, c_float_p, c_double_p,
                            c_double_p]),
    "to_simulate_rov": (C.c_int, [C.c_void_p, C.POINTER(RovProblem), C.POINTER(RovResult)]),
    "to_knn": (C.c_int, [C.c_void_p, c_float_p, C.c_int, c_float_p, C.c_int, C.c_int, C.c_int,
                         c_float_p, c_int_p]),
    "to_build_surrogate_mte": (C.c_int, [C.c_void_p, C.c_int, c_double_p, c_double_p,
                                         c_double_p, C.c_int, c_double_p, c_double_p]),
    "to_build_surrogate_rov": (C.c_int, [C.c_void_p, C.c_int, C.c_int, c_double_p, c_double_p,
                                         c_double_p, C.c_int, C.c_int, c_double_p, c_double_p]),
    "to_scene_create": (C.c_int, [C.c_void_p, C.POINTER(Scene), C.POINTER(C.c_void_p)]),
    "to_scene_destroy": (C.c_int, [C.c_void_p]),
    "to_evaluate_roads": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, c_int_p, c_int_p,
                                    c_int_p, c_double_p, C.POINTER(EvalOpts), c_double_p]),
    "to_evaluate_roads_d": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p,
                                      C.c_void_p, C.c_void_p, C.c_void_p,
                                      C.POINTER(EvalOpts), C.c_void_p]),
    "to_ctx_tuning": (C.c_int, [C.c_void_p, C.c_char_p, C.c_int]),
    "to_scene_set_penalty": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "to_scene_set_rov": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "to_gen_end_pops": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int,
                                  c_float_p]),
    "to_gen_species_model": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int,
                                       c_int_p, c_float_p, c_float_p, c_float_p, c_int_p]),
    "to_select_samples": (C.c_int, [C.c_void_p, C.c_int, c_double_p, C.c_int, c_double_p,
                                    C.c_int, C.c_int, c_int_p]),
    "to_interpolate_surrogate": (C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_int, c_double_p,
                                           c_double_p, c_double_p, C.c_int]),
    "to_road_features": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, c_int_p, c_double_p,
                                   c_float_p]),
    "to_road_features_d": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p,
                                     C.c_void_p, C.c_void_p, C.c_void_p]),
    "to_adjoint_forward": (C.c_int, [C.c_void_p, C.c_void_p, c_double_p, c_double_p,
                                     C.POINTER(C.c_void_p)]),
    "to_adjoint_backward": (C.c_int, [C.c_void_p, C.c_void_p, c_double_p, c_double_p]),
    "to_tape_destroy": (C.c_int, [C.c_void_p]),
    "to_mlp_predict": (C.c_int, [C.c_void_p, c_float_p, C.c_int, c_float_p, c_float_p]),
    "to_mlp_predict_d": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_void_p, C.c_void_p]),
    "to_mlp_grad": (C.c_int, [C.c_void_p, c_float_p, C.c_int, c_float_p, c_float_p, c_float_p,
                              c_double_p]),
    "to_mlp_train": (C.c_int, [C.c_void_p, c_float_p, C.c_int, c_float_p, c_float_p, C.c_int,
                               C.c_int, C.c_float, C.c_uint64, c_double_p]),
}

_lib = None


def load(path: Path | None = None) -> C.CDLL:
    """Load libtransopt.so (raises if it has not been built)."""
    global _lib
    if _lib is not None:
        return _lib
    p = Path(path) if path else _LIB_PATH
    if not p.exists():
        raise RuntimeError(
            f"{p} is missing: build it with `python -c 'import __graft_entry__ as g; g.build()'`")
    lib = C.CDLL(str(p))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


class TransOptError(RuntimeError):
    def __init__(self, status: int, where: str, detail: str = ""):
        self.status = status
        super().__init__(f"{where}: {STATUS_NAMES.get(status, status)} {detail}".strip())


def ptr(a: np.ndarray | None, ctype):
    if a is None:
        return None
    assert a.flags["C_CONTIGUOUS"], "array must be C-contiguous"
    return a.ctypes.data_as(C.POINTER(ctype))


class Context:
    """Owns a to_ctx (device, stream, scratch arena)."""

    def __init__(self, device: int = 0):
        self.lib = load()
        h = C.c_void_p()
        st = self.lib.to_ctx_create(device, C.byref(h))
        if st != TO_OK:
            raise TransOptError(st, "to_ctx_create")
        self.handle = h

    def check(self, st: int, where: str) -> None:
        if st != TO_OK:
            msg = self.lib.to_last_error(self.handle)
            raise TransOptError(st, where, msg.decode() if msg else "")

    @property
    def launches(self) -> int:
        return int(self.lib.to_ctx_launch_count(self.handle))

    def set_stream(self, stream_ptr: int) -> None:
        self.check(self.lib.to_ctx_set_stream(self.handle, C.c_void_p(stream_ptr)),
                   "to_ctx_set_stream")

    def synchronize(self) -> None:
        self.check(self.lib.to_ctx_synchronize(self.handle), "to_ctx_synchronize")

    def profile(self, enable: bool = True) -> None:
        self.check(self.lib.to_ctx_profile(self.handle, int(enable)), "to_ctx_profile")

    # kernels bracketed by the context's event timing (to_ctx_profile)
    KERNEL_NAMES = ("adjoint_backward", "adjoint_forward", "knn", "knn_grid", "knn_solve",
                    "lsm_prepare", "mte_simt", "mte_sparse", "mte_tc", "pack_csc", "rasterise",
                    "road_features", "rov_backward", "rov_exog", "rov_forward",
                    "rov_forward_sparse", "rov_resim", "select_samples", "species_labels",
                    "species_links", "species_patches", "surrogate_regress", "tc_pack")

    def kernel_names(self):
        return self.KERNEL_NAMES

    def kernel_time(self, name: str):
        ms = C.c_double(0.0)
        n = C.c_int(0)
        self.check(self.lib.to_ctx_kernel_time(self.handle, name.encode(), C.byref(ms),
                                               C.byref(n)), "to_ctx_kernel_time")
        return ms.value, n.value

    def tuning(self) -> str:
        """The autotuner's record of measured migration-kernel choices."""
        buf = C.create_string_buffer(8192)
        self.lib.to_ctx_tuning(self.handle, buf, len(buf))
        return buf.value.decode()

    def close(self) -> None:
        if getattr(self, "handle", None):
            self.lib.to_ctx_destroy(self.handle)
            self.handle = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
