"""Helpers shared by the ROV tests."""
import numpy as np


def problem_from_golden(g):
    sp = {k[3:]: g[k] for k in g if k.startswith("sp_")}
    sp["N"] = int(sp["N"])
    rp = {k: g[k] for k in g if not k.startswith(("sp_", "out_"))}
    for k in ("n_paths", "n_years", "dim_res", "seed", "road", "sem", "demand_idx"):
        rp[k] = int(rp[k])
    for k in ("dt", "rrr", "unit_cost", "unit_revenue"):
        rp[k] = float(rp[k])
    rp["species"] = [sp]
    return rp


def ref_outputs(g):
    return {k[4:]: g[k] for k in g if k.startswith("out_")}
