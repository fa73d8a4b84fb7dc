"""ROV (controlled traffic) problem description shared by the GPU entry
point and the synthetic workloads.

A problem is a dict:
    n_paths, n_years, dim_res, dt, rrr, unit_cost, unit_revenue, seed, road, sem
    species:  list of {N, params[8], init_pops[N], caps[N], mmm[C][N][N]}
    flows[C]: traffic flow of each control (the reference's Q)
    uncert[U*6]: per exogenous process (fuels first, then commodities):
                 current, mean, sd, reversion, jump size, jump probability
    fuel_costs[nF], fuel_idx[nF]: unit fuel use and the process it prices
    ore_content[Cm], ore_sd[Cm]: ore composition per commodity
    demand_idx: process that multiplies the unit profit (-1: none)
"""
from __future__ import annotations

import numpy as np


def rov_problem_from_models(models, scene, n_paths, n_years=50, dim_res=16, seed=0, road=0,
                            sem=0, rrr=7.0, n_processes=3, demand=False, algo=4):
    """Builds a ROV problem from species models (dicts with N, init_pops,
    caps, mmm) of a synthetic scene.  Processes: fuel price, commodity price
    and (corrected semantics) traffic demand, mean-reverting with theta
    0.2/0.35/0.5 and sigma 0.1/0.2/0.3, no jumps.  algo 4: regression values
    (ALGO4); 6: values of paths re-simulated under the optimal policy
    (ALGO6, sem 1)."""
    species = []
    for m, sp in zip(models, scene.species):
        params = np.array(sp.params, np.float32).copy()
        params[2] = 0.05          # growth-rate noise sd
        species.append(dict(N=int(m["N"]), params=params, init_pops=m["init_pops"],
                            caps=m["caps"], mmm=np.ascontiguousarray(m["mmm"])))
    theta = [0.2, 0.35, 0.5]
    sigma = [0.1, 0.2, 0.3]
    uncert = []
    for u in range(n_processes):
        uncert += [1.0, 1.0, sigma[u], theta[u], 0.0, 0.0]
    return dict(n_paths=n_paths, n_years=n_years, dim_res=dim_res, dt=1.0, rrr=rrr,
                unit_cost=0.5, unit_revenue=1.2, seed=seed, road=road, sem=sem,
                species=species, flows=np.asarray(scene.flows, np.float32) * 100.0,
                uncert=np.asarray(uncert, np.float32),
                fuel_costs=np.array([0.3], np.float32), fuel_idx=np.array([0], np.int32),
                ore_content=np.array([0.8], np.float32), ore_sd=np.array([0.05], np.float32),
                demand_idx=(2 if (demand and n_processes > 2) else -1), algo=algo)
