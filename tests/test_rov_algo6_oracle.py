"""ALGO6 oracle (path re-simulation under the optimal policy) on the CPU:
the year's value is the realised discounted payoff along the re-simulated
path, and the terminal year is shared with ALGO4."""
import numpy as np

from oracle import pyoracle as po
from transportoptimiser_gb300 import synth
from transportoptimiser_gb300.rov import rov_problem_from_models


def _problem(algo, Y=3, P=300):
    sc = synth.rov_road(3, n_species=2)
    models = [po.species_model(sc, sc.species[s], sc.roads[0], sem=1) for s in range(2)]
    return rov_problem_from_models(models, sc, n_paths=P, n_years=Y, dim_res=8, sem=1,
                                   n_processes=3, demand=True, seed=4, road=7, algo=algo)


def test_three_years_value_is_realised_two_year_payoff():
    rp = _problem(6)
    o = po.simulate_rov(rp, threads=4)
    P, Y = rp["n_paths"], rp["n_years"]
    ce = o["cond_exp"].reshape(Y, P)
    oc = o["opt_cont"].reshape(Y, P)
    up = o["unit_profits"].reshape(Y, P)
    flows = np.asarray(rp["flows"], np.float32)
    disc = np.float32(1.0) + np.float32(rp["rrr"]) * np.float32(rp["dt"]) / np.float32(100.0)
    df = np.float32(1.0) / disc
    for p in range(P):
        first = flows[oc[1, p]] * up[1, p]
        # the year-2 control is the terminal decision on the re-simulated state
        cands = [np.float32(first) + (flows[c] * up[2, p]) * df for c in range(len(flows))]
        assert any(ce[1, p] == c for c in cands), (p, ce[1, p], cands)


def test_terminal_year_shared_with_algo4():
    a4 = po.simulate_rov(_problem(4, Y=8), threads=4)
    a6 = po.simulate_rov(_problem(6, Y=8), threads=4)
    P, Y = 300, 8
    assert np.array_equal(a4["cond_exp"].reshape(Y, P)[Y - 1], a6["cond_exp"].reshape(Y, P)[Y - 1])
    assert np.array_equal(a4["opt_cont"].reshape(Y, P)[Y - 1], a6["opt_cont"].reshape(Y, P)[Y - 1])
    assert not np.array_equal(a4["cond_exp"].reshape(Y, P)[1], a6["cond_exp"].reshape(Y, P)[1])
