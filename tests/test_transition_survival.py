"""The species model's FP64 host arithmetic, restated a second time in numpy
straight from the reference's formulas and compared with the oracle:

* habitatPatchDistances (include/road/SpeciesRoadPatches.cpp:270-294):
  d(i, j) = sqrt((cx_i - cx_j)^2 + (cy_i - cy_j)^2);
* computeTransitionProbabilities (:383-426): lda = lambda_mult * lambda_sd +
  lambda_mean, hp = hab_pref_mult, the cut-off log(0.05) / -(lambda_mean +
  lambda_sd * lda); w(i, j) = area_j * lda * exp(pref_mean_j + pref_sd_j *
  hp), divided by exp(-lda d(i, j)) off the diagonal, each row normalised
  by its sum over the destinations within the cut-off.  The corrected
  semantics multiply by exp(-lda d) within log(20) / lda;
* computeSurvivalProbabilities (:428-451): surv_c(i, j) = exp(-crossings(i, j)
  * hazard_c), hazard_c = flow_c (vehicle width + animal length) / (speed
  3600), which the scenes carry precomputed.

The oracle's restatement (oracle/oracle.c) is what the GPU species kernels
are checked against to 1e-12; this pins it to the reference's own formulas.
"""
import math

import numpy as np
import pytest

from oracle import pyoracle as po
from transportoptimiser_gb300 import synth


def _scene():
    sc = synth.mte_road(0)
    sp = sc.species[0]
    # non-trivial variable parameters, so every term of the formulas counts
    sp.lambda_sd = 0.05
    sp.lambda_mult = 0.7
    sp.hab_pref_mult = 0.4
    for i, h in enumerate(sp.habitats):
        h.pref_sd = 0.1 * (i + 1)
    return sc, sp


@pytest.mark.parametrize("sem", [0, 1])
def test_distances_transitions_survival_follow_the_reference_formulas(sem):
    sc, sp = _scene()
    m = po.species_model(sc, sp, sc.roads[0], sem=sem)
    N = m["N"]
    cx, cy = m["cx"], m["cy"]
    d = np.sqrt((cx[:, None] - cx[None, :]) ** 2 + (cy[:, None] - cy[None, :]) ** 2)
    np.testing.assert_allclose(m["dists"], d, rtol=1e-14, atol=0)

    lda = sp.lambda_mult * sp.lambda_sd + sp.lambda_mean
    hp = sp.hab_pref_mult
    cut = (math.log(0.05) / -(sp.lambda_mean + sp.lambda_sd * lda)) if sem == 0 \
        else math.log(0.05) / -lda
    pref = np.array([sp.habitats[t].pref_mean + sp.habitats[t].pref_sd * hp for t in m["type"]])
    w = m["area"] * lda * np.exp(pref)                        # by destination
    trans = np.zeros((N, N))
    for i in range(N):
        row = np.zeros(N)
        inside = d[i] <= cut
        for j in np.nonzero(inside)[0]:
            if i == j:
                row[j] = w[j]
            elif sem == 0:
                row[j] = w[j] / math.exp(-lda * d[i, j])
            else:
                row[j] = w[j] * math.exp(-lda * d[i, j])
        trans[i] = row / math.fsum(row)
    np.testing.assert_allclose(m["trans"], trans, rtol=1e-13, atol=1e-300)
    assert (m["trans"] > 0).sum() == (trans > 0).sum()

    for c, hz in enumerate(sp.hazard):
        np.testing.assert_allclose(m["surv"][c], np.exp(-m["crossings"] * hz), rtol=1e-14)
    # the migration matrix is trans o surv_c in float, transposed to
    # destination-major, entries at or below 1e-5 dropped (dense2Sparse)
    for c in range(len(sp.hazard)):
        mm = (m["trans"] * m["surv"][c]).astype(np.float32)
        mm = np.where(mm.astype(np.float64) > 1e-5, mm, np.float32(0.0))
        assert np.array_equal(m["mmm"][c], mm.T)
