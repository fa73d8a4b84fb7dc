"""to_simulate_mte_noalloc_d: MTE statistics for callers that cannot
allocate device memory (a host program whose pool allocator owns the whole
device, or a GA loop that must not add allocations and the synchronisation
they bring).  The caller passes every input and output in its own device
memory; the per-path scratch lives in a fixed array inside the library.

Checked through the C ABI against the allocating entry point
(to_simulate_mte) on the same inputs, on two calls in a row, with the same
exact-equality tolerance as the other SIMT MTE tests.  Collected last."""
import ctypes as C

import numpy as np
import pytest

from oracle import pyoracle as po
from transportoptimiser_gb300 import _capi
from transportoptimiser_gb300 import simulate_gpu as sg
from transportoptimiser_gb300 import synth

pytestmark = pytest.mark.gpu


def _device_problem(torch, models, params, P, Y, seed, road, sem):
    S = len(models)
    NP = (max(int(m["N"]) for m in models) + 3) & ~3
    n = np.array([int(m["N"]) for m in models], np.int32)
    prm = np.zeros((S, 8), np.float32)
    ip = np.zeros((S, NP), np.float32)
    cp = np.ones((S, NP), np.float32)
    mm = np.zeros((S, NP, NP), np.float32)
    for s, m in enumerate(models):
        N = int(m["N"])
        prm[s] = params[s]
        ip[s, :N] = m["init_pops"]
        cp[s, :N] = m["caps"]
        mm[s, :N, :N] = m["mmm"][-1]
    dev = [torch.from_numpy(x).cuda() for x in (n, prm, ip, cp, mm)]
    prob = _capi.MteDeviceProblem(S, P, Y, NP, 1.0, seed, road, sem,
                                  *[t.data_ptr() for t in dev])
    return prob, dev


def test_noalloc_matches_allocating_entry_point(ctx):
    torch = pytest.importorskip("torch")
    lib = _capi.load()
    sc = synth.rov_road(0, n_species=2)
    models = [po.species_model(sc, sc.species[s], sc.roads[0], sem=0) for s in range(2)]
    params = [sc.species[s].params for s in range(2)]
    stream = torch.cuda.current_stream()
    for seed, P, Y, sem in ((1, 700, 30, 0), (2, 333, 50, 1)):
        prob, keep = _device_problem(torch, models, params, P, Y, seed, 5, sem)
        d_stats = torch.full((2 * 5,), -1.0, dtype=torch.float64, device="cuda")
        st = lib.to_simulate_mte_noalloc_d(C.c_void_p(stream.cuda_stream), C.byref(prob),
                                           C.c_void_p(d_stats.data_ptr()))
        assert st == 0
        torch.cuda.synchronize()
        got = d_stats.cpu().numpy().reshape(2, 5)
        _, want = sg.simulateMTECUDA(models, params, P, Y, seed=seed, road=5, sem=sem,
                                     migration=_capi.MIG_SIMT_FP32, ctx=ctx)
        for s in range(2):
            exp = [want[s][k] for k in ("mean", "sd", "se", "p_below", "init_total")]
            assert list(got[s]) == exp, (seed, s, got[s], exp)


def test_noalloc_rejects_oversized_problem(ctx):
    torch = pytest.importorskip("torch")
    lib = _capi.load()
    sc = synth.mte_road(0)
    m = po.species_model(sc, sc.species[0], sc.roads[0], sem=0)
    prob, keep = _device_problem(torch, [m], [sc.species[0].params], (1 << 21) + 1, 5, 0, 0, 0)
    d_stats = torch.zeros(5, dtype=torch.float64, device="cuda")
    st = lib.to_simulate_mte_noalloc_d(None, C.byref(prob), C.c_void_p(d_stats.data_ptr()))
    assert st == 6          # TO_ERR_UNSUPPORTED, nothing launched


def test_noalloc_patch_count_above_npad_gives_nan_statistics(ctx):
    """n_patches lives in the caller's device memory, so only the kernels can
    see that it exceeds npad: that species' statistics are NaN (nothing is
    read past its rows), the call returns TO_OK, and the other species are
    unaffected."""
    torch = pytest.importorskip("torch")
    lib = _capi.load()
    sc = synth.rov_road(0, n_species=2)
    models = [po.species_model(sc, sc.species[s], sc.roads[0], sem=0) for s in range(2)]
    params = [sc.species[s].params for s in range(2)]
    P, Y = 256, 20
    prob, keep = _device_problem(torch, models, params, P, Y, 3, 7, 0)
    n_dev = keep[0]
    n_dev[1] = prob.npad + 4          # the last species claims more patches than its rows hold
    torch.cuda.synchronize()
    d_stats = torch.zeros(2 * 5, dtype=torch.float64, device="cuda")
    st = lib.to_simulate_mte_noalloc_d(None, C.byref(prob), C.c_void_p(d_stats.data_ptr()))
    assert st == 0
    torch.cuda.synchronize()
    got = d_stats.cpu().numpy().reshape(2, 5)
    assert np.isnan(got[1]).all(), got[1]
    _, want = sg.simulateMTECUDA(models, params, P, Y, seed=3, road=7, sem=0,
                                 migration=_capi.MIG_SIMT_FP32, ctx=ctx)
    exp = [want[0][k] for k in ("mean", "sd", "se", "p_below", "init_total")]
    assert list(got[0]) == exp
