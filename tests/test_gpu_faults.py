"""Failure paths, made to fail from the host or by a bounded device wait
that runs out on a barrier with nothing in flight (to_ctx_inject_fault).
Nothing here faults, traps or hangs the GPU: the allocation failure is a
refused reservation on the host, and the wait gives up at once and takes the
kernel's abort path (error word, TMEM freed) before any copy or MMA is
issued.  After each, the same context values the same problem correctly."""
import numpy as np
import pytest

from oracle import pyoracle as po
from transportoptimiser_gb300 import _capi
from transportoptimiser_gb300 import simulate_gpu as sg
from transportoptimiser_gb300 import synth
from transportoptimiser_gb300._capi import MIG_SPARSE_FP32, MIG_TC_3XTF32, TransOptError

pytestmark = pytest.mark.gpu

TO_ERR_ALLOC, TO_ERR_TIMEOUT = 3, 5
TO_FAULT_ALLOC, TO_FAULT_WAIT = 1, 2


def _problem():
    sc = synth.mte_road(0)
    sp = sc.species[0]
    return po.species_model(sc, sp, sc.roads[0], sem=0), sp.params


def _inject(ctx, fault):
    assert ctx.lib.to_ctx_inject_fault(ctx.handle, fault) == 0


def test_injected_allocation_failure_returns_alloc_and_context_survives(ctx):
    m, prm = _problem()
    want, _ = sg.simulateMTECUDA([m], [prm], 512, 20, seed=3, migration=MIG_SPARSE_FP32, ctx=ctx)
    _inject(ctx, TO_FAULT_ALLOC)
    with pytest.raises(TransOptError) as e:
        sg.simulateMTECUDA([m], [prm], 512, 20, seed=3, migration=MIG_SPARSE_FP32, ctx=ctx)
    assert e.value.status == TO_ERR_ALLOC
    got, _ = sg.simulateMTECUDA([m], [prm], 512, 20, seed=3, migration=MIG_SPARSE_FP32, ctx=ctx)
    assert np.array_equal(got, want)


def test_injected_wait_timeout_returns_timeout_and_context_survives(ctx):
    m, prm = _problem()
    want, _ = sg.simulateMTECUDA([m], [prm], 256, 10, seed=4, migration=MIG_TC_3XTF32, ctx=ctx)
    _inject(ctx, TO_FAULT_WAIT)
    with pytest.raises(TransOptError) as e:
        sg.simulateMTECUDA([m], [prm], 256, 10, seed=4, migration=MIG_TC_3XTF32, ctx=ctx)
    assert e.value.status == TO_ERR_TIMEOUT
    # the error word was cleared, TMEM was freed: the kernel runs again
    got, _ = sg.simulateMTECUDA([m], [prm], 256, 10, seed=4, migration=MIG_TC_3XTF32, ctx=ctx)
    assert np.array_equal(got, want)
    assert ctx.lib.to_ctx_inject_fault(ctx.handle, 7) == 1      # unknown fault: TO_ERR_INVALID
