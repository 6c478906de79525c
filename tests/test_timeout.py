"""The bounded device waits: with wait_limit_us = 1 ms a persistent frame
whose grid barrier is one arrival short (sbs_gpu_withhold_barrier_arrival,
a wait that nothing satisfies - no fault, no trap) stops after the limit;
the next synchronising call reports SBS_ETIMEOUT, and the same handle then
steps normally again."""
import numpy as np
import pytest

from sbs_gb300 import scenes

pytestmark = pytest.mark.gpu


def test_withheld_arrival_times_out_and_the_handle_recovers(capi_mod):
    sc = scenes.beam_c1()
    g = capi_mod.Solver(sc, exec_mode=capi_mod.EXEC_PERSISTENT, wait_limit_us=1000)
    assert g.stats().exec_mode == capi_mod.EXEC_PERSISTENT
    g.step(2)
    x_before = g.positions()
    capi_mod.load().sbs_gpu_withhold_barrier_arrival(g.h)
    with pytest.raises(capi_mod.SbsError) as e:
        g.step_timed()
    assert e.value.status == capi_mod.SBS_ETIMEOUT
    # the frame stopped at its first grid barrier: nothing was projected
    assert np.array_equal(g.positions(), x_before)
    ms = g.step_timed()                       # the handle is usable again
    assert ms > 0.0
    x = g.positions()
    assert np.isfinite(x).all() and not np.array_equal(x, x_before)


def test_withhold_needs_the_persistent_mode(capi_mod):
    g = capi_mod.Solver(scenes.beam_c1(), exec_mode=capi_mod.EXEC_GRAPH)
    assert capi_mod.load().sbs_gpu_withhold_barrier_arrival(g.h) == capi_mod.SBS_ESTATE
