"""Bounded device-side waits: a barrier wait that runs out returns an error status.

The persistent V1 kernel separates consecutive steps by a grid barrier whose waits poll a
counter a bounded number of times (pv1_set_wait_limit).  With the limit at 0 polls the CTAs
that are not the last to arrive give up at the first barrier: they raise the barrier bit of
the error word and the abort bit of the counter, every other CTA is released, the kernel
returns, and the run reports PV1_E_DEVICE -- no trap and no hang.  The GPU context stays
usable: a new plan on the same device runs normally afterwards.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def test_barrier_wait_that_runs_out_returns_an_error(native):
    from visual_cortex_gb300 import synth
    from visual_cortex_gb300.model import Simulation
    wl = synth.make_workload("wait", seed=3, nblock=2, n_lgn=512, m=20, width=64, height=64, nt=256,
                             nFrame=40)
    a = Simulation(wl.spec, wl.net, wl.lgn, wl.stim, wl.init, wl.seeds)
    try:
        assert a.persistent(1)
        native.check(a.plan, native.lib.pv1_set_wait_limit(a.plan, 0), "pv1_set_wait_limit")
        rc = native.lib.pv1_run(a.plan, 256, 1)
        assert rc == -5                                    # PV1_E_DEVICE
        msg = native.lib.pv1_last_error(a.plan).decode()
        assert "barrier wait gave up" in msg, msg
    finally:
        a.close()
    # the context is still usable: a fresh plan runs the same steps with the default limit
    b = Simulation(wl.spec, wl.net, wl.lgn, wl.stim, wl.init, wl.seeds)
    try:
        assert b.persistent(1)
        b.run(256)
        assert np.isfinite(b.state("v")).all()
    finally:
        b.close()
