"""Allocation-free LGN stepping (pv1_lgn_spikes_noalloc) against the regular entry point.

pv1_lgn_spikes_noalloc is for callers that cannot allocate device memory when they step the
LGN stage: it keeps its scratch in a fixed device array of the library and writes into
buffers the caller provides.  Here the caller's buffers come from torch; the entry point is
called through the C ABI twice in a row and its spike words and rates are compared with the
LGN records of a plan stepped by pv1_run on the same seeds.  This file runs last so that a
run stopping at the first failure has run every other test first.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _fptr(t):
    return C.cast(C.c_void_p(t.data_ptr()), C.POINTER(C.c_float))


def test_noalloc_lgn_matches_regular_entry_point(native):
    import torch
    from visual_cortex_gb300 import synth
    from visual_cortex_gb300.model import Simulation

    wl = synth.config1(seed=11)
    nLGN = wl.lgn.nLGN
    K = 64
    ref = Simulation(wl.spec, wl.net, wl.lgn, wl.stim, wl.init, wl.seeds)
    noa = Simulation(wl.spec, wl.net, wl.lgn, wl.stim, wl.init, wl.seeds)
    try:
        ref.set_record(native.REC_LGN_SP | native.REC_LGN_FR, 2 * K + 1)
        ref.run(2 * K)
        _, sp_ref, fr_ref = ref.fetch_records(0, 2 * K, raw=False, lgn_sp=True, lgn_fr=True)

        outs = []
        for call in range(2):   # two calls in a row share (and reuse) the fixed scratch
            sp = torch.full((K, nLGN), -1.0, dtype=torch.float32, device="cuda")
            fr = torch.full((K, nLGN), -1.0, dtype=torch.float32, device="cuda")
            rc = native.lib.pv1_lgn_spikes_noalloc(noa.plan, K, _fptr(sp), _fptr(fr))
            native.check(noa.plan, rc, "pv1_lgn_spikes_noalloc")
            noa.state("lgn_lnl")        # waits for the plan's stream
            outs.append((sp.cpu().numpy(), fr.cpu().numpy()))
        sp_noa = np.concatenate([o[0] for o in outs])
        fr_noa = np.concatenate([o[1] for o in outs])
        np.testing.assert_allclose(sp_noa, sp_ref, rtol=1e-5, atol=0)
        np.testing.assert_allclose(fr_noa, fr_ref, rtol=1e-5, atol=0)
        assert (sp_noa >= 1).sum() > 0
        np.testing.assert_array_equal(noa.state("lgn_lnl"), ref.state("lgn_lnl"))
    finally:
        ref.close()
        noa.close()


def test_noalloc_rejects_work_beyond_its_scratch(native):
    from visual_cortex_gb300 import synth
    from visual_cortex_gb300.model import Simulation
    import torch

    wl = synth.config1(seed=12)
    sim = Simulation(wl.spec, wl.net, wl.lgn, wl.stim, wl.init, wl.seeds)
    try:
        too_many = (1 << 20) // wl.lgn.nLGN + 1
        buf = torch.zeros(16, dtype=torch.float32, device="cuda")
        rc = native.lib.pv1_lgn_spikes_noalloc(sim.plan, too_many, _fptr(buf), None)
        assert rc == -1
        assert "exceeds the fixed scratch" in native.lib.pv1_last_error(sim.plan).decode()
    finally:
        sim.close()


def test_noalloc_limits_and_lgn_only_plans(native):
    """At most 65535 steps per call; a plan stepped by this entry point is refused by pv1_run
    and by checkpoints, and a plan stepped by pv1_run is refused here."""
    import torch
    from visual_cortex_gb300 import synth
    from visual_cortex_gb300.model import Simulation

    wl = synth.config1(seed=13)
    a = Simulation(wl.spec, wl.net, wl.lgn, wl.stim, wl.init, wl.seeds)
    b = Simulation(wl.spec, wl.net, wl.lgn, wl.stim, wl.init, wl.seeds)
    try:
        buf = torch.zeros((4, wl.lgn.nLGN), dtype=torch.float32, device="cuda")
        rc = native.lib.pv1_lgn_spikes_noalloc(a.plan, 65536, _fptr(buf), None)
        assert rc == -1
        assert "65535" in native.lib.pv1_last_error(a.plan).decode()
        native.check(a.plan, native.lib.pv1_lgn_spikes_noalloc(a.plan, 4, _fptr(buf), None), "noalloc")
        assert native.lib.pv1_run(a.plan, 1, 1) == -3
        assert "LGN only" in native.lib.pv1_last_error(a.plan).decode()
        n = C.c_uint64()
        native.check(a.plan, native.lib.pv1_checkpoint_size(a.plan, C.byref(n)), "size")
        host = np.zeros(n.value, dtype=np.uint8)
        assert native.lib.pv1_checkpoint_save(a.plan, host.ctypes.data_as(C.c_void_p), n.value) == -3

        b.run(4)
        rc = native.lib.pv1_lgn_spikes_noalloc(b.plan, 4, _fptr(buf), None)
        assert rc == -3
        assert "stepped by pv1_run" in native.lib.pv1_last_error(b.plan).decode()
    finally:
        a.close()
        b.close()
