"""Batched trials: every trial of a batch ends bit-identical to the same trial run alone."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

STATE = ("v", "w", "tBack", "gE", "hE", "gI", "hI", "gFF", "hFF", "lgn_lnl", "lgn_ltr")


def _trials(**kw):
    from visual_cortex_gb300 import synth
    args = dict(n_trials=4, nblock=2, n_lgn=512, width=64, height=64, nFrame=60, far_partners=50,
                dur_ms=(8.0, 25.0))
    args.update(kw)
    return synth.batch_trials(**args)


def _sim(wl):
    from visual_cortex_gb300.model import Simulation
    return Simulation(wl.spec, wl.net, wl.lgn, wl.stim, wl.init, wl.seeds)


@pytest.mark.parametrize("autotune", [False, True])
def test_batch_equals_trials_alone(native, autotune):
    from visual_cortex_gb300.batch import Batch
    trials = _trials()
    alone, batched = [], []
    try:
        for tr in trials:
            s = _sim(tr.wl)
            s.persistent(0)
            s.run(tr.steps)
            alone.append(s)
        batched = [_sim(tr.wl) for tr in trials]
        b = Batch(batched, [tr.steps for tr in trials], autotune=autotune)
        try:
            left, ms = b.run()
            assert left == 0 and ms > 0
            for q, tr in enumerate(trials):
                assert batched[q].step == tr.steps
                for k in STATE:
                    np.testing.assert_array_equal(batched[q].state(k), alone[q].state(k),
                                                  err_msg=f"trial {q} {k}")
                t, mean, rates = b.stats(q, rates=True)
                assert t == pytest.approx(tr.steps * tr.wl.spec.dt, rel=1e-12)
                assert mean == pytest.approx(rates.mean(), rel=1e-12)
        finally:
            b.close()
    finally:
        for s in alone + batched:
            s.close()


def test_batch_sweep_in_one_launch(native):
    """pv1_batch_sweep: the rest of every trial (uneven durations and sizes) as one graph of
    three launches -- the LGN stage of every remaining step, one cooperative V1 launch with the
    trials scheduled longest first on the slots, the advance -- after a chunked start; every
    trial ends bit-identical to the same trial run alone."""
    from visual_cortex_gb300.batch import Batch
    from visual_cortex_gb300 import synth
    trials = _trials(n_trials=5, dur_ms=(6.0, 30.0))
    big = synth.batch_trials(n_trials=1, seed=7, nblock=3, n_lgn=512, width=64, height=64, nFrame=60,
                             far_partners=50, dur_ms=(20.0, 20.0))
    trials = trials + big
    alone, batched = [], []
    try:
        for tr in trials:
            s = _sim(tr.wl)
            s.persistent(0)
            s.run(tr.steps)
            alone.append(s)
        batched = [_sim(tr.wl) for tr in trials]
        b = Batch(batched, [tr.steps for tr in trials], autotune=False)
        try:
            b.run(max_steps=20)
            ms = b.sweep()
            assert ms > 0 and b.launches() == 3
            for q, tr in enumerate(trials):
                assert batched[q].step == tr.steps
                for k in STATE:
                    np.testing.assert_array_equal(batched[q].state(k), alone[q].state(k),
                                                  err_msg=f"trial {q} {k}")
                t, mean, rates = b.stats(q, rates=True)
                assert t == pytest.approx(tr.steps * tr.wl.spec.dt, rel=1e-12)
            assert b.sweep() == 0.0
        finally:
            b.close()
    finally:
        for s in alone + batched:
            s.close()


def test_batch_in_pieces_with_noise(native):
    """maxSteps slices, a trial continuing after the batch, noise and failure draws."""
    from visual_cortex_gb300.batch import Batch
    from visual_cortex_gb300 import synth
    base = synth.make_workload("nz", seed=9, nblock=2, n_lgn=512, width=64, height=64, nt=0,
                               far_partners=50, adex_inh=True, nFrame=60, noisyDep=(0.2, 0.2),
                               synFailFF=(0.1, 0.1), synFail=(0.1, 0.1, 0.1, 0.1))
    # batched trials take no far synaptic failure (its host-engine path runs one plan at a time):
    # drop the far synapses for the failure case
    import dataclasses
    net = dataclasses.replace(base.net, nVec=np.zeros_like(base.net.nVec),
                              vecID=np.zeros(0, np.uint32), conVec=np.zeros(0, np.float32),
                              delayVec=np.zeros(0, np.float32))
    base = dataclasses.replace(base, net=net)
    trials = _trials(n_trials=3, base=base, dur_ms=(10.0, 20.0))
    alone, batched = [], []
    try:
        for tr in trials:
            s = _sim(tr.wl)
            s.persistent(0)
            s.run(tr.steps + 30)
            alone.append(s)
        batched = [_sim(tr.wl) for tr in trials]
        b = Batch(batched, [tr.steps for tr in trials], autotune=False)
        try:
            while b.run(max_steps=37)[0] > 0:
                pass
        finally:
            b.close()
        for q, tr in enumerate(trials):
            batched[q].run(30)      # the plan continues on its own after the batch
            for k in STATE:
                np.testing.assert_array_equal(batched[q].state(k), alone[q].state(k),
                                              err_msg=f"trial {q} {k}")
    finally:
        for s in alone + batched:
            s.close()


def test_batch_uneven_sizes_persistent(native):
    """Trials of 2 and 1 blocks in one batch: the persistent variant's slots are sized for the
    larger trial, the smaller one leaves CTAs idle; every trial still ends as it does alone."""
    from visual_cortex_gb300.batch import Batch
    big = _trials(n_trials=2, dur_ms=(10.0, 16.0))
    small = _trials(n_trials=2, nblock=1, far_partners=0, dur_ms=(12.0, 18.0), seed=5)
    trials = [big[0], small[0], big[1], small[1]]
    alone, batched = [], []
    try:
        for tr in trials:
            s = _sim(tr.wl)
            s.persistent(0)
            s.run(tr.steps)
            alone.append(s)
        batched = [_sim(tr.wl) for tr in trials]
        b = Batch(batched, [tr.steps for tr in trials], autotune=False)
        try:
            assert b.tuning()["variant"] == "persistent"
            assert b.run()[0] == 0
            for q in range(len(trials)):
                for k in STATE:
                    np.testing.assert_array_equal(batched[q].state(k), alone[q].state(k),
                                                  err_msg=f"trial {q} {k}")
        finally:
            b.close()
    finally:
        for s in alone + batched:
            s.close()


def test_batch_parvo_and_multi_spike_trials(native):
    """Trials whose LGN has parvo cells (per-trial LGN launches instead of the batched class
    kernel) and trials in the multi-spike regime (dt > min tRef) batch like any other."""
    from visual_cortex_gb300.batch import Batch
    from visual_cortex_gb300 import synth
    parvo = synth.make_workload("parvo", seed=9, nblock=1, n_lgn=256, m=20, width=64, height=64, nt=0,
                                nFrame=40, n_parvo=64, tau=300.0, nKernelSample=150)
    multi = synth.make_workload("multi", seed=11, nblock=1, n_lgn=256, m=20, width=64, height=64, nt=0,
                                nFrame=40)
    multi.spec.tRef = [0.1, 0.05]
    trials = [synth.Trial(wl=parvo, steps=120, orient=0.0, contrast=0.5),
              synth.Trial(wl=multi, steps=100, orient=0.0, contrast=0.5),
              synth.Trial(wl=parvo, steps=90, orient=0.0, contrast=0.5)]
    alone, batched = [], []
    try:
        for tr in trials:
            s = _sim(tr.wl)
            s.persistent(0)
            s.run(tr.steps)
            alone.append(s)
        batched = [_sim(tr.wl) for tr in trials]
        b = Batch(batched, [tr.steps for tr in trials], autotune=True)
        try:
            assert b.run()[0] == 0
            for q in range(len(trials)):
                for k in STATE:
                    np.testing.assert_array_equal(batched[q].state(k), alone[q].state(k),
                                                  err_msg=f"trial {q} {k}")
        finally:
            b.close()
    finally:
        for s in alone + batched:
            s.close()
