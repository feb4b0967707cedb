"""LGN->V1 plasticity (learning 1-4): the library against the oracle's restatement.

The oracle restates the learning block of compute_V_collect_spike_learnFF_fast
(src/coredynamics.cu:1631-1993) and the presynaptic trace of LGN_nonlinear
(src/discrete_input_convol.cu:1774-1808); it replays the GPU run on the recorded LGN uniforms.
While the rasters are identical, the weights, the post traces, the filtered rates, the
homeostasis totals and the presynaptic traces must agree to 1e-5 relative to each array's
largest magnitude (GPU and CPU expf differ by an ulp; every step adds a few such roundings).
"""
import numpy as np
import pytest

STEPS = 240


def _learning(**kw):
    from visual_cortex_gb300.model import FFLearning
    base = dict(tauLTP=16.8, tauLTD=33.7, tauTrip=114.0, tauAvg=1000.0, targetFR=0.0, A_LGN=0.02, r_LTD=1.0,
                gmaxLGN=0.6, gminLGN=0.0, sRatioLGN=1.0, decayTimeHomeoFF=250.0, FF_InfRatio=1.0, applyHomeo=0)
    base.update(kw)
    return FFLearning(**base)


def _rel(a, b):
    a = np.asarray(a, np.float64)
    b = np.asarray(b, np.float64)
    return float(np.max(np.abs(a - b)) / max(np.max(np.abs(b)), 1e-30))


def test_oracle_learning_keeps_weights_in_bounds_and_totals():
    """CPU: with multiplicative homeostasis the total each neuron carries stays the sum of its
    current LGN weights (the homeostatic factor moves the sum to the new total, the learning
    and the clipping add their changes to both), and the weights stay within [gmin, gmax]."""
    from oracle import LgnOracle, V1Oracle
    from visual_cortex_gb300 import synth
    wl = synth.config1(seed=2)
    L = _learning(applyHomeo=1, gmaxLGN=0.5)
    lo = LgnOracle(wl.lgn, wl.stim)
    lo.spatial()
    vo = V1Oracle(wl.spec, wl.net)
    vo.set_state(wl.init)
    vo.set_ff_learning(L)
    s0 = vo.get("sLGN").copy()
    rng = np.random.default_rng(0)
    for it in range(120):
        s, _, _ = lo.nonlinear(lo.convol(it), rng.random((wl.lgn.nLGN, 8)).astype(np.float32), None, 8)
        a, b = lo.ff_pre(L.tauLTP)
        vo.step(s)
        vo.learn_ff(s, a, b)
    s1 = vo.get("sLGN")
    tot = vo.get("total_ff").reshape(2, -1)
    assert np.abs(s1 - s0).max() > 1e-4
    assert s1.min() >= 0 and s1.max() <= 0.5 + 1e-7
    E = np.arange(wl.spec.nV1) % wl.spec.blockSize < wl.spec.nE
    sums = s1.reshape(-1, wl.spec.nV1).sum(axis=0, dtype=np.float64)
    np.testing.assert_allclose(tot[0][E], sums[E], rtol=1e-4)
    vo.close()


@pytest.mark.gpu
@pytest.mark.parametrize("homeo,targetFR", [(0, 0.0), (1, 2.0), (2, 0.0)])
def test_ff_learning_parity(native, homeo, targetFR):
    from oracle.parity import run_parity, compare
    from visual_cortex_gb300 import synth
    wl = synth.config1(seed=5 + homeo)
    L = _learning(applyHomeo=homeo, targetFR=targetFR, FF_InfRatio=0.9 if homeo else 1.0)
    res = run_parity(wl, STEPS, cap=8, learning=L)
    cmp = compare(res, wl.spec)
    div = cmp["first_raster_divergence"]
    if div is not None:
        # compare the learning state over the steps both rasters share
        assert div >= 100 and cmp["divergence_is_knife_edge"], cmp
        res = run_parity(wl, div, cap=8, learning=L)
        cmp = compare(res, wl.spec)
        assert cmp["first_raster_divergence"] is None, cmp
    assert res["draw_count_mismatch"] == 0
    assert cmp["lgn_spike_mismatch"] == 0, cmp
    assert cmp["v1_spikes_gpu"] > 50, cmp
    g, o = res["gpu"]["learn"], res["ora"]["learn"]
    s0 = wl.net.sLGN.astype(np.float64)
    assert np.abs(g["sLGN"].reshape(s0.shape) - s0).max() > 1e-3 * s0.max(), "the weights did not learn"
    for k in ("sLGN", "ff_post", "ff_pre") + (("total_ff",) if homeo else ()):
        assert _rel(g[k], o[k]) < 1e-5, (k, _rel(g[k], o[k]))
    for k in ("v", "gE", "gI", "gFF"):
        assert cmp[f"max_rel_{k}"] < 1e-5, cmp


def _learning_mode(mode):
    """learning 1: FF->E with the excitatory filtered rate advanced in the delivery (a cortical
    E type's tauAvg); 2: FF->E and FF->I (own constants, targetFR_I > 0), additive
    homeostasis; 4: the cortical filtered rate alone.  The FF->E targetFR stays 0: with
    learning != 3 vAvgE sums floor(membrane potential) every step, and its square in the LTD
    would clip every weight at once and leave totals made of rounding."""
    kw = dict(learning=mode, tauAvgCortical=700.0)
    if mode == 1:
        kw.update(applyHomeo=1, FF_InfRatio=0.9)
    if mode == 2:
        kw.update(applyHomeo=2, nLearnTypeFF_I=1, tauLTP_I=20.0, tauLTD_I=40.0, tauTrip_I=90.0, tauAvg_I=800.0,
                  targetFR_I=5.0, A_LGN_I=0.015, r_LTD_I=0.8, gmaxLGN_I=0.8, gminLGN_I=0.0, sRatioLGN_I=1.2)
    return _learning(**kw)


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [1, 2, 4])
def test_ff_learning_modes_parity(native, mode):
    """learning 1, 2 and 4 (src/coredynamics.cu:1631-1993 and the filtered-rate update of
    recal_G_mat_nd_fast, src/coredynamics.cu:2326-2346): the weights, the E (and with learning 2
    the I) post traces and filtered rates, and the presynaptic traces of each FF type as the
    oracle has them; with learning 4 the LGN->V1 weights do not move."""
    from oracle.parity import run_parity, compare
    from visual_cortex_gb300 import synth
    wl = synth.config1(seed=11 + mode)
    L = _learning_mode(mode)
    res = run_parity(wl, STEPS, cap=8, learning=L)
    cmp = compare(res, wl.spec)
    div = cmp["first_raster_divergence"]
    if div is not None:
        assert div >= 100 and cmp["divergence_is_knife_edge"], cmp
        res = run_parity(wl, div, cap=8, learning=L)
        cmp = compare(res, wl.spec)
        assert cmp["first_raster_divergence"] is None, cmp
    assert res["draw_count_mismatch"] == 0
    assert cmp["lgn_spike_mismatch"] == 0, cmp
    g, o = res["gpu"]["learn"], res["ora"]["learn"]
    s0 = wl.net.sLGN.astype(np.float32)
    if mode == 4:
        np.testing.assert_array_equal(g["sLGN"].reshape(s0.shape), s0)
        assert g["ff_pre"].size == 0
    else:
        assert np.abs(g["sLGN"].reshape(s0.shape) - s0).max() > 1e-3 * s0.max(), "the weights did not learn"
    if mode == 2:
        n = wl.spec.nV1
        inh = np.arange(n) % wl.spec.blockSize >= wl.spec.nE
        d = np.abs(g["sLGN"].reshape(-1, n) - s0.reshape(-1, n))[:, inh]
        assert d.max() > 1e-3 * s0.max(), "the FF->I weights did not learn"
        assert g["ff_pre"].size == 2 * wl.lgn.nLGN
    keys = ("sLGN",) + (("ff_pre", "total_ff") if mode != 4 else ())
    for k in keys:
        assert _rel(g[k], o[k]) < 1e-5, (k, _rel(g[k], o[k]))
    # the post block: traces within 1e-5; vAvgE adds floor(spike word) each step (the membrane
    # potential when the neuron did not spike), so it is compared with the steps at which the
    # two sides' words floor to different integers accounted for
    from oracle.parity import avg_floor_flips, compare_avg, split_record
    nEt, nIt = wl.spec.nE * wl.spec.nblock, wl.spec.nI * wl.spec.nblock
    a0 = g["ff_post"].size - 2 * nEt - nIt
    gp, op = g["ff_post"], o["ff_post"]
    if a0:
        assert _rel(gp[:a0], op[:a0]) < 1e-5
    if mode == 2:
        assert _rel(gp[a0 + 2 * nEt:], op[a0 + 2 * nEt:]) < 1e-5
    steps = res["gpu"]["raw"].shape[0]
    flips = avg_floor_flips(wl.spec, split_record(wl.spec, res["gpu"]["raw"])["sInfo"][:steps],
                            split_record(wl.spec, res["ora"]["raw"])["sInfo"][:steps])
    assert (flips > 0).sum() <= 0.01 * nEt
    assert compare_avg(gp[a0:a0 + 2 * nEt], op[a0:a0 + 2 * nEt], flips) < 1e-5
    assert np.abs(gp[a0:a0 + 2 * nEt]).max() > 0, "the filtered rates did not move"
    for k in ("v", "gE", "gI", "gFF"):
        assert cmp[f"max_rel_{k}"] < 1e-5, cmp


@pytest.mark.gpu
def test_ff_learning_checkpoint_resume_bitwise(native):
    """The learning state travels in the checkpoint: a plan restored after 120 steps runs the
    next 120 exactly as the plan that saved it and one that never stopped."""
    from visual_cortex_gb300 import _native as N
    from visual_cortex_gb300 import synth
    from visual_cortex_gb300.model import Simulation
    wl = synth.config1(seed=9)
    L = _learning(applyHomeo=1)
    sims = [Simulation(wl.spec, wl.net, wl.lgn, wl.stim, wl.init, wl.seeds) for _ in range(3)]
    a, b, c = sims
    try:
        for s in sims:
            s.set_ff_learning(L)
            s.set_record(N.REC_SPIKES, 241)
        a.run(120)
        ck = a.checkpoint()
        a.run(120)
        b.restore(ck)
        b.run(120)
        c.run(240)
        np.testing.assert_array_equal(a.fetch_spikes(120, 120), b.fetch_spikes(120, 120))
        np.testing.assert_array_equal(a.fetch_spikes(120, 120), c.fetch_spikes(120, 120))
        for k in ("sLGN", "ff_post", "ff_pre", "total_ff"):
            np.testing.assert_array_equal(a.state(k), b.state(k), err_msg=k)
            np.testing.assert_array_equal(a.state(k), c.state(k), err_msg=k)
    finally:
        for s in sims:
            s.close()


@pytest.mark.gpu
def test_ff_learning_modes_refused(native):
    """Learning modes outside 1-4, FF type counts the reference does not allow, and the
    persistent kernel with plasticity are refused loudly."""
    from visual_cortex_gb300 import synth
    from visual_cortex_gb300.model import Simulation
    wl = synth.config1(seed=1)
    sim = Simulation(wl.spec, wl.net, wl.lgn, wl.stim, wl.init, wl.seeds)
    try:
        with pytest.raises(RuntimeError, match="learning is 1, 2, 3 or 4"):
            sim.set_ff_learning(_learning(learning=5))
        with pytest.raises(RuntimeError, match="nLearnTypeFF_E"):
            sim.set_ff_learning(_learning(learning=1, nLearnTypeFF_E=0))
        with pytest.raises(RuntimeError, match="nLearnTypeFF_I"):
            sim.set_ff_learning(_learning(learning=2, nLearnTypeFF_I=2))
        sim.set_ff_learning(_learning())
        assert not sim.persistent()
    finally:
        sim.close()
