"""The oracle and the library held to the reference's OWN GPU kernels.

tests/golden/ref_kernels.npz holds what the reference's kernels -- logRand_init,
LGN_nonlinear, rand_spInit, compute_V_collect_spike_learnFF_fast and recal_G_mat_nd_fast,
compiled from its sources (oracle/ref/build_ref_kernels.sh) and launched as its step loop
launches them (oracle/ref/ref_kernel_runner.cu) -- computed on a GB300 for the seeded cases of
oracle/ref_cases.py (tests/golden/make_ref_kernel_golden.py).

CPU tests: the oracle replays the same cases and must reproduce those outputs.  GPU tests:
the library's own kernels must reproduce them -- generator states byte for byte (RNG indexing
bit-exact), and the V1 steps spike for spike with traces within 1e-5.
"""
import ctypes as C
import os

import numpy as np
import pytest

from oracle import ref_cases as RC

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_kernels.npz")
f32 = np.float32


@pytest.fixture(scope="module")
def gold():
    return dict(np.load(GOLD))


def _lgn_cfg(n, convolRatio, frRatio, dt):
    from visual_cortex_gb300 import _native as N
    c = N.LgnConfig()
    c.nLGN, c.convolRatio, c.frRatio, c.dt = n, convolRatio, frRatio, dt
    return c


def test_oracle_lgn_nonlinear_matches_reference_kernel(gold):
    """48 steps of LGN_nonlinear (logistic rate, exact-time Poisson spikes with the carried
    rate integral) from the reference's logRand_init state, replayed by the oracle on the same
    uniforms: rates to 1e-6, the same spike counts, spike times and carried integrals to 1e-5
    relative (one spike time in this case differs by 6e-6 relative: CPU and GPU logf, and the
    reference's own build contracts multiply-adds)."""
    import oracle
    case = RC.lgn_case()
    n, K, NU = RC.LGN_N, RC.LGN_K, RC.LGN_NU
    L = oracle.lib()
    cfg = _lgn_cfg(n, 1.0, 80.0, 0.125)
    u0 = gold["lgn_u0"].reshape(n, NU)
    ltr = gold["lgn_ltr0"].copy()
    lnl = gold["lgn_lnl0"].copy()
    assert (ltr == 0).all()
    used = np.zeros(n, np.int64)
    conv = case["convol"].reshape(K, n)
    fr_ref = gold["lgn_fr"].reshape(K, n)
    si_ref = gold["lgn_sInfo"].reshape(K, n)
    cap = 8
    for k in range(K):
        u = np.zeros((n, cap), f32)
        for i in range(n):
            take = u0[i, used[i]:used[i] + cap]
            u[i, :take.size] = take
        si = np.zeros(n, f32)
        fr = np.zeros(n, f32)
        L.orc_lgn_nonlinear(C.byref(cfg), oracle.fp(conv[k]), oracle.fp(case["max_convol"]), oracle.fp(case["c50"]),
                            oracle.fp(case["sharpness"]), oracle.fp(case["a"]), oracle.fp(case["b"]), oracle.fp(ltr),
                            oracle.fp(lnl), oracle.fp(u), None, cap, oracle.fp(si), oracle.fp(fr))
        np.testing.assert_allclose(fr, fr_ref[k], rtol=1e-6, atol=1e-6)
        np.testing.assert_array_equal(np.floor(si), np.floor(si_ref[k]))
        np.testing.assert_allclose(si, si_ref[k], rtol=1e-5, atol=1e-6)
        used += np.floor(si).astype(np.int64)
        assert used.max() <= NU
    np.testing.assert_allclose(ltr, gold["lgn_ltr"], rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(lnl, gold["lgn_lnl"], rtol=1e-5, atol=1e-6)
    assert (si_ref >= 1).sum() > 200                      # the case really spikes
    np.testing.assert_array_equal(gold["lgn_surf"], gold["lgn_sInfo"])   # spike words on the surface


def test_oracle_magno_setup_and_convolution_match_reference_kernels(gold):
    """store_PM for magno cells (time-reversed L1-normalised temporal weights, DoG spatial
    weights, texture coordinates, maxConvol) and 400 steps of LGN_convol_magno over a grating
    movie in layered textures: the oracle's tables to 1e-5 (temporal weights relative to the
    cell's largest weight: the biphasic kernel cancels where it crosses zero), and its
    convolutions (spatial stage per frame with emulated bilinear texture reads, then the
    temporal contraction) as stated below."""
    from oracle import LgnOracle
    wl = RC.magno_workload()
    lo = LgnOracle(wl.lgn, wl.stim)
    nm, ns = wl.lgn.nMagno, wl.lgn.mSample1D ** 2
    TWr = gold["magno_TW"].reshape(lo.TW.shape)
    assert np.max(np.abs(lo.TW - TWr) / np.abs(TWr).max(axis=1, keepdims=True)) < 1e-5
    np.testing.assert_allclose(lo.SW, gold["magno_SW"].reshape(nm, ns), rtol=1e-5, atol=1e-7)
    np.testing.assert_allclose(lo.SC, gold["magno_SC"].reshape(2, nm, ns), rtol=1e-6, atol=1e-7)
    np.testing.assert_allclose(lo.maxConvol, gold["magno_maxConvol"], rtol=1e-5)
    lo.spatial()
    ref = gold["magno_convol"].reshape(-1, nm)
    err = np.zeros(nm)
    scale = np.abs(ref).max()
    for q, it in enumerate(range(0, RC.MAGNO_T, RC.MAGNO_STRIDE)):
        err = np.maximum(err, np.abs(lo.convol(it) - ref[q]) / scale)
    # relative to the largest convolution of the run: every cell within 1e-3, 99% of them
    # within 1e-5 (the oracle emulates the texture unit's bilinear weights; one cell whose
    # samples straddle the texture's centre column differs by 7e-4, the others by < 2e-6)
    assert err.max() < 1e-3, err.max()
    assert np.mean(err < 1e-5) >= 0.99, np.sort(err)[-5:]
    assert np.abs(ref[-1]).max() > 1e-2          # the movie has reached the kernels' peak


def _replay_v1(gold, upto=None):
    """The oracle's V1 steps (compute_V + near delivery, no noise, no failure) from the
    reference run's initial state on its LGN spike words."""
    import oracle
    wl = RC.v1_workload(sp=False, host_init=oracle.host_init_state)
    vo = oracle.V1Oracle(wl.spec, wl.net)
    for k in ("v", "w", "gFF", "hFF", "gE", "hE", "gI", "hI"):
        vo.put(k, gold["run_in_" + k])
    T = RC.V1_T if upto is None else upto
    lgn = gold["run_lgnSInfo"]
    n = wl.spec.nV1
    raster = np.zeros((T, n), f32)
    snaps = {}
    for it in range(T):
        vo.step(lgn[it])
        raster[it] = vo.get("sInfo")
        if (it + 1) % RC.V1_SNAP == 0:
            snaps[it + 1] = {k: vo.get(k) for k in ("v", "w", "tBack", "gFF", "gE", "gI")}
    vo.close()
    return wl, raster, snaps


def _compare_runs(spec, ref_raster, raster, gold, snaps, tag):
    """Rasters identical (a difference allowed only at a float-rounding threshold crossing,
    and not before 10 ms); up to the first difference: the membrane potential in every step's
    spike words (non-spikers) within 1e-5 relative, spike times within 5e-4 of a step (the
    interpolated crossing time amplifies ulp differences of v), and v, w, gFF, gE, gI within
    1e-5 relative and tBack within 1e-4 ms at every snapshot."""
    from oracle.parity import first_divergence, knife_edge
    T = ref_raster.shape[0]
    div = first_divergence(ref_raster, raster)
    if div is not None:
        assert knife_edge(spec, ref_raster, raster, div), (tag, div)
    upto = T if div is None else div
    assert upto >= 80, (tag, upto)
    sp = ref_raster[:upto] >= 1
    assert sp.sum() > 50, (tag, sp.sum())
    np.testing.assert_allclose(raster[:upto][sp], ref_raster[:upto][sp], rtol=0, atol=5e-4, err_msg=tag)
    ns = ~sp
    a, b = raster[:upto][ns].astype(np.float64), ref_raster[:upto][ns].astype(np.float64)
    assert np.max(np.abs(a - b) / np.maximum(np.abs(b), 1.0)) < 1e-5, tag
    checked = 0
    for step, st in snaps.items():
        if step > upto:
            continue
        for k in ("v", "w", "tBack", "gFF", "gE", "gI"):
            a, b = st[k].astype(np.float64), gold[f"run_{k}_{step}"].astype(np.float64)
            if k == "tBack":
                err, tol = np.max(np.abs(a - b)), 1e-4
            else:
                scale = np.maximum(np.abs(b), 1.0) if k in ("v", "w") else max(np.abs(b).max(), 1e-12)
                err, tol = np.max(np.abs(a - b) / scale), 1e-5
            assert err < tol, (tag, k, step, err)
        checked += 1
    assert checked >= 2, (tag, checked)


def test_oracle_v1_steps_match_reference_kernels(gold):
    """160 steps of the reference's compute_V_collect_spike_learnFF_fast + recal_G_mat_nd_fast
    (two blocks, near delivery within and across blocks, AdEx inhibitory neurons) on recorded
    LGN spike words: the oracle's rasters are identical (or part at a float-rounding threshold
    crossing after 10 ms) and its traces agree to 1e-5 before that (_compare_runs)."""
    wl, raster, snaps = _replay_v1(gold)
    ref = gold["run_raster"].reshape(RC.V1_T, wl.spec.nV1)
    _compare_runs(wl.spec, ref, raster, gold, snaps, "oracle")


@pytest.mark.gpu
def test_lgn_generators_match_reference(native, gold):
    """The library's LGN generators after setup are the reference's logRand_init states byte
    for byte (curand_init(seed, id, 0) per cell, one uniform discarded, the next one's -log as
    lastNegLogRand)."""
    from visual_cortex_gb300 import synth
    from visual_cortex_gb300.model import Simulation
    wl = synth.make_workload("lgn-rng", seed=RC.LGN_SEED, nblock=1, n_lgn=RC.LGN_N, nt=8, nFrame=8)
    assert wl.lgn.nLGN == RC.LGN_N and wl.seeds.lgn == RC.LGN_SEED
    sim = Simulation(wl.spec, wl.net, wl.lgn, wl.stim, wl.init, wl.seeds)
    try:
        np.testing.assert_array_equal(sim.state("lgn_rng"), gold["lgn_state0"])
        np.testing.assert_array_equal(sim.state("lgn_lnl"), gold["lgn_lnl0"])
        np.testing.assert_array_equal(sim.state("lgn_ltr"), gold["lgn_ltr0"])
    finally:
        sim.close()


@pytest.mark.gpu
@pytest.mark.parametrize("sp", [False, True])
def test_v1_initial_state_matches_reference(native, gold, sp):
    """rand_spInit: the library's rGenCond and rNoisy generators are the reference's byte for
    byte; with initial spikes (spE0/spI0 > 0) also the spike-word history, v, w and tBack."""
    from visual_cortex_gb300.model import InitState, Simulation
    wl = RC.v1_workload(sp=sp)
    tag = "init1_" if sp else "init0_"
    if sp:
        wl.init = InitState(**{k: gold["init1_in_" + k] for k in ("v", "w", "gFF", "hFF", "gE", "hE", "gI", "hI")})
    sim = Simulation(wl.spec, wl.net, wl.lgn, wl.stim, wl.init, wl.seeds, record_init=16 if sp else 0)
    try:
        np.testing.assert_array_equal(sim.state("v1_rng_cond"), gold[tag + "rGenCond"])
        np.testing.assert_array_equal(sim.state("v1_rng_noisy"), gold[tag + "rNoisy"])
        if sp:
            n, d = wl.spec.nV1, wl.seeds.trainDepth
            hist = sim.init_record["history"]
            np.testing.assert_array_equal(hist, gold["init1_spikeTrain"].reshape(d, n))
            np.testing.assert_array_equal(sim.state("v"), gold["init1_v"])
            np.testing.assert_allclose(sim.state("w"), gold["init1_w"], rtol=1e-6, atol=1e-7)
            np.testing.assert_array_equal(sim.state("tBack"), gold["init1_tBack"])
            assert (hist >= 1).sum() > 20
    finally:
        sim.close()


@pytest.mark.gpu
def test_library_v1_steps_match_reference_kernels(native, gold):
    """The library's own run of the workload: its LGN spike words are the ones the reference's
    V1 kernels were fed, and its V1 rasters and state match the reference's kernels as the
    oracle's do (identical rasters up to a float-rounding threshold crossing, state to 1e-5)."""
    from visual_cortex_gb300 import _native as N
    from visual_cortex_gb300.model import InitState, Simulation
    from oracle.parity import split_record
    wl = RC.v1_workload(sp=False)
    wl.init = InitState(**{k: gold["run_in_" + k] for k in ("v", "w", "gFF", "hFF", "gE", "hE", "gI", "hI")})
    T = RC.V1_T
    sim = Simulation(wl.spec, wl.net, wl.lgn, wl.stim, wl.init, wl.seeds)
    try:
        sim.set_record(N.REC_RAW | N.REC_LGN_SP, T + 1)
        snaps = {}
        raws, lsps = [], []
        for s0 in range(0, T, RC.V1_SNAP):
            sim.run(RC.V1_SNAP)
            raw, lsp, _ = sim.fetch_records(s0, RC.V1_SNAP, raw=True, lgn_sp=True, lgn_fr=False)
            raws.append(raw)
            lsps.append(lsp)
            snaps[s0 + RC.V1_SNAP] = {k: sim.state(k) for k in ("v", "w", "tBack", "gFF", "gE", "gI")}
        lsp = np.concatenate(lsps)
        np.testing.assert_array_equal(lsp, gold["run_lgnSInfo"])
        raster = split_record(wl.spec, np.concatenate(raws))["sInfo"]
    finally:
        sim.close()
    ref = gold["run_raster"].reshape(T, wl.spec.nV1)
    _compare_runs(wl.spec, ref, raster, gold, snaps, "library")


@pytest.mark.gpu
def test_library_magno_tables_and_rates_match_reference_kernels(native, gold):
    """The library's store_PM tables equal the reference's (1e-5), and its LGN firing rates
    over the 400 steps equal the logistic of the reference's LGN_convol_magno outputs (1e-4
    relative; the library contracts a per-frame spatial stage instead of re-walking the
    window, as a sum in another order)."""
    from visual_cortex_gb300 import _native as N
    from visual_cortex_gb300.model import Simulation
    import oracle
    wl = RC.magno_workload()
    nm, ns = wl.lgn.nMagno, wl.lgn.mSample1D ** 2
    sim = Simulation(wl.spec, wl.net, wl.lgn, wl.stim, wl.init, wl.seeds)
    try:
        TW, SW, SC, mc = sim.lgn_tables()
        sim.set_record(N.REC_LGN_FR, RC.MAGNO_T + 1)
        sim.run(RC.MAGNO_T)
        _, _, fr = sim.fetch_records(0, RC.MAGNO_T, raw=False, lgn_sp=False, lgn_fr=True)
    finally:
        sim.close()
    TWr = gold["magno_TW"].reshape(TW.shape)
    assert np.max(np.abs(TW - TWr) / np.abs(TWr).max(axis=1, keepdims=True)) < 1e-5
    np.testing.assert_allclose(SW, gold["magno_SW"].reshape(nm, ns), rtol=1e-5, atol=1e-7)
    np.testing.assert_allclose(SC, gold["magno_SC"].reshape(2, nm, ns), rtol=1e-6, atol=1e-7)
    np.testing.assert_allclose(mc, gold["magno_maxConvol"], rtol=1e-5)
    lo = oracle.LgnOracle(wl.lgn, wl.stim)
    ref = gold["magno_convol"].reshape(-1, nm)
    L = oracle.lib()
    for q, it in enumerate(range(0, RC.MAGNO_T, RC.MAGNO_STRIDE)):
        conv = np.zeros(wl.lgn.nLGN, f32)
        conv[wl.lgn.magno_ids()] = ref[q]
        want, _ = _rates(L, lo, conv)
        np.testing.assert_allclose(fr[it], want, rtol=1e-4, atol=1e-4)


def _rates(L, lo, conv):
    """LGN_nonlinear's logistic rate of given convolutions (the oracle's, no spikes kept)."""
    import oracle
    n = lo.lgn.nLGN
    si, fr = np.zeros(n, f32), np.zeros(n, f32)
    ltr, lnl = np.zeros(n, f32), np.full(n, 1e30, f32)
    L.orc_lgn_nonlinear(C.byref(lo.cfg), oracle.fp(conv), oracle.fp(lo.maxConvol), oracle.fp(lo.c50),
                        oracle.fp(lo.sharp), oracle.fp(lo.la), oracle.fp(lo.lb), oracle.fp(ltr), oracle.fp(lnl),
                        oracle.fp(np.zeros((n, 1), f32)), None, 1, oracle.fp(si), oracle.fp(fr))
    return fr, si


GOLD_LEARN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "ref_learning.npz")


@pytest.fixture(scope="module")
def gold_learn():
    return dict(np.load(GOLD_LEARN))


def test_oracle_lgn_trace_matches_reference_kernel(gold, gold_learn):
    """LGN_nonlinear with learning = 3 (src/discrete_input_convol.cu:1774-1808) on the LGN case:
    the oracle's presynaptic trace at the start of each step, right after each cell's spikes,
    and at the end of the step (lVar) within 1e-5 of the reference's over 48 steps."""
    import oracle
    case = RC.lgn_case()
    n, K, NU = RC.LGN_N, RC.LGN_K, RC.LGN_NU
    L = oracle.lib()
    cfg = _lgn_cfg(n, 1.0, 80.0, 0.125)
    tau = RC.learning_params().tauLTP
    u0 = gold["lgn_u0"].reshape(n, NU)
    ltr = gold["lgn_ltr0"].copy()
    lnl = gold["lgn_lnl0"].copy()
    used = np.zeros(n, np.int64)
    conv = case["convol"].reshape(K, n)
    var = np.zeros(n, f32)
    ref_end = gold_learn["lgn_ffvar"].reshape(K, n)
    ref_start = gold_learn["lgn_ffstart"].reshape(K, n)
    ref_spk = gold_learn["lgn_ffspk"].reshape(K, n)
    np.testing.assert_array_equal(gold_learn["lgn_sInfo"].reshape(K, n), gold["lgn_sInfo"].reshape(K, n))
    cap = 8
    spiked = 0
    for k in range(K):
        u = np.zeros((n, cap), f32)
        for i in range(n):
            take = u0[i, used[i]:used[i] + cap]
            u[i, :take.size] = take
        si, fr, tsp = np.zeros(n, f32), np.zeros(n, f32), np.zeros(n, f32)
        nsp = np.zeros(n, np.uint32)
        L.orc_lgn_nonlinear_ex(C.byref(cfg), oracle.fp(conv[k]), oracle.fp(case["max_convol"]), oracle.fp(case["c50"]),
                               oracle.fp(case["sharpness"]), oracle.fp(case["a"]), oracle.fp(case["b"]), oracle.fp(ltr),
                               oracle.fp(lnl), oracle.fp(u), None, cap, oracle.fp(si), oracle.fp(fr), oracle.up(nsp),
                               oracle.fp(tsp))
        start, at = np.zeros(n, f32), np.zeros(n, f32)
        L.orc_lgn_ff_pre(n, f32(0.125), f32(tau), oracle.up(nsp), oracle.fp(tsp), oracle.fp(si), oracle.fp(var),
                         oracle.fp(start), oracle.fp(at))
        np.testing.assert_allclose(start, ref_start[k], rtol=1e-5, atol=1e-7)
        np.testing.assert_allclose(var, ref_end[k], rtol=1e-5, atol=1e-7)
        s = si > 0
        np.testing.assert_allclose(at[s], ref_spk[k][s], rtol=1e-5, atol=1e-7)
        spiked += int(s.sum())
        used += np.floor(si).astype(np.int64)
    assert spiked > 200 and ref_end.max() > 0.5


def test_oracle_v1_learning_matches_reference_kernels(gold_learn):
    """120 steps of the reference's compute_V_collect_spike_learnFF_fast with learning = 3
    (multiplicative homeostasis, targetFR > 0) + recal_G_mat_nd_fast on recorded LGN spike
    words and presynaptic traces: the oracle's rasters are identical, and the LGN->V1 weights,
    the post LTD and triplet traces, the filtered rates and the homeostasis totals agree to
    1e-5 of each array's largest value (the weights change by several percent)."""
    import oracle
    wl = RC.v1_workload(sp=False, host_init=oracle.host_init_state)
    g = gold_learn
    vo = oracle.V1Oracle(wl.spec, wl.net)
    for k in ("v", "w", "gFF", "hFF", "gE", "hE", "gI", "hI"):
        vo.put(k, g["v1_in_" + k])
    vo.set_ff_learning(RC.learning_params())
    T, n = RC.LEARN_T, wl.spec.nV1
    lgn = g["v1_lgnSInfo"]
    raster = np.zeros((T, n), f32)
    for it in range(T):
        vo.step(lgn[it])
        vo.learn_ff(lgn[it], np.ascontiguousarray(g["v1_preStart"][it]), np.ascontiguousarray(g["v1_preSpk"][it]))
        raster[it] = vo.get("sInfo")
    ref = g["v1_raster"].reshape(T, n)
    np.testing.assert_array_equal(raster >= 1, ref >= 1)
    assert (ref >= 1).sum() > 50
    s1 = vo.get("sLGN")
    rel = lambda a, b: float(np.max(np.abs(a.astype(np.float64) - b)) / np.max(np.abs(b)))
    assert rel(s1, g["v1_sLGN"]) < 1e-5
    assert np.abs(g["v1_sLGN"] - wl.net.sLGN.reshape(-1)).max() > 0.01 * wl.net.sLGN.max()
    post = vo.get("ff_post")
    nEt = wl.spec.nE * wl.spec.nblock
    assert rel(post[:nEt], g["v1_vLTD"]) < 1e-5
    assert rel(post[nEt:2 * nEt], g["v1_vTrip"]) < 1e-5
    assert rel(post[2 * nEt:4 * nEt], g["v1_vAvgE"]) < 1e-5
    assert rel(vo.get("total_ff")[:n], g["v1_totalFF"]) < 1e-5
    vo.close()


def test_oracle_v1_learning2_matches_reference_kernels(gold_learn):
    """The same 120 steps with learning = 2: an FF->I type beside the FF->E one (its own
    constants; the reference's inhibitory posts read presynaptic trace 0), additive homeostasis,
    and the excitatory filtered rate advanced by recal_G_mat_nd_fast with the cortical E type's
    tauAvg (src/coredynamics.cu:2326-2346).  Rasters identical; weights, the E and I post
    traces, both filtered rates and the totals within 1e-5 of each array's largest value."""
    import oracle
    wl = RC.v1_workload(sp=False, host_init=oracle.host_init_state)
    g = gold_learn
    L = RC.learning_params2()
    vo = oracle.V1Oracle(wl.spec, wl.net)
    for k in ("v", "w", "gFF", "hFF", "gE", "hE", "gI", "hI"):
        vo.put(k, g["v1_in_" + k])
    vo.set_ff_learning(L)
    T, n = RC.LEARN_T, wl.spec.nV1
    lgn = g["v1_lgnSInfo"]
    raster = np.zeros((T, n), f32)
    for it in range(T):
        vo.step(lgn[it])
        vo.learn_ff(lgn[it], np.ascontiguousarray(g["v1_preStart"][it]), np.ascontiguousarray(g["v1_preSpk"][it]))
        vo.learn_avg()
        raster[it] = vo.get("sInfo")
    ref = g["v2_raster"].reshape(T, n)
    np.testing.assert_array_equal(raster >= 1, ref >= 1)
    E = np.arange(n) % wl.spec.blockSize < wl.spec.nE
    assert (ref.reshape(T, n)[:, E] >= 1).sum() > 50 and (ref.reshape(T, n)[:, ~E] >= 1).sum() > 20
    rel = lambda a, b: float(np.max(np.abs(a.astype(np.float64) - b)) / np.max(np.abs(b)))
    s1 = vo.get("sLGN")
    assert rel(s1, g["v2_sLGN"]) < 1e-5
    s0 = wl.net.sLGN.reshape(-1, n)
    dI = np.abs(g["v2_sLGN"].reshape(-1, n) - s0)[:, ~E].max()
    assert dI > 0.01 * s0.max(), "the FF->I weights did not learn"
    post = vo.get("ff_post")
    nEt, nIt = wl.spec.nE * wl.spec.nblock, wl.spec.nI * wl.spec.nblock
    o = 2 * nEt
    for name, a, b in (("vLTD", 0, nEt), ("vTrip", nEt, 2 * nEt), ("vLTDi", o, o + nIt), ("vTripi", o + nIt, o + 2 * nIt),
                       ("vAvgI", o + 2 * nIt + 2 * nEt, post.size)):
        assert np.abs(g["v2_" + name]).max() > 0, name
        assert rel(post[a:b], g["v2_" + name]) < 1e-5, (name, rel(post[a:b], g["v2_" + name]))
    # vAvgE adds floor(spike word) every step -- the membrane potential when the neuron did not
    # spike -- so a potential within an ulp of an integer moves it by 1 on one side only
    from oracle.parity import avg_floor_flips, compare_avg
    flips = avg_floor_flips(wl.spec, raster, ref)
    assert (flips > 0).sum() <= 0.01 * nEt
    assert compare_avg(post[o + 2 * nIt:o + 2 * nIt + 2 * nEt], g["v2_vAvgE"], flips) < 1e-5
    assert rel(vo.get("total_ff")[:n], g["v2_totalFF"]) < 1e-5
    vo.close()


def test_oracle_v1_learning4_matches_reference_kernels(gold_learn):
    """The same 120 steps with learning = 4: the V1 kernel skips the FF learning block, so the
    LGN->V1 weights stay bit for bit and the spike-time slot of vAvgE stays 0; the delivery
    advances vAvgE with the cortical E type's tauAvg.  Rasters identical, vAvgE as in the
    learning = 2 case (floor flips counted)."""
    import oracle
    from oracle.parity import avg_floor_flips, compare_avg
    wl = RC.v1_workload(sp=False, host_init=oracle.host_init_state)
    g = gold_learn
    vo = oracle.V1Oracle(wl.spec, wl.net)
    for k in ("v", "w", "gFF", "hFF", "gE", "hE", "gI", "hI"):
        vo.put(k, g["v1_in_" + k])
    vo.set_ff_learning(RC.learning_params4())
    T, n = RC.LEARN_T, wl.spec.nV1
    lgn = g["v1_lgnSInfo"]
    raster = np.zeros((T, n), f32)
    for it in range(T):
        vo.step(lgn[it])
        vo.learn_avg()
        raster[it] = vo.get("sInfo")
    ref = g["v4_raster"].reshape(T, n)
    np.testing.assert_array_equal(raster >= 1, ref >= 1)
    assert (ref >= 1).sum() > 50
    np.testing.assert_array_equal(g["v4_sLGN"], wl.net.sLGN.reshape(-1))
    np.testing.assert_array_equal(vo.get("sLGN"), wl.net.sLGN.reshape(-1))
    nEt = wl.spec.nE * wl.spec.nblock
    post = vo.get("ff_post")
    assert post.size == 2 * nEt + wl.spec.nI * wl.spec.nblock
    flips = avg_floor_flips(wl.spec, raster, ref)
    assert (flips > 0).sum() <= 0.01 * nEt
    assert np.abs(g["v4_vAvgE"]).max() > 100
    assert compare_avg(post[:2 * nEt], g["v4_vAvgE"], flips) < 1e-5
    vo.close()
