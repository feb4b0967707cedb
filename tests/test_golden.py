"""The oracle against golden vectors computed by the reference's own code.

tests/golden/ref_golden.npz holds inputs and the outputs of the reference's ConductanceShape,
AdEx struct, hStatic_nonlinear, find_denorm and fill_fSpikeTrain + recal_G_vec, compiled on
the host from its sources (oracle/ref/build_ref.sh, tests/golden/make_golden.py).  The
oracle's restatements must reproduce them bit for bit (same float operations, same order).
"""
import ctypes as C
import os

import numpy as np
import pytest

GOLD = os.path.join(os.path.dirname(__file__), "golden", "ref_golden.npz")
f32 = np.float32


@pytest.fixture(scope="module")
def gold():
    return np.load(GOLD)


@pytest.fixture(scope="module")
def L():
    import oracle
    return oracle.lib()


def fp(a):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def test_conductance_shape(gold, L):
    x, y = gold["cond_in"], gold["cond_out"]
    out = np.empty(4, f32)
    got = np.empty_like(y)
    for q in range(x.shape[0]):
        L.orc_cond_eval(*[float(v) for v in x[q]], fp(out))
        got[q] = out
    np.testing.assert_array_equal(got, y)


def test_adex_step(gold, L):
    """Tonic drive (constructor), set_p0/set_p1 + rk2 and compute_spike_time."""
    x, y = gold["adex_in"], gold["adex_out"]
    vE, vI, vL = 0.0, -75.0, -65.0        # the reference's compile-time reversal potentials
    v, w = C.c_float(), C.c_float()
    ratio, w0 = C.c_float(), C.c_float()
    for q in range(x.shape[0]):
        (w_0, tau_w, a, b, v0, vR, vThres, gL, Cm, tRef, vT, deltaT, dep, gE0, gI0, gE1, gI1, dt) = \
            [float(t) for t in x[q]]
        depC = L.orc_adex_depc(vL, vT, gL, a, deltaT, dep)
        assert np.float32(depC) == y[q, 0], q
        L.orc_adex_rk2(vE, vI, vL, gE0, gI0, gE1, gI1, depC, gL, vT, deltaT, Cm, a, tau_w, v0, w_0, dt,
                       0.0, 0.0, C.byref(v), C.byref(w))
        assert (np.float32(v.value), np.float32(w.value)) == (y[q, 1], y[q, 2]), q
        w0.value = w_0
        L.orc_adex_spike(vThres, v0, v.value, w.value, b, C.byref(ratio), C.byref(w0))
        # compute_spike_time with t0 = 0: tsp = ratio * dt
        assert np.float32(np.float32(ratio.value) * np.float32(dt)) == y[q, 3], q
        assert np.float32(w0.value) == y[q, 4], q


def test_logistic_parameters(gold, L):
    spont, c50, sharp = [np.ascontiguousarray(r, f32) for r in gold["logistic_in"]]
    n = spont.size
    a, b = np.empty(n, f32), np.empty(n, f32)
    L.orc_logistic_ab(fp(spont), fp(c50), fp(sharp), n, fp(a), fp(b))
    np.testing.assert_array_equal(a, gold["logistic_out"][0])
    np.testing.assert_array_equal(b, gold["logistic_out"][1])


def test_find_denorm(gold):
    from visual_cortex_gb300.schedule import find_denorm
    for (u1, u2, morn), (d, nrm) in zip(gold["denorm_in"], gold["denorm_out"]):
        assert find_denorm(int(u1), int(u2), bool(morn)) == (int(d), int(nrm))


def _far_replay(gold, key, synFail=None, synPerCon=None, seed=None, nChunk=1):
    import oracle
    from visual_cortex_gb300.model import V1Network, V1Spec
    nV1, bs, nE, ngE, ngI, T = [int(v) for v in gold[key + "_hdr"][:6]]
    prm = gold["far_prm"]
    spec = V1Spec(nblock=nV1 // bs, blockSize=bs, typeAcc=[nE, bs], nTypeE=1, ngFF=1, ngE=ngE, ngI=ngI,
                  dt=float(prm[0]), riseFF=[1.0], decayFF=[5.0], riseE=[float(prm[2]), float(prm[3])],
                  decayE=[float(prm[4]), float(prm[5])], riseI=[float(prm[6])], decayI=[float(prm[8])],
                  vR=[-60.0] * 2, vThres=[-50.0] * 2, gL=[0.05] * 2, C=[1.0] * 2, tRef=[2.0] * 2,
                  vT=[-50.0] * 2, deltaT=[1.0] * 2, tau_w=[150.0] * 2, a=[0.0] * 2, b=[0.0] * 2,
                  pFF=[1.0, 1.0], pE=[float(v) for v in prm[10:14]], pI=[float(prm[14]), float(prm[15])],
                  synFail=synFail or [0.0] * 4, synPerCon=synPerCon or [1.0] * 4, synFailFF=[0.0] * 2,
                  synPerConFF=[1.0] * 2, noisyDep=[0.0] * 2, noFarDelay=0, speedOfThought=float(prm[1]))
    u32 = np.uint32
    net = V1Network(nLGNperV1=np.zeros(nV1, u32), lgnId=np.zeros((1, nV1), u32), sLGN=np.zeros((1, nV1), f32),
                    nNearNB=np.zeros(spec.nblock, u32), nbId=np.zeros((spec.nblock, 1), u32),
                    conMat=np.zeros((spec.nblock, 1, bs, bs), f32), nVec=gold[key + "_nVec"],
                    vecID=gold[key + "_vecID"], conVec=gold[key + "_conVec"], delayVec=gold[key + "_delayVec"],
                    tonicDep=np.zeros(nV1, f32))
    vo = oracle.V1Oracle(spec, net)
    if seed is not None:
        vo.set_far_failure(seed, nChunk)
    L = oracle.lib()
    zE, zI = np.zeros(ngE * nV1, f32), np.zeros(ngI * nV1, f32)
    for t in range(T):
        for name, z in (("gE", zE), ("hE", zE), ("gI", zI), ("hI", zI)):
            vo.put(name, z)
        vo.put("sInfo", gold[key + "_sInfo"][t])
        L.orc_v1_deliver_far(vo.h)
        got = np.concatenate([vo.get("gE").reshape(ngE, nV1), vo.get("hE").reshape(ngE, nV1),
                              vo.get("gI").reshape(ngI, nV1), vo.get("hI").reshape(ngI, nV1)])
        np.testing.assert_array_equal(got, gold[key + "_out"][t], err_msg=f"step {t}")
    assert np.abs(gold[key + "_out"]).sum() > 0


def test_far_delivery_matches_recal_G_vec(gold):
    """fill_fSpikeTrain + recal_G_vec over a 120-step spike sequence: the oracle's
    restatement gives the same far conductances, bit for bit, every step."""
    _far_replay(gold, "far")


def test_far_failure_matches_recal_G_vec(gold):
    """The same with synaptic failure on every pair: the reference's host engines (seeded
    seed + i) drawn through one normal_distribution per chunk call, 3 blocks in chunks of 2
    and 1; the oracle's libstdc++ restatement reproduces every draw, bit for bit."""
    fail = [float(v) for v in gold["farfail_fail"]]
    _far_replay(gold, "farfail", synFail=fail[:4], synPerCon=fail[4:], seed=int(gold["farfail_seed"][0]),
                nChunk=int(gold["farfail_hdr"][7]))


def test_oracle_host_init_matches_the_library():
    """The oracle's restatement of the reference's host-drawn initial state (v, w, g, h from
    one default_random_engine and one shared normal_distribution) equals the library's, which
    calls libstdc++'s <random> itself: bit for bit, with AdEx w and uniform v0."""
    from visual_cortex_gb300 import synth
    from visual_cortex_gb300.model import host_init_state
    import oracle
    for kw in (dict(nblock=2, adex_inh=True), dict(nblock=1)):
        wl = synth.make_workload("init", seed=3, n_lgn=256, nt=16, nFrame=8, **kw)
        s = wl.spec
        tonic = wl.net.tonicDep
        nl = wl.net.nLGNperV1.copy()
        nl[::7] = 0
        gFF0 = np.tile([0.01, 0.2, 0.003, 0.3], s.nType * s.ngFF).astype(np.float32)
        gE0 = np.tile([0.005, 0.2, 0.001, 0.2], s.nType * s.ngE).astype(np.float32)
        gI0 = np.tile([0.01, 0.25, 0.002, 0.2], s.nType * s.ngI).astype(np.float32)
        w0 = np.tile([0.01, 0.005], s.nType).astype(np.float32)
        for use_v0 in (False, True):
            a = host_init_state(s, 77, tonic, nl, None, w0, gFF0, gE0, gI0, use_v0=use_v0)
            b = oracle.host_init_state(s, 77, tonic, nl, None, w0, gFF0, gE0, gI0, use_v0=use_v0)
            for k in ("v", "w", "gFF", "hFF", "gE", "hE", "gI", "hI"):
                x, y = getattr(a, k), getattr(b, k)
                if x is None:
                    assert y is None
                    continue
                np.testing.assert_array_equal(x, y, err_msg=k)


def _ff_rows(gold):
    """The learnff rows as pv1_ff_learning structs and the reference's derived constants
    (LearnVarShapeFF_E_pre: n, tauLTP; LearnVarShapeFF_E_post: n, tau[3], A_LTP, A_ratio,
    targetFR, gmax, gmin; then exp_homeo)."""
    from visual_cortex_gb300 import _native as N
    rows = gold["learnff_in"]
    out = gold["learnff_out"]
    for r, b in zip(rows, out):
        cfg = N.FFLearning(learning=3, tauLTP=r[0], tauLTD=r[1], tauTrip=r[2], tauAvg=r[3], targetFR=r[4],
                           A_LGN=r[5], r_LTD=r[6], gmaxLGN=r[7], gminLGN=r[8], sRatioLGN=r[9],
                           decayTimeHomeoFF=r[11], FF_InfRatio=1.0, applyHomeo=0, symmetricHomeo=1, rebound=0)
        pre = np.frombuffer(b[:8].tobytes(), np.uint32)
        post = np.frombuffer(b[8:44].tobytes(), f32)
        assert pre[0] == 1 and np.frombuffer(b[8:12].tobytes(), np.uint32)[0] == 1
        want = np.array([post[4], post[5], post[7], post[8], np.frombuffer(b[44:48].tobytes(), f32)[0]], f32)
        yield cfg, r, want, np.frombuffer(b[4:8].tobytes(), f32)[0], post


def test_learning_constants_match_learnFF_post(gold, L):
    """The oracle's and the library's derived LGN->V1 learning constants (A_LTP, the LTD rate
    A_ratio with its targetFR scaling, gmax, gmin, exp_homeo) equal the reference's learnFF_post
    and exp_homeo bit for bit, and its tau fields are the cfg's."""
    from visual_cortex_gb300 import _native as N
    for cfg, r, want, tauLTP, post in _ff_rows(gold):
        assert tauLTP == r[0] and post[1] == r[1] and post[2] == r[2] and post[3] == r[3] and post[6] == r[4]
        a = np.zeros(5, f32)
        L.orc_ff_learning_rates(C.byref(cfg), f32(r[10]), fp(a))
        np.testing.assert_array_equal(a, want)
        b = np.zeros(5, f32)
        assert N.lib.pv1_ff_learning_rates(C.byref(cfg), f32(r[10]), N.fptr(b)) == 0
        np.testing.assert_array_equal(b, want)
