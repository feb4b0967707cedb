"""Cases on which the reference's own GPU kernels were run -- TEST INFRASTRUCTURE.

tests/golden/make_ref_kernel_golden.py feeds these inputs to oracle/ref/ref_kernel_runner.cu
(the reference's kernels, src/coredynamics.cu and src/discrete_input_convol.cu, compiled from
its sources into oracle/_ref/ref_kernels.cubin) and stores inputs and outputs in
tests/golden/ref_kernels.npz; tests/test_ref_kernels.py rebuilds the same networks from the
seeds here and holds the oracle (CPU) and the library (GPU) to those outputs.

Bundles are the runner's file format: records {char name[32]; char type[4]; u64 count; data}.
"""
from __future__ import annotations

import numpy as np

f32, u32, i32, u64, u8 = np.float32, np.uint32, np.int32, np.uint64, np.uint8
_CODES = {np.dtype(f32): "f4", np.dtype(u32): "u4", np.dtype(i32): "i4", np.dtype(u64): "u8",
          np.dtype(u8): "u1"}
_TYPES = {"f4": f32, "u4": u32, "i4": i32, "u8": u64, "u1": u8}

STATE_BYTES = 48     # curandStateMRG32k3a


def write_bundle(path: str, arrays: dict):
    with open(path, "wb") as f:
        for name, a in arrays.items():
            a = np.ascontiguousarray(a)
            code = _CODES[a.dtype]
            f.write(name.encode().ljust(32, b"\0")[:32])
            f.write(code.encode().ljust(4, b"\0"))
            f.write(np.uint64(a.size).tobytes())
            f.write(a.tobytes())


def read_bundle(path: str) -> dict:
    out = {}
    data = open(path, "rb").read()
    off = 0
    while off < len(data):
        name = data[off:off + 32].split(b"\0")[0].decode()
        code = data[off + 32:off + 34].decode()
        n = int(np.frombuffer(data, u64, 1, off + 36)[0])
        off += 44
        t = np.dtype(_TYPES[code])
        out[name] = np.frombuffer(data, t, n, off).copy()
        off += n * t.itemsize
    return out


def scalar(v, t):
    return np.array([v], dtype=t)


# ---- LGN: logRand_init + LGN_nonlinear ----------------------------------------------------
LGN_N, LGN_K, LGN_NU, LGN_NSX = 512, 48, 24, 32
LGN_SEED = 1234567


def lgn_case() -> dict:
    """512 cells on a 32 x 16 spike surface, 48 steps of seeded convolutions (a mix of silent,
    moderate and saturating drive) with per-cell logistic parameters; the draws of the first
    24 uniforms of every generator are returned by the runner for the oracle's replay."""
    rng = np.random.default_rng(77)
    n, K = LGN_N, LGN_K
    ids = np.arange(n)
    maxc = rng.uniform(0.5, 2.0, n).astype(f32)
    convol = (rng.uniform(-0.3, 1.2, (K, n)) * maxc).astype(f32)
    c50 = rng.uniform(0.2, 0.5, n).astype(f32)
    sharp = rng.uniform(4.0, 12.0, n).astype(f32)
    a = rng.uniform(0.9, 1.3, n).astype(f32)
    b = rng.uniform(0.0, 0.05, n).astype(f32)
    return dict(seed=scalar(LGN_SEED, u64), n=scalar(n, u32), K=scalar(K, u32), NU=scalar(LGN_NU, u32),
                nsx=scalar(LGN_NSX, u32), nsy=scalar(n // LGN_NSX, u32),
                sx=(ids % LGN_NSX).astype(i32), sy=(ids // LGN_NSX).astype(i32),
                convol=convol.reshape(-1), max_convol=maxc, c50=c50, sharpness=sharp, a=a, b=b,
                convolRatio=scalar(1.0, f32), frRatio=scalar(80.0, f32), dt=scalar(0.125, f32))


# ---- V1: rand_spInit, compute_V_collect_spike_learnFF_fast, recal_G_mat_nd_fast -----------
V1_T, V1_SNAP = 160, 32
V1_SEED = 4242


def v1_workload(sp: bool = False, host_init=None):
    """Two blocks of 1024 (768 LIF E / 256 AdEx I), 512 LGN cells, 20 LGN synapses each, no far
    partners; each block has the other as a second near-neighbour block (its tile is the
    other block's own tile at half strength), so near delivery crosses blocks."""
    from visual_cortex_gb300 import synth
    kw = dict(spE0=[60.0, 20.0], spI0=[80.0, 30.0]) if sp else {}
    wl = synth.make_workload("ref-pin", seed=21, nblock=2, n_lgn=512, m=20, width=64, height=64,
                             nt=V1_T, adex_inh=True, nFrame=40, host_init=host_init, **kw)
    net = wl.net
    nb, bs = wl.spec.nblock, wl.spec.blockSize
    own = net.conMat[:, 0]
    cm = np.empty((nb, 2, bs, bs), f32)
    cm[:, 0] = own
    cm[:, 1] = own[::-1] * f32(0.5)
    net.conMat = cm
    net.nNearNB = np.full(nb, 2, u32)
    net.nbId = np.array([[b, (b + 1) % nb] for b in range(nb)], u32)
    return wl


def v1_inputs(wl, sp0=None, lgn_rows=None, T: int = 0) -> dict:
    """The runner's V1 inputs for a workload (LGN surface 32 wide, cell id = y * 32 + x)."""
    s, net = wl.spec, wl.net
    n = s.nV1
    nsx = 32
    nl = wl.lgn.nLGN
    ids = net.lgnId.astype(np.int64)
    init = wl.init
    d = dict(
        nblock=scalar(s.nblock, u32), blockSize=scalar(s.blockSize, u32), nType=scalar(s.nType, u32),
        nTypeE=scalar(s.nTypeE, u32), nE=scalar(s.nE, u32), ngFF=scalar(s.ngFF, u32), ngE=scalar(s.ngE, u32),
        ngI=scalar(s.ngI, u32), trainDepth=scalar(wl.seeds.trainDepth, u32), dt=scalar(s.dt, f32),
        typeAcc=np.asarray(s.typeAcc, u32),
        v=init.v, w=init.w if init.w is not None else np.zeros(n, f32), tBack=np.zeros(n, f32),
        gFF=init.gFF, hFF=init.hFF, gE=init.gE, hE=init.hE, gI=init.gI, hI=init.hI,
        pFF=np.asarray(s.pFF, f32), pE=np.asarray(s.pE, f32), pI=np.asarray(s.pI, f32),
        vR=np.asarray(s.vR, f32), vThres=np.asarray(s.vThres, f32), gL=np.asarray(s.gL, f32),
        C=np.asarray(s.C, f32), tRef=np.asarray(s.tRef, f32), vT=np.asarray(s.vT, f32),
        deltaT=np.asarray(s.deltaT, f32), tau_w=np.asarray(s.tau_w, f32), a=np.asarray(s.a, f32),
        b=np.asarray(s.b, f32), synFailFF=np.asarray(s.synFailFF, f32),
        synPerConFF=np.asarray(s.synPerConFF, f32), synFail=np.asarray(s.synFail, f32),
        synPerCon=np.asarray(s.synPerCon, f32), noisyDep=np.asarray(s.noisyDep, f32),
        riseFF=np.asarray(s.riseFF, f32), decayFF=np.asarray(s.decayFF, f32),
        riseE=np.asarray(s.riseE, f32), decayE=np.asarray(s.decayE, f32),
        riseI=np.asarray(s.riseI, f32), decayI=np.asarray(s.decayI, f32),
        sp0=np.asarray(sp0 if sp0 is not None else np.zeros(2 * s.nType), f32),
        tonicDep=net.tonicDep, nLGNperV1=net.nLGNperV1, maxLGN=scalar(net.maxLGN, u32),
        sLGN=net.sLGN, LGN_idx=(ids % nsx).astype(i32), LGN_idy=(ids // nsx).astype(i32),
        seed=scalar(wl.seeds.cond, u64), SCsplit=scalar(wl.seeds.SCsplit, u32),
        noDelay=scalar(1, i32), iModel=scalar(s.iModel, i32), noiseOnTonic=scalar(int(bool(s.noiseOnTonic)), i32))
    for k in list(d):
        d[k] = np.ascontiguousarray(d[k])
    if lgn_rows is not None:
        cells = np.arange(nl)
        d.update(T=scalar(T, u32), snapEvery=scalar(V1_SNAP, u32), nLGNcells=scalar(nl, u32),
                 nsx=scalar(nsx, u32), nsy=scalar((nl + nsx - 1) // nsx, u32),
                 cell_x=(cells % nsx).astype(i32), cell_y=(cells // nsx).astype(i32),
                 lgnSInfo=np.ascontiguousarray(lgn_rows[:T], f32).reshape(-1),
                 nnb=scalar(net.nnb, u32), conMat=np.ascontiguousarray(net.conMat, f32).reshape(-1),
                 nNearNB=net.nNearNB, nbId=np.ascontiguousarray(net.nbId).reshape(-1))
    return d


STATE_KEYS = ("v", "w", "tBack", "gFF", "hFF", "gE", "hE", "gI", "hI")


# ---- LGN convolution: store_PM (magno) + LGN_convol_magno ---------------------------------
MAGNO_T, MAGNO_STRIDE = 400, 4


def magno_workload():
    """128 ON/OFF magno cells (16 x 16 samples, 250-tap temporal kernels at 1 ms) on 64 x 64
    grating frames at 120 Hz; 400 steps reach the sixth frame."""
    from visual_cortex_gb300 import synth
    return synth.make_workload("magno-pin", seed=5, nblock=1, n_lgn=128, m=20, width=64, height=64,
                               nt=MAGNO_T, nFrame=8)


def magno_inputs(wl) -> dict:
    lg, s = wl.lgn, wl.lgn.sched
    assert lg.nParvo == 0 and lg.nMagno_C == 0
    fr = np.ascontiguousarray(wl.stim.frames, f32)
    spatial = np.concatenate([np.asarray(getattr(lg, k), f32) for k in ("polar", "rw", "ecc", "rh", "orient", "k")])
    temporal = np.concatenate([np.asarray(getattr(lg, k), f32) for k in ("tauR", "tauD", "delay", "ratio", "nR", "nD")])
    return dict(nLGN=scalar(lg.nLGN, u32), mSample1D=scalar(lg.mSample1D, u32),
                mKernelSample=scalar(s.mKernelSample, u32), kernelSampleDt=scalar(s.mKernelSampleDt, f32),
                kernelSampleT0=scalar(s.mKernelSampleT0f, f32), spatial=spatial, temporal=temporal,
                coneType=np.asarray(lg.coneType, u32), L_x0=scalar(lg.L_x0, f32), L_y0=scalar(lg.L_y0, f32),
                R_x0=scalar(lg.R_x0, f32), R_y0=scalar(lg.R_y0, f32),
                normViewDistance=scalar(lg.normViewDistance, f32), nsig=scalar(lg.nsig, f32),
                flat_retina=scalar(int(bool(lg.flat_retina)), i32), width=scalar(fr.shape[3], u32),
                height=scalar(fr.shape[2], u32), nFrame=scalar(fr.shape[0], u32), frames=fr.reshape(-1),
                initLMS=np.asarray(wl.stim.init_LMS, f32), maxFrame=scalar(s.maxFrame, u32),
                ntPerFrame=scalar(s.ntPerFrame, u32), denorm=scalar(s.denorm, u32),
                magnoComp=scalar(s.magnoComp, u32), frameOffset=scalar(s.dFrame if s.pLongerThanM else 0, u32),
                kernelSampleInterval=scalar(s.mKernelSampleInterval, u32),
                iKernelSampleT0=scalar(s.mKernelSampleT0, u32), dt=scalar(s.dt, f32),
                T=scalar(MAGNO_T, u32), stride=scalar(MAGNO_STRIDE, u32))


# ---- LGN->V1 plasticity (learning = 3) ---------------------------------------------------
LEARN_T = 120


def learning_params():
    """The FFLearning of the pinned learning cases (multiplicative homeostasis, targetFR > 0)."""
    from visual_cortex_gb300.model import FFLearning
    return FFLearning(tauLTP=16.8, tauLTD=33.7, tauTrip=114.0, tauAvg=1000.0, targetFR=2.0, A_LGN=0.02,
                      r_LTD=1.0, gmaxLGN=0.6, gminLGN=0.0, sRatioLGN=1.0, decayTimeHomeoFF=250.0,
                      FF_InfRatio=0.9, applyHomeo=1)


def learning_params2():
    """The FFLearning of the learning = 2 case: both FF types (FF->I with its own constants,
    targetFR[1] > 0), one cortical E type (its tauAvg filters vAvgE in the delivery), additive
    homeostasis.  targetFR[0] is 0: with learning != 3 the delivery adds floor(spike word) --
    the membrane potential, about -60, when the neuron did not spike -- to vAvgE every step
    (src/coredynamics.cu:2548-2560), so vAvgE runs to about -7000 within 100 steps, and with
    targetFR[0] > 0 the LTD factor tauLTP vAvgE^2 clips every active FF->E weight to gmin at
    its first LGN spike; the homeostasis total is then the difference of terms of that size
    and carries their rounding (ulps of 1e4), the same on no two machines."""
    from visual_cortex_gb300.model import FFLearning
    return FFLearning(tauLTP=16.8, tauLTD=33.7, tauTrip=114.0, tauAvg=1000.0, targetFR=0.0, A_LGN=0.02,
                      r_LTD=1.0, gmaxLGN=0.6, gminLGN=0.0, sRatioLGN=1.0, decayTimeHomeoFF=250.0,
                      FF_InfRatio=0.9, applyHomeo=2, learning=2, nLearnTypeFF_E=1, nLearnTypeFF_I=1,
                      tauLTP_I=20.0, tauLTD_I=40.0, tauTrip_I=90.0, tauAvg_I=800.0, targetFR_I=5.0, A_LGN_I=0.015,
                      r_LTD_I=0.8, gmaxLGN_I=0.8, gminLGN_I=0.0, sRatioLGN_I=1.2, tauAvgCortical=1000.0)


def learning_params4():
    """The FFLearning of the learning = 4 case: no FF learning (the LGN->V1 weights stay), the
    excitatory filtered rate in the delivery with one cortical E type's tauAvg."""
    from visual_cortex_gb300.model import FFLearning
    return FFLearning(tauLTP=16.8, tauLTD=33.7, tauTrip=114.0, tauAvg=1000.0, targetFR=2.0, A_LGN=0.02,
                      r_LTD=1.0, gmaxLGN=0.6, gminLGN=0.0, sRatioLGN=1.0, decayTimeHomeoFF=250.0,
                      FF_InfRatio=1.0, applyHomeo=0, learning=4, tauAvgCortical=700.0)


def _type_structs(tauLTP, tauLTD, tauTrip, tauAvg, targetFR, A_LGN, r_LTD, gmax, gmin, ratio, L, dt):
    import ctypes as C
    from visual_cortex_gb300 import _native as N
    cfg = N.FFLearning(learning=3, tauLTP=tauLTP, tauLTD=tauLTD, tauTrip=tauTrip, tauAvg=tauAvg, targetFR=targetFR,
                       A_LGN=A_LGN, r_LTD=r_LTD, gmaxLGN=gmax, gminLGN=gmin, sRatioLGN=ratio,
                       decayTimeHomeoFF=L.decayTimeHomeoFF, FF_InfRatio=L.FF_InfRatio)
    r = np.zeros(5, f32)
    assert N.lib.pv1_ff_learning_rates(C.byref(cfg), f32(dt), N.fptr(r)) == 0
    pre = np.array([1], u32).tobytes() + np.array([tauLTP], f32).tobytes()
    post = np.array([1], u32).tobytes() + np.array([tauLTD, tauTrip, tauAvg, r[0], r[1], targetFR, r[2], r[3]],
                                                   f32).tobytes()
    return np.frombuffer(pre, u8).copy(), np.frombuffer(post, u8).copy(), f32(r[4])


def learning_structs(L, dt: float):
    """The bytes of LearnVarShapeFF_E_pre and LearnVarShapeFF_E_post (src/condShape.h:85-126)
    for the FF->E type, with the derived constants of pv1_ff_learning_rates (held bit for bit
    to learnFF_post by tests/test_golden.py), and exp_homeo."""
    return _type_structs(L.tauLTP, L.tauLTD, L.tauTrip, L.tauAvg, L.targetFR, L.A_LGN, L.r_LTD, L.gmaxLGN,
                         L.gminLGN, L.sRatioLGN, L, dt)


def learning_structs_i(L, dt: float):
    """LearnVarShapeFF_I_pre / _post of the FF->I type (zeroed when it is off)."""
    if not (L.learning == 2 and L.nLearnTypeFF_I):
        return np.zeros(8, u8), np.zeros(36, u8)
    pre, post, _ = _type_structs(L.tauLTP_I, L.tauLTD_I, L.tauTrip_I, L.tauAvg_I, L.targetFR_I, L.A_LGN_I, L.r_LTD_I,
                                 L.gmaxLGN_I, L.gminLGN_I, L.sRatioLGN_I, L, dt)
    return pre, post


def cortical_struct(L):
    """LearnVarShapeE (src/condShape.h:159-167) with one cortical E type whose tauAvg is
    L.tauAvgCortical (learnE, src/condShape.cu:22-36; the other fields only shape variables no
    output holds), or zeroed when L.tauAvgCortical is 0."""
    if not L.tauAvgCortical:
        return np.zeros(60, u8)
    tau = np.zeros(7, f32)
    tau[0:3] = (L.tauLTP, L.tauLTD, L.tauTrip)
    tau[3] = L.tauAvgCortical
    b = (np.array([1], u32).tobytes() + tau.tobytes() + np.zeros(2, f32).tobytes() + np.zeros(2, f32).tobytes() +
         np.array([L.targetFR, L.gmaxLGN, L.gminLGN], f32).tobytes())
    return np.frombuffer(b, u8).copy()


def lgn_learn_case() -> dict:
    """The LGN case above with the presynaptic trace of one FF_E type (tauLTP of
    learning_params())."""
    d = lgn_case()
    d["tauLTP"] = scalar(learning_params().tauLTP, f32)
    return d


def pre_traces(lgn_rows, dt: float, tauLTP: float):
    """Presynaptic traces for given LGN spike words (the oracle's trace step, nsp and tsp taken
    from the words): ([T][n] at the step start, [T][n] right after the step's spikes)."""
    import oracle
    T, n = lgn_rows.shape
    var = np.zeros(n, f32)
    start = np.zeros((T, n), f32)
    spk = np.zeros((T, n), f32)
    for t in range(T):
        s = np.ascontiguousarray(lgn_rows[t], f32)
        nsp = np.floor(s).clip(0).astype(u32)
        tsp = np.where(s > 0, (s - nsp.astype(f32)) * f32(dt), 0).astype(f32)
        a, b = np.zeros(n, f32), np.zeros(n, f32)
        oracle.lib().orc_lgn_ff_pre(n, f32(dt), f32(tauLTP), oracle.up(nsp), oracle.fp(tsp), oracle.fp(s),
                                    oracle.fp(var), oracle.fp(a), oracle.fp(b))
        start[t], spk[t] = a, b
    return start, spk


def learning_totals(net, L=None):
    """The homeostasis totals of src/patch.cu:4335-4352: each neuron's LGN weights summed in
    synapse order (float), and that times FF_InfRatio."""
    n = net.sLGN.shape[1]
    tot = np.zeros(2 * n, f32)
    L = learning_params() if L is None else L
    for i in range(n):
        t = f32(0)
        for j in range(int(net.nLGNperV1[i])):
            t = f32(t + net.sLGN[j, i])
        tot[i] = t
        tot[n + i] = f32(t * f32(L.FF_InfRatio))
    return tot


def v1_learn_inputs(wl, lgn_rows, T: int, L=None) -> dict:
    L = learning_params() if L is None else L
    d = v1_inputs(wl, lgn_rows=lgn_rows, T=T)
    pre, post, eh = learning_structs(L, wl.spec.dt)
    if L.learning == 4:
        # nLearnTypeFF_E = 0: the reference passes zeroed FF_E structs (src/patch.cu:1174, 1281-1300)
        pre, post = np.zeros_like(pre), np.zeros_like(post)
    ipre, ipost = learning_structs_i(L, wl.spec.dt)
    start, spk = pre_traces(np.asarray(lgn_rows[:T], f32), wl.spec.dt, L.tauLTP)
    d.update(learning=scalar(int(L.learning), i32), lFF_E_pre=pre, lFF_E_post=post, lFF_I_pre=ipre, lFF_I_post=ipost,
             lE=cortical_struct(L), expHomeo=scalar(eh, f32), applyHomeo=scalar(int(L.applyHomeo), i32),
             symmetricHomeo=scalar(int(L.symmetricHomeo), i32), rebound=scalar(int(L.rebound), i32),
             preStart=start.reshape(-1), preSpk=spk.reshape(-1), totalFF=learning_totals(wl.net, L))
    return d
