"""Model description objects and the Simulation handle over the native plan.

The dataclasses hold exactly what the reference's `patch` reads from its cfg and binary
input files for the hot path (after the per-type expansion of src/patch.cu:890-1000); the
Simulation uploads them through the C ABI and steps the network on the GPU.
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _native as N
from .schedule import FrameSchedule

f32 = np.float32
u32 = np.uint32


def _pad(vals, n, fill=0.0):
    out = [float(x) for x in vals][:n]
    return out + [fill] * (n - len(out))


@dataclass
class V1Spec:
    nblock: int
    blockSize: int
    typeAcc: list            # cumulative per type, last == blockSize
    nTypeE: int
    ngFF: int
    ngE: int
    ngI: int
    dt: float
    riseFF: list
    decayFF: list
    riseE: list
    decayE: list
    riseI: list
    decayI: list
    vR: list
    vThres: list
    gL: list
    C: list
    tRef: list
    vT: list
    deltaT: list
    tau_w: list
    a: list
    b: list
    pFF: list                # [nType][ngFF]
    pE: list                 # [nType][ngE]
    pI: list                 # [nType][ngI]
    synFail: list            # [nType][nType] (pre, post)
    synPerCon: list
    synFailFF: list
    synPerConFF: list
    noisyDep: list
    tau_noise: float = 0.0
    noiseOnTonic: bool = True
    iModel: int = 1
    noDelay: int = 1
    noFarDelay: int = 0
    speedOfThought: float = 1.0
    hWrite: bool = True
    vE: float = 0.0
    vI: float = -75.0
    vL: float = -65.0

    @property
    def nType(self) -> int:
        return len(self.typeAcc)

    @property
    def nV1(self) -> int:
        return self.nblock * self.blockSize

    @property
    def nE(self) -> int:
        return self.typeAcc[self.nTypeE - 1]

    @property
    def nI(self) -> int:
        return self.blockSize - self.nE

    def type_of(self, local):
        local = np.asarray(local)
        t = np.full(local.shape, self.nType - 1, dtype=np.int64)
        for j in reversed(range(self.nType)):
            t[local < self.typeAcc[j]] = j
        return t

    def to_struct(self) -> N.V1Config:
        c = N.V1Config()
        c.nblock, c.blockSize, c.nType, c.nTypeE = self.nblock, self.blockSize, self.nType, self.nTypeE
        for j in range(N.MAX_NTYPE):
            c.typeAcc[j] = self.typeAcc[j] if j < self.nType else self.blockSize
        c.ngFF, c.ngE, c.ngI, c.dt = self.ngFF, self.ngE, self.ngI, self.dt
        for name in ("riseFF", "decayFF", "riseE", "decayE", "riseI", "decayI"):
            getattr(c, name)[:] = _pad(getattr(self, name), N.MAX_NG, 1.0)
        c.vE, c.vI, c.vL = self.vE, self.vI, self.vL
        for name in ("vR", "vThres", "gL", "C", "tRef", "vT", "deltaT", "tau_w", "a", "b",
                     "synFailFF", "synPerConFF", "noisyDep"):
            getattr(c, name)[:] = _pad(getattr(self, name), N.MAX_NTYPE,
                                       1.0 if name in ("tau_w", "C", "deltaT", "synPerConFF") else 0.0)
        for name in ("pFF", "pE", "pI", "synFail", "synPerCon"):
            getattr(c, name)[:] = _pad(getattr(self, name), N.MAX_NTYPE * N.MAX_NTYPE,
                                       1.0 if name == "synPerCon" else 0.0)
        c.tau_noise = self.tau_noise
        c.noiseOnTonic = int(bool(self.noiseOnTonic))
        c.iModel, c.noDelay, c.noFarDelay = self.iModel, self.noDelay, self.noFarDelay
        c.speedOfThought = self.speedOfThought
        c.hWrite = int(bool(self.hWrite))
        return c


@dataclass
class V1Network:
    """Connectivity arrays in the reference's device layouts."""
    nLGNperV1: np.ndarray     # u32 [nV1]
    lgnId: np.ndarray         # u32 [maxLGN][nV1]
    sLGN: np.ndarray          # f32 [maxLGN][nV1] (sRatioLGN applied)
    nNearNB: np.ndarray       # u32 [nblock]
    nbId: np.ndarray          # u32 [nblock][nnb]
    conMat: np.ndarray        # f32 [nblock][nnb][bs][bs] (sRatioV1 applied)
    nVec: np.ndarray          # u32 [nV1]
    vecID: np.ndarray         # u32 [sum nVec]
    conVec: np.ndarray        # f32 [sum nVec] (sRatioV1 applied)
    delayVec: np.ndarray      # f32 [sum nVec] (mm)
    tonicDep: np.ndarray      # f32 [nV1]
    delayMat: np.ndarray | None = None   # f32 like conMat: distances (mm), used when noDelay = 0

    @property
    def maxLGN(self) -> int:
        return int(self.lgnId.shape[0])

    @property
    def nnb(self) -> int:
        return int(self.nbId.shape[1])


@dataclass
class LgnSpec:
    """Magno LGN cells (ON/OFF DoG) and the kernel-sampling bookkeeping."""
    nParvo_I: int
    nMagno_I: int
    nParvo_C: int
    nMagno_C: int
    mSample1D: int
    sched: FrameSchedule
    polar: np.ndarray   # f32 [2*nLGN] center then surround
    ecc: np.ndarray
    rw: np.ndarray
    rh: np.ndarray
    orient: np.ndarray
    k: np.ndarray
    ratio: np.ndarray
    tauR: np.ndarray
    tauD: np.ndarray
    nR: np.ndarray
    nD: np.ndarray
    delay: np.ndarray
    spont: np.ndarray   # f32 [nLGN]
    c50: np.ndarray
    sharpness: np.ndarray
    coneType: np.ndarray  # u32 [2*nLGN]
    normViewDistance: float
    L_x0: float
    L_y0: float
    R_x0: float
    R_y0: float
    nsig: float = 3.0
    convolRatio: float = 1.0
    frRatio: float = 1.0
    flat_retina: bool = True
    nSample1D: int = 0                 # parvo nSpatialSample1D
    covariant: np.ndarray | None = None  # f32 [nLGN] (parvo_maxConvol)

    @property
    def nLGN(self) -> int:
        return self.nParvo_I + self.nMagno_I + self.nParvo_C + self.nMagno_C

    @property
    def nMagno(self) -> int:
        return self.nMagno_I + self.nMagno_C

    @property
    def nParvo(self) -> int:
        return self.nParvo_I + self.nParvo_C

    def parvo_ids(self) -> np.ndarray:
        c = np.arange(self.nParvo)
        return np.where(c < self.nParvo_I, c, c + self.nMagno_I)

    def to_parvo_struct(self) -> N.LgnParvoConfig:
        s = self.sched
        q = N.LgnParvoConfig()
        q.nSample1D = self.nSample1D
        q.nKernelSample = s.nKernelSample
        q.kernelSampleInterval = s.kernelSampleInterval
        q.iKernelSampleT0 = s.iKernelSampleT0
        q.parvoComp = s.parvoComp
        q.frameOffset = 0 if s.pLongerThanM else s.dFrame
        q.kernelSampleDt = s.kernelSampleDt
        q.kernelSampleT0 = s.kernelSampleT0f
        return q

    def magno_ids(self) -> np.ndarray:
        m = np.arange(self.nMagno)
        ids = self.nParvo_I + m
        ids[m >= self.nMagno_I] += self.nParvo_C
        return ids

    def to_struct(self) -> N.LgnConfig:
        s = self.sched
        c = N.LgnConfig()
        c.nLGN = self.nLGN
        c.nParvo_I, c.nMagno_I, c.nParvo_C, c.nMagno_C = (self.nParvo_I, self.nMagno_I,
                                                          self.nParvo_C, self.nMagno_C)
        c.mSample1D = self.mSample1D
        c.nKernelSample = s.mKernelSample
        c.kernelSampleInterval = s.mKernelSampleInterval
        c.iKernelSampleT0 = s.mKernelSampleT0
        c.denorm, c.ntPerFrame, c.maxFrame = s.denorm, s.ntPerFrame, s.maxFrame
        c.magnoComp = s.magnoComp
        c.frameOffset = s.dFrame if s.pLongerThanM else 0
        c.dt = s.dt
        c.kernelSampleDt = s.mKernelSampleDt
        c.kernelSampleT0 = s.mKernelSampleT0f
        c.convolRatio, c.frRatio = self.convolRatio, self.frRatio
        c.normViewDistance = self.normViewDistance
        c.L_x0, c.L_y0, c.R_x0, c.R_y0 = self.L_x0, self.L_y0, self.R_x0, self.R_y0
        c.nsig = self.nsig
        c.flat_retina = int(bool(self.flat_retina))
        return c

    def params_struct(self):
        keep = {}
        p = N.LgnParams()
        for name in ("polar", "ecc", "rw", "rh", "orient", "k", "ratio", "tauR", "tauD", "nR",
                     "nD", "delay", "spont", "c50", "sharpness"):
            a = np.ascontiguousarray(getattr(self, name), dtype=f32)
            keep[name] = a
            setattr(p, name, N.fptr(a))
        ct = np.ascontiguousarray(self.coneType, dtype=u32)
        keep["coneType"] = ct
        p.coneType = N.uptr(ct)
        return p, keep


@dataclass
class Stimulus:
    frames: np.ndarray     # f32 [nFrame][3][h][w]
    init_LMS: tuple = (0.5, 0.5, 0.5)

    @property
    def shape(self):
        return self.frames.shape


@dataclass
class InitState:
    v: np.ndarray
    w: np.ndarray | None
    gFF: np.ndarray
    hFF: np.ndarray
    gE: np.ndarray
    hE: np.ndarray
    gI: np.ndarray
    hI: np.ndarray


@dataclass
class FFLearning:
    """LGN->V1 plasticity parameters as the reference's cfg gives them: `learning` 1 (FF->E
    triplet rule, the excitatory filtered rate advanced in the delivery), 2 (FF->E and FF->I),
    3 (FF->E alone) or 4 (the filtered rate alone).  The plain fields are the FF->E type's
    (element [0] of the cfg arrays, gmax/gmin before sRatioLGN), the *_I fields the FF->I
    type's (element [nLearnTypeFF_E])."""
    tauLTP: float
    tauLTD: float
    tauTrip: float
    tauAvg: float
    targetFR: float
    A_LGN: float
    r_LTD: float
    gmaxLGN: float
    gminLGN: float
    sRatioLGN: float
    decayTimeHomeoFF: float = 250.0
    FF_InfRatio: float = 1.0
    applyHomeo: int = 0
    symmetricHomeo: bool = True
    rebound: bool = False
    learning: int = 3
    nLearnTypeFF_E: int = 1
    nLearnTypeFF_I: int = 0
    # the FF->I type (learning = 2 with nLearnTypeFF_I = 1)
    tauLTP_I: float = 0.0
    tauLTD_I: float = 0.0
    tauTrip_I: float = 0.0
    tauAvg_I: float = 0.0
    targetFR_I: float = 0.0
    A_LGN_I: float = 0.0
    r_LTD_I: float = 0.0
    gmaxLGN_I: float = 0.0
    gminLGN_I: float = 0.0
    sRatioLGN_I: float = 1.0
    # vAvgE's time constant in the delivery (learning 1, 2, 4): tauAvg[0] with cortical E types
    tauAvgCortical: float = 0.0

    def to_struct(self):
        from . import _native as N
        import dataclasses
        kw = {f.name: getattr(self, f.name) for f in dataclasses.fields(self)}
        for k in ("learning", "applyHomeo", "symmetricHomeo", "rebound", "nLearnTypeFF_E", "nLearnTypeFF_I"):
            kw[k] = int(kw[k])
        return N.FFLearning(**kw)


def ff_post_size(spec: V1Spec, mode: int, ff_i: int) -> int:
    """Floats of learnVar's FF block (src/patch.cu:4367-4369): the FF->E post traces (none with
    learning 4), the FF->I ones (ff_i types), vAvgE [nE_total][2] and vAvgI [nI_total]."""
    nEt, nIt = spec.nE * spec.nblock, (spec.blockSize - spec.nE) * spec.nblock
    return (0 if mode == 4 else 2 * nEt) + 2 * ff_i * nIt + 2 * nEt + nIt


@dataclass
class Seeds:
    lgn: int          # logRand_init seed
    cond: int         # rand_spInit seed
    trainDepth: int = 2
    sp0: tuple | None = None   # initial spikes: per-step chance [nType][2] (spE0, spI0 x dt/1000)
    SCsplit: int = 0
    nChunk: int = 1            # chunks of blocks of the far delivery (far synaptic failure)

    @property
    def far_engine_seed(self) -> int:
        """Seed of the first far-failure host engine: the one after logRand_init's."""
        return int(self.lgn) + 1

    def has_sp0(self) -> bool:
        return self.sp0 is not None and any(float(x) > 0 for x in np.ravel(self.sp0))


class Simulation:
    """One patch on the current GPU: owns a native plan."""

    def __init__(self, spec: V1Spec, net: V1Network, lgn: LgnSpec, stim: Stimulus,
                 init: InitState, seeds: Seeds, record_init: int = 0):
        """record_init > 0 keeps what pv1_v1_init_spikes drew (init_record) with room for that
        many near failure draws per neuron."""
        self.spec, self.net, self.lgn, self.stim = spec, net, lgn, stim
        self._cfg = spec.to_struct()
        plan = C.c_void_p()
        rc = N.lib.pv1_plan_create(C.byref(self._cfg), C.byref(plan))
        self.plan = plan
        N.check(plan, rc, "pv1_plan_create")
        lc = lgn.to_struct()
        lp, keep = lgn.params_struct()
        if lgn.nParvo > 0:
            pc = lgn.to_parvo_struct()
            cov = np.ascontiguousarray(lgn.covariant, dtype=f32)
            N.check(plan, N.lib.pv1_lgn_setup_parvo(plan, C.byref(lc), C.byref(pc), C.byref(lp), N.fptr(cov),
                                                    int(seeds.lgn)), "pv1_lgn_setup_parvo")
        else:
            N.check(plan, N.lib.pv1_lgn_setup(plan, C.byref(lc), C.byref(lp), int(seeds.lgn)), "pv1_lgn_setup")
        del keep
        fr = np.ascontiguousarray(stim.frames, dtype=f32)
        nF, _, h, w = fr.shape
        init3 = np.asarray(stim.init_LMS, dtype=f32)
        N.check(plan, N.lib.pv1_stimulus_load(plan, nF, h, w, N.fptr(init3), N.fptr(fr)), "pv1_stimulus_load")
        self._set_network(net)
        N.check(plan, N.lib.pv1_v1_far_failure_engines(plan, seeds.far_engine_seed, int(seeds.nChunk)),
                "pv1_v1_far_failure_engines")
        self.put_initial_state(init)
        self.init_record = None
        if seeds.has_sp0():
            self._init_spikes(seeds, record_init)
        else:
            N.check(plan, N.lib.pv1_v1_init_rng(plan, int(seeds.cond), int(seeds.trainDepth)), "pv1_v1_init_rng")
        self.step = 0

    def _init_spikes(self, seeds: Seeds, record_init: int):
        sp0 = np.ascontiguousarray(np.ravel(seeds.sp0), dtype=f32)
        if sp0.size != 2 * self.spec.nType:
            raise ValueError("sp0 holds two chances per neuron type")
        rec = None
        if record_init:
            n, d, cap = self.spec.nV1, int(seeds.trainDepth), int(record_init)
            self.init_record = dict(uniforms=np.zeros((n, 2 * d), f32), nUniform=np.zeros(n, u32),
                                    normals=np.zeros((n, cap), f32), nNormal=np.zeros(n, u32),
                                    history=np.zeros((d, n), f32))
            r = self.init_record
            rec = N.InitRecord(N.fptr(r["uniforms"]), N.uptr(r["nUniform"]), N.fptr(r["normals"]),
                               N.uptr(r["nNormal"]), cap, N.fptr(r["history"]))
        N.check(self.plan, N.lib.pv1_v1_init_spikes(self.plan, int(seeds.cond), int(seeds.trainDepth), N.fptr(sp0),
                                                    int(seeds.SCsplit), None if rec is None else C.byref(rec)),
                "pv1_v1_init_spikes")

    def _set_network(self, net: V1Network):
        c = lambda a, t: np.ascontiguousarray(a, dtype=t)
        self._net_keep = [c(net.nLGNperV1, u32), c(net.lgnId, u32), c(net.sLGN, f32)]
        n, ids, s = self._net_keep
        N.check(self.plan, N.lib.pv1_v1_set_lgn_synapses(self.plan, net.maxLGN, N.uptr(n), N.uptr(ids), N.fptr(s)),
                "pv1_v1_set_lgn_synapses")
        nn, nb, cm = c(net.nNearNB, u32), c(net.nbId, u32), c(net.conMat, f32)
        if self.spec.noDelay:
            N.check(self.plan, N.lib.pv1_v1_set_near(self.plan, net.nnb, N.uptr(nn), N.uptr(nb), N.fptr(cm)),
                    "pv1_v1_set_near")
        else:
            if net.delayMat is None:
                raise ValueError("noDelay = 0 needs the network's delayMat")
            dm = c(net.delayMat, f32)
            N.check(self.plan, N.lib.pv1_v1_set_near_delayed(self.plan, net.nnb, N.uptr(nn), N.uptr(nb),
                                                             N.fptr(cm), N.fptr(dm)), "pv1_v1_set_near_delayed")
        nv, vid, cv, dv = c(net.nVec, u32), c(net.vecID, u32), c(net.conVec, f32), c(net.delayVec, f32)
        N.check(self.plan, N.lib.pv1_v1_set_far(self.plan, N.uptr(nv), N.uptr(vid), N.fptr(cv), N.fptr(dv)),
                "pv1_v1_set_far")

    def put_initial_state(self, st: InitState):
        c = lambda a: None if a is None else np.ascontiguousarray(a, dtype=f32)
        arrs = [c(st.v), c(st.w), c(st.gFF), c(st.hFF), c(st.gE), c(st.hE), c(st.gI), c(st.hI),
                c(self.net.tonicDep)]
        N.check(self.plan, N.lib.pv1_v1_set_state(self.plan, *[N.fptr(a) for a in arrs]), "pv1_v1_set_state")

    # -- stepping ------------------------------------------------------------------------
    def run(self, nsteps: int, sync: bool = True):
        N.check(self.plan, N.lib.pv1_run(self.plan, int(nsteps), int(sync)), "pv1_run")
        self.step += nsteps

    def run_spikes_to_host(self, nsteps: int, out: np.ndarray) -> np.ndarray:
        """Runs nsteps and writes their spike words into out [nsteps][nV1] (float32, best
        page-locked: N.pinned_empty), the copies overlapping the run."""
        if out.shape != (nsteps, self.spec.nV1) or out.dtype != f32 or not out.flags.c_contiguous:
            raise ValueError("out must be a contiguous float32 array [nsteps][nV1]")
        N.check(self.plan, N.lib.pv1_run_spikes_to_host(self.plan, int(nsteps), N.fptr(out)), "pv1_run_spikes_to_host")
        self.step += nsteps
        return out

    def launches(self) -> int:
        return int(N.lib.pv1_last_launch_count(self.plan))

    def run_timed(self, nsteps: int, flush_bytes: int = 0) -> float:
        """Runs nsteps after an optional L2 flush; returns device milliseconds (CUDA events
        on the plan's stream)."""
        ms = C.c_float()
        N.check(self.plan, N.lib.pv1_run_timed(self.plan, int(nsteps), int(flush_bytes), C.byref(ms)),
                "pv1_run_timed")
        self.step += nsteps
        return float(ms.value)

    def time_kernels(self, nsteps: int):
        """Mean device ms per V1-step launch and per LGN chunk (rate + spike kernels)."""
        v1, lgn, k = C.c_float(), C.c_float(), C.c_int()
        N.check(self.plan, N.lib.pv1_time_kernels(self.plan, int(nsteps), C.byref(v1), C.byref(lgn), C.byref(k)),
                "pv1_time_kernels")
        self.step += (int(nsteps) // k.value) * k.value
        return float(v1.value), float(lgn.value), int(k.value)

    def set_ff_learning(self, learning: "FFLearning"):
        """LGN->V1 plasticity (learning 1-4) with the cfg values of `learning` (pv1_set_ff_learning)."""
        c = learning.to_struct()
        N.check(self.plan, N.lib.pv1_set_ff_learning(self.plan, C.byref(c)), "pv1_set_ff_learning")
        mode = int(learning.learning)
        self.ff_mode = mode
        self.ff_i = int(learning.nLearnTypeFF_I) if mode == 2 else 0
        self.ff_types = 0 if mode == 4 else 1 + self.ff_i

    def set_lgn_source(self, device_ptr: int | None, step0: int = 0, nsteps: int = 0):
        """Feed steps [step0, step0 + nsteps) from caller-computed LGN spike words: device_ptr
        is the address of a device array [nsteps][nLGN] on the plan's device (e.g. a torch CUDA
        tensor's data_ptr(), or LgnTensorCore.device_spikes()); None returns to the plan's own
        LGN stage (pv1_set_lgn_source)."""
        N.check(self.plan, N.lib.pv1_set_lgn_source(self.plan, device_ptr, int(step0), int(nsteps)),
                "pv1_set_lgn_source")

    def persistent(self, allow: int = -1) -> bool:
        """Queries (allow=-1) or sets whether V1 steps run as one cooperative launch per
        chunk of steps."""
        rc = N.lib.pv1_persistent_mode(self.plan, int(allow))
        if rc < 0:
            N.check(self.plan, rc, "pv1_persistent_mode")
        return rc == 1

    def fetch_spikes(self, step0: int, n: int, out: np.ndarray | None = None) -> np.ndarray:
        """Spike words [n][nV1] of steps step0..step0+n-1; `out` may be a caller-owned
        (e.g. N.pinned_empty) float32 array of that shape."""
        if out is None:
            out = np.empty((n, self.spec.nV1), f32)
        elif out.shape != (n, self.spec.nV1) or out.dtype != f32 or not out.flags.c_contiguous:
            raise ValueError("out must be a contiguous float32 array [n][nV1]")
        N.check(self.plan, N.lib.pv1_fetch_spikes(self.plan, int(step0), int(n), N.fptr(out)), "pv1_fetch_spikes")
        return out

    def load_stimulus(self, stim: Stimulus):
        fr = np.ascontiguousarray(stim.frames, dtype=f32)
        nF, _, h, w = fr.shape
        init3 = np.asarray(stim.init_LMS, dtype=f32)
        N.check(self.plan, N.lib.pv1_stimulus_load(self.plan, nF, h, w, N.fptr(init3), N.fptr(fr)),
                "pv1_stimulus_load")
        self.stim = stim

    def set_record(self, flags: int, slots: int):
        N.check(self.plan, N.lib.pv1_set_record(self.plan, int(flags), int(slots)), "pv1_set_record")

    def record_floats(self) -> int:
        return int(N.lib.pv1_raw_record_floats(self.plan))

    def fetch_records(self, step0: int, n: int, raw=True, lgn_sp=False, lgn_fr=False):
        rawb = np.empty((n, self.record_floats()), f32) if raw else None
        sp = np.empty((n, self.lgn.nLGN), f32) if lgn_sp else None
        fr = np.empty((n, self.lgn.nLGN), f32) if lgn_fr else None
        N.check(self.plan, N.lib.pv1_fetch_records(self.plan, int(step0), int(n), N.fptr(rawb), N.fptr(sp),
                                                   N.fptr(fr)), "pv1_fetch_records")
        return rawb, sp, fr

    def state(self, name: str) -> np.ndarray:
        spec = self.spec
        n = spec.nV1
        sizes = dict(gFF=spec.ngFF * n, hFF=spec.ngFF * n, gE=spec.ngE * n, hE=spec.ngE * n,
                     gI=spec.ngI * n, hI=spec.ngI * n, lgn_ltr=self.lgn.nLGN, lgn_lnl=self.lgn.nLGN,
                     lgn_sInfo=self.lgn.nLGN, farPull=(spec.ngE + spec.ngI) * 2 * n,
                     lgn_rng=12 * self.lgn.nLGN, v1_rng_cond=12 * n, v1_rng_noisy=12 * n,
                     sLGN=self.net.maxLGN * n,
                     ff_post=ff_post_size(spec, getattr(self, "ff_mode", 3), getattr(self, "ff_i", 0)),
                     ff_pre=getattr(self, "ff_types", 1) * self.lgn.nLGN, total_ff=2 * n)
        out = np.empty(sizes.get(name, n), f32)
        N.check(self.plan, N.lib.pv1_get_state(self.plan, N.ST[name], N.fptr(out)), f"pv1_get_state({name})")
        if name.endswith("_rng") or name.startswith("v1_rng"):
            return out.view(np.uint8)       # 48 raw bytes (one curandStateMRG32k3a) per entry
        return out

    def frames_setup(self, pix_off: np.ndarray, pix_ids: np.ndarray, n_spike_pixel: int, ot: int, odt: float):
        """Framed output (pv1_frames_setup): V1 pixels first (REC_SPIKES), LGN pixels after
        (REC_LGN_FR)."""
        self._pix = (np.ascontiguousarray(pix_off, u32), np.ascontiguousarray(pix_ids, u32))
        self._npix = len(self._pix[0]) - 1
        self._ot = int(ot)
        N.check(self.plan, N.lib.pv1_frames_setup(self.plan, self._npix, int(n_spike_pixel), N.uptr(self._pix[0]),
                                                  N.uptr(self._pix[1]), int(ot), float(odt)), "pv1_frames_setup")

    def frames_collect(self, step0: int, n: int) -> np.ndarray:
        """The frames completed within steps [step0, step0 + n), [k][nPixel]."""
        out = np.empty((n // self._ot + 1, self._npix), f32)
        k = C.c_uint32()
        N.check(self.plan, N.lib.pv1_frames_collect(self.plan, int(step0), int(n), N.fptr(out), C.byref(k)),
                "pv1_frames_collect")
        return out[:k.value]

    def checkpoint(self) -> np.ndarray:
        """The plan's evolving state and step count (pv1_checkpoint_save) as bytes."""
        size = C.c_uint64()
        N.check(self.plan, N.lib.pv1_checkpoint_size(self.plan, C.byref(size)), "pv1_checkpoint_size")
        buf = np.empty(size.value, np.uint8)
        N.check(self.plan, N.lib.pv1_checkpoint_save(self.plan, buf.ctypes.data_as(C.c_void_p), size.value),
                "pv1_checkpoint_save")
        return buf

    def restore(self, buf: np.ndarray):
        """Continues from a checkpoint of a plan of the same configuration and network."""
        b = np.ascontiguousarray(buf, dtype=np.uint8)
        N.check(self.plan, N.lib.pv1_checkpoint_load(self.plan, b.ctypes.data_as(C.c_void_p), b.size),
                "pv1_checkpoint_load")
        self.step = int(np.frombuffer(b[56:64].tobytes(), np.int64)[0])   # the header's step field

    def put_state(self, name: str, arr: np.ndarray):
        if name.endswith("_rng") or name.startswith("v1_rng"):
            a = np.ascontiguousarray(arr, dtype=np.uint8).view(f32)     # raw generator bytes
        else:
            a = np.ascontiguousarray(arr, dtype=f32)
        N.check(self.plan, N.lib.pv1_put_state(self.plan, N.ST[name], N.fptr(a)), f"pv1_put_state({name})")

    def lgn_tables(self):
        nm, ns, nks = self.lgn.nMagno, self.lgn.mSample1D ** 2, self.lgn.sched.mKernelSample
        TW = np.empty((nm, nks), f32)
        SW = np.empty((nm, ns), f32)
        SC = np.empty((2, nm, ns), f32)
        mc = np.empty(self.lgn.nLGN, f32)
        N.check(self.plan, N.lib.pv1_lgn_get_tables(self.plan, N.fptr(TW), N.fptr(SW), N.fptr(SC), N.fptr(mc)),
                "pv1_lgn_get_tables")
        return TW, SW, SC, mc

    def lgn_parvo_tables(self):
        np_, ns, nks = self.lgn.nParvo, self.lgn.nSample1D ** 2, self.lgn.sched.nKernelSample
        TW = np.empty((np_, 2, nks), f32)
        SW = np.empty(ns, f32)
        SC = np.empty((2, np_, 2, ns), f32)
        N.check(self.plan, N.lib.pv1_lgn_get_parvo_tables(self.plan, N.fptr(TW), N.fptr(SW), N.fptr(SC)),
                "pv1_lgn_get_parvo_tables")
        return TW, SW, SC

    def lgn_parvo_spatial(self):
        PS = np.empty((self.stim.frames.shape[0] + 1, 2, self.lgn.nParvo), f32)
        N.check(self.plan, N.lib.pv1_lgn_get_parvo_spatial(self.plan, N.fptr(PS)), "pv1_lgn_get_parvo_spatial")
        return PS

    def lgn_spatial(self):
        S = np.empty((self.stim.frames.shape[0] + 1, self.lgn.nMagno), f32)
        N.check(self.plan, N.lib.pv1_lgn_get_spatial(self.plan, N.fptr(S)), "pv1_lgn_get_spatial")
        return S

    def set_draw_record(self, steps: int, cap: int):
        N.check(self.plan, N.lib.pv1_set_draw_record(self.plan, int(steps), int(cap)), "pv1_set_draw_record")
        self._draw = (steps, cap)

    def fetch_draws(self, kind: int):
        steps, cap = self._draw
        n = self.lgn.nLGN if kind == 0 else self.spec.nV1
        if kind == 1:
            d = np.empty((steps, n), f32)
            N.check(self.plan, N.lib.pv1_fetch_draws(self.plan, kind, N.fptr(d), None), "pv1_fetch_draws")
            return d, None
        d = np.empty((steps, n, cap), f32)
        cnt = np.empty((steps, n), np.int32)
        N.check(self.plan, N.lib.pv1_fetch_draws(self.plan, kind, N.fptr(d), cnt.ctypes.data_as(C.POINTER(C.c_int32))),
                "pv1_fetch_draws")
        return d, cnt

    def close(self):
        if getattr(self, "plan", None):
            N.lib.pv1_plan_destroy(self.plan)
            self.plan = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def host_init_state(spec: V1Spec, seed: int, tonicDep, nLGNperV1, v0, w0, gFF0, gE0, gI0,
                    use_v0=False, tonicMax=None) -> InitState:
    """Initial v, w, g, h drawn on the host exactly as src/patch.cu:4405-4560 does."""
    n = spec.nV1
    cfg = spec.to_struct()
    td = np.ascontiguousarray(tonicDep, dtype=f32)
    nl = np.ascontiguousarray(nLGNperV1, dtype=u32)
    if tonicMax is None:
        tonicMax = float(td.max())
    out = dict(v=np.empty(n, f32), w=np.empty(n, f32), gFF=np.empty(spec.ngFF * n, f32),
               hFF=np.empty(spec.ngFF * n, f32), gE=np.empty(spec.ngE * n, f32),
               hE=np.empty(spec.ngE * n, f32), gI=np.empty(spec.ngI * n, f32),
               hI=np.empty(spec.ngI * n, f32))
    w0a = np.ascontiguousarray(w0 if w0 is not None else np.zeros(2 * spec.nType), dtype=f32)
    g = [np.ascontiguousarray(x, dtype=f32) for x in (gFF0, gE0, gI0)]
    rc = N.lib.pv1_host_init_state(C.byref(cfg), int(seed), N.fptr(td), N.uptr(nl), int(bool(use_v0)),
                                   float(tonicMax), N.fptr(w0a), N.fptr(g[0]), N.fptr(g[1]), N.fptr(g[2]),
                                   N.fptr(out["v"]), N.fptr(out["w"]), N.fptr(out["gFF"]), N.fptr(out["hFF"]),
                                   N.fptr(out["gE"]), N.fptr(out["hE"]), N.fptr(out["gI"]), N.fptr(out["hI"]))
    N.check(None, rc, "pv1_host_init_state")
    if spec.iModel != 1:
        out["w"] = None
    return InitState(**out)
