"""The `patch` run as a library call: config + binary inputs -> GPU simulation -> outputs.

``python -m visual_cortex_gb300 -c patchV1.cfg [-s seed]`` reads the keys of cfg.py, the input
files of formats.py, builds the model objects with the reference's scaling and expansion
rules (src/patch.cu:612-1060 options, 3313-3700 connectivity, 4100-4220 tonic drive, 4278-4301
LGN->V1 lists, 4405-4560 initial state), runs the steps on the GPU and writes rawData,
LGN_fr, LGN_sp and patchV1_cfg with the reference's headers and record order.

Supported: magno and parvo LGN cells in one or two eyes read from the LGN parameter file
(useNewLGN = false), flat or curved retina, initial spikes, synaptic failure (not on
distance-delayed near synapses), learning = 0, no gap junctions, the orientation boost
(nOri with readFeature), snapshots in the reference's layout (resumed, or the initial state with
asInit = true), framed output
(physical V1, visual-field V1 and LGN), minimal output (the sample file).  Anything else
raises ConfigError naming the key.
"""
from __future__ import annotations

import ctypes
import math
import sys
from dataclasses import dataclass

import numpy as np

from . import formats as FM
from .cfg import Config, ConfigError, load, resolve_paths
from .model import InitState, LgnSpec, Seeds, Stimulus, V1Network, V1Spec, host_init_state
from .retina import retina_geometry
from .schedule import make_schedule

f32, u32 = np.float32, np.uint32
DEG = math.pi / 180.0


def _per_type(c: Config, key: str, n: int, required=True, default=None):
    """Size-1 vectors are replicated to n; otherwise the size must be n (src/patch.cu:849-1035)."""
    v = c.values.get(key)
    if v is None:
        if required:
            raise ConfigError(f"option '{key}' is required")
        return list(default) if default is not None else None
    if len(v) == 1:
        return [v[0]] * n
    if len(v) != n:
        raise ConfigError(f"size of {key} is {len(v)} != {n}")
    return list(v)


def _exact(c: Config, key: str, n: int):
    v = c.values.get(key)
    if v is None or len(v) != n:
        raise ConfigError(f"the size of {key} is {0 if v is None else len(v)} != {n}")
    return list(v)


@dataclass
class Model:
    spec: V1Spec
    net: V1Network
    lgn: LgnSpec
    stim: Stimulus
    init: InitState
    seeds: Seeds
    nt: int
    seed: int
    extra: dict


def _check_supported(c: Config):
    bad = []
    if c.learning not in (0, 1, 2, 3, 4):
        bad.append(f"learning = {c.learning} (learning 0-4 are read)")
    if c.learning in (1, 2, 3) and int(c.values.get("nLearnTypeFF_E", 1)) != 1:
        bad.append(f"learning = {c.learning} with nLearnTypeFF_E != 1")
    if c.learning == 2 and int(c.values.get("nLearnTypeFF_I", 1)) > 1:
        bad.append("learning = 2 with nLearnTypeFF_I > 1")
    if c.learning and int(c.learnData_FF) > 1:
        bad.append("learnData_FF = 2 (per-step learning dumps)")
    if c.InhGap:
        bad.append("InhGap (gap junctions)")
    if c.useNewLGN:
        bad.append("useNewLGN = true (LGN parameters drawn from distributions)")
    if c.virtual_LGN or c.LGN_switch or c.reverseInput:
        bad.append("virtual_LGN / LGN_switch / reverseInput")
    if c.fSnapshot and not c.asInit and (c.snapshot_suffix or "") != (c.output_suffix or ""):
        raise ConfigError("to use snapshot to resume simulation, it needs to have the same suffix as the output_suffix")
    if c.manual:
        bad.append("manual connections")
    if bad:
        raise ConfigError("not supported by this library: " + "; ".join(bad))


class _SampleWriter:
    """minimal = true: the sample file (fSample + output suffix).  Header {sampleSize, sample_t0,
    nt*dt, nt, nLGN}; then, for every step s but the last with (s+1)*dt >= sample_t0, its LGN
    spike words, the sampled neurons' spike counts accumulating; then the last step's LGN
    spike words and counts (unconditionally), the sample ids and the counts
    (src/patch.cu:4916-4946, 6122-6137, 7031-7050)."""

    def __init__(self, c: Config, m: Model, P):
        from .cfg import _prefixed, _suffix
        from . import _native as N
        spec = m.spec
        f32 = np.float32
        nE = int(spec.typeAcc[spec.nTypeE - 1])
        ids = np.zeros(max(spec.nblock * nE, 1), np.uint32)
        n = ctypes.c_uint32()
        N.check(None, N.lib.pv1_sample_ids(int(m.seeds.cond) + 1, spec.nblock, spec.blockSize, nE,
                                           int(c.sampleSize), N.uptr(ids), ctypes.byref(n)), "pv1_sample_ids")
        self.ids = ids[:n.value]
        self.counts = np.zeros(len(self.ids), np.uint32)
        self.nt, self.dt, self.t0 = m.nt, f32(c.dt), f32(c.sample_t0)
        self.f = open(_prefixed(c.outputFolder, c.fSample) + _suffix(c.output_suffix), "wb")
        self.f.write(np.array([len(self.ids)], np.uint32).tobytes())
        self.f.write(np.array([self.t0, f32(f32(self.nt) * self.dt)], f32).tobytes())
        self.f.write(np.array([self.nt, m.extra["nLGN"]], np.uint32).tobytes())

    def add(self, s0: int, sinfo: np.ndarray, lgn: np.ndarray):
        for j in range(sinfo.shape[0]):
            s = s0 + j
            if s == self.nt - 1 or np.float32(np.float32(s + 1) * self.dt) >= self.t0:
                w = sinfo[j, self.ids]
                self.counts += np.where(w >= 1, np.floor(w), 0).astype(np.uint32)
                self.f.write(np.ascontiguousarray(lgn[j], np.float32).tobytes())

    def close(self):
        self.f.write(self.ids.astype(np.uint32).tobytes())
        self.f.write(self.counts.tobytes())
        self.f.close()


def _setup_frames(sim, c: Config, m: Model, P):
    """Framed output: the frame sizes of src/patch.cu:2936-2956, the pixel lists of
    getUnderlyingID (physical V1 sheet: src/patch.cu:2959-3037; visual-field V1, all neurons
    ipsilateral without feature files: 3146-3272; visual-field LGN by eye: 3040-3145) in the
    order of the frame buffer (physical, visual V1 ipsi then contra, visual LGN ipsi then
    contra), and the frame interval of :580-584, 5471, with the reference's float arithmetic;
    returns the outputFrame writer."""
    from .cfg import _prefixed, _suffix
    f32 = np.float32
    width = int(m.stim.frames.shape[-1])
    ot = int(f32(c.dot) / f32(c.dt))
    if ot < 1:
        raise ConfigError("dot must be at least one time step")
    odt = f32(float(f32(f32(ot) * f32(c.dt))) / 1000.0)
    offs, idss, sizes, kinds, nSpike = [], [], [], 0, 0

    def add(off, ids):
        base = sum(len(x) for x in idss)
        offs.append((off[1:] if offs else off).astype(np.int64) + base)
        idss.append(ids)

    if c.framePhyV1output:
        phyWidth = int(f32(f32(width) * f32(c.phyWidth_scale)))
        x0, xspan, y0, yspan = FM.read_v1_allpos_spans(P.v1_allpos)
        phyHeight = int(math.ceil(f32(f32(yspan / xspan) * f32(phyWidth))))
        phyHeight += phyHeight % 2
        _, _, pos = FM.read_v1_allpos(P.v1_allpos)
        add(*FM.underlying_ids(pos[:, 0], pos[:, 1], phyWidth, phyHeight, x0, xspan, y0, yspan))
        sizes.append((phyWidth, phyHeight))
        kinds |= 1
    if c.frameVisV1output or c.frameVisLGNoutput:
        visWidth = int(f32(f32(width) * f32(c.visWidth_scale)))
        lx0, lxspan, ly0, lyspan = FM.read_lgn_vpos_spans(P.lgn_vpos)
        visHeight = int(math.ceil(f32(f32(f32(lyspan) / f32(lxspan)) * f32(visWidth))))
        visHeight += visHeight % 2
    if c.frameVisV1output:
        try:
            vx0, vxspan, vy0, vyspan, vx, vy = FM.read_v1_allpos_visual(P.v1_allpos)
        except EOFError as e:
            raise ConfigError("frameVisV1output needs the visual positions in V1_allpos") from e
        feat = m.extra.get("feature")
        ipsi = np.ones(len(vx), bool) if feat is None else feat[0] < 0      # ocular dominance
        add(*FM.underlying_ids(vx, vy, visWidth, visHeight, vx0, vxspan, vy0, vyspan, pick=ipsi))
        add(*FM.underlying_ids(vx, vy, visWidth, visHeight, vx0, vxspan, vy0, vyspan, pick=~ipsi))
        sizes.append((visWidth, visHeight))
        kinds |= 2
    nSpike = sum(len(o) for o in offs) - (1 if offs else 0)
    if c.frameVisLGNoutput:
        nI, nC, _, lx, ly, _ = FM.read_lgn_vpos(P.lgn_vpos)
        add(*FM.underlying_ids(lx[:nI], ly[:nI], visWidth, visHeight, lx0, lxspan, ly0, lyspan, dtype=f32))
        add(*FM.underlying_ids(lx[nI:], ly[nI:], visWidth, visHeight, lx0, lxspan, ly0, lyspan, dtype=f32, n0=nI))
        sizes.append((visWidth, visHeight))
        kinds |= 4
    off = np.concatenate(offs).astype(np.uint32)
    ids = np.concatenate(idss).astype(np.uint32)
    sim.frames_setup(off, ids, nSpike, ot, float(odt))
    fn = _prefixed(c.outputFolder, c.fOutputFrame) + _suffix(c.output_suffix)
    return FM.OutputFrameWriter(fn, c.dt, ot, kinds, sizes)


def _restore(sim, c: Config, m) -> int:
    """Loads the snapshot named by fSnapshot (inputFolder + name + '_' + snapshot_suffix +
    '.bin', src/patch.cu:438-445, 611-613) and returns the step the run starts at.  A snapshot
    in the reference's layout (src/patch.cu:5489-5685) sets the neuron state, tBack, the
    generators and the LGN integrals; with asInit = true it is the initial state of a new run
    (step 0, frame bookkeeping from the start), otherwise the run resumes at its step, whose
    frame bookkeeping must be the one this configuration reaches there.  Its far events in
    flight are not in it (the reference keeps them in host vectors it does not save).  When
    this library wrote the snapshot, its own checkpoint follows the reference's fields, and
    resuming (asInit = false) loads that instead: bit for bit, far events included."""
    from . import _native as N
    from .cfg import _prefixed
    path = _prefixed(c.inputFolder, c.fSnapshot) + "_" + (c.snapshot_suffix or "") + ".bin"
    head = np.fromfile(path, np.uint8, 8)
    if head.tobytes() == b"PV1CKPT\0":           # a bare checkpoint of this library
        if c.asInit:
            raise ConfigError(f"{path}: a checkpoint of this library resumes a run (asInit = false)")
        sim.restore(np.fromfile(path, np.uint8))
        return sim.step
    spec = m.spec
    try:
        nFE, nFI, _ = _learn_types(c) if c.learning else (0, 0, 0)
        snap, trailer = FM.read_reference_snapshot(path, spec.nI * spec.nblock, maxLGN=m.net.maxLGN,
                                                   nE_total=spec.nE * spec.nblock, nFF_E=nFE, nFF_I=nFI)
    except ValueError as e:
        raise ConfigError(str(e)) from None
    sz = snap["sizes"]
    if (snap["learning"] != int(c.learning) or snap["iModel"] != spec.iModel or sz["nV1"] != spec.nV1 or
            sz["nLGN"] != m.lgn.nLGN or sz["ngFF"] != spec.ngFF or sz["ngE"] != spec.ngE or sz["ngI"] != spec.ngI):
        raise ConfigError(f"{path}: patchV1 config is incompatible with the restore file config")
    if not c.asInit and trailer[:8] == b"PV1CKPT\0":
        sim.restore(np.frombuffer(trailer, np.uint8).copy())
        return sim.step
    step = 0 if c.asInit else snap["idx"]["step"]
    if not c.asInit:
        want = m.lgn.sched.snapshot_indices(step, sz["trainDepth"])
        diff = [k for k in FM.SNAPSHOT_INDICES[:-2] if want[k] != snap["idx"][k]]
        if diff:
            raise ConfigError(f"{path}: the snapshot's frame bookkeeping ({', '.join(diff)}) is not this "
                              "configuration's at its step")
    st = snap["state"]
    for k in ("v", "gFF", "hFF", "gE", "hE", "gI", "hI", "dep"):
        sim.put_state(k, st[k])
    if spec.iModel == 1:
        sim.put_state("w", st["w"])
    sim.put_state("tBack", snap["v1"]["tBack"])
    sim.put_state("v1_rng_cond", snap["v1"]["rng_cond"])
    sim.put_state("v1_rng_noisy", snap["v1"]["rng_noisy"])
    sim.put_state("lgn_ltr", snap["lgn"]["ltr"])
    sim.put_state("lgn_lnl", snap["lgn"]["lnl"])
    sim.put_state("lgn_rng", snap["lgn"]["rng"])
    if snap["learn"] is not None:
        # the weights and learning variables; the homeostasis totals stay those of the
        # connectome's weights, as the reference computes them before it restores
        for k in ("sLGN", "ff_post", "ff_pre"):
            sim.put_state(k, snap["learn"][k])
    N.check(sim.plan, N.lib.pv1_set_step(sim.plan, int(step)), "pv1_set_step")
    sim.step = int(step)
    return int(step)


def _learn_types(c: Config):
    """(nLearnTypeFF_E, nLearnTypeFF_I, nLearnTypeE) after the learning mode's overrides
    (src/patch.cu:1160-1176): 1 drops FF->I, 3 keeps FF->E alone, 4 drops both FF types."""
    v, mode = c.values, int(c.learning)
    nE = int(v.get("nLearnTypeFF_E", 1))
    nI = int(v.get("nLearnTypeFF_I", 1))
    nC = int(v.get("nLearnTypeE", 1))
    if mode in (1, 3):
        nI = 0
    if mode == 3:
        nC = 0
    if mode == 4:
        nE = nI = 0
    return nE, nI, nC


def _ff_learning(c: Config, sRatioLGN):
    """The FFLearning of learning 1-4 from the cfg (src/patch.cu:1092-1330): the FF->E type is
    element [0] of the triplet-rule arrays (a single value stands for every type), the FF->I
    type element [nLearnTypeFF_E] with tauAvg[1], targetFR[1] and sRatioLGN[1]; tauAvg and
    targetFR have 1 or 2 values (E, I); the Q arrays must agree in size even though Q learning
    is off; with cortical E types (nLearnTypeE > 0) the excitatory filtered rate of the delivery
    decays with tauAvg[0] (learnE's tau[3 n]), with none it is zeroed each step."""
    from .model import FFLearning
    v, mode = c.values, int(c.learning)
    nE, nI, nC = _learn_types(c)
    nFF = nE + nI

    def arr(key, required=True):
        a = [float(x) for x in (v.get(key) or [])]
        if not a and required:
            raise ConfigError(f"learning = {mode} needs '{key}'")
        return a

    tauAvg, targetFR = arr("tauAvg"), arr("targetFR")
    for key, a in (("tauAvg", tauAvg), ("targetFR", targetFR)):
        if len(a) not in (1, 2):
            raise ConfigError(f"{key} must have 1 or 2 values (E, I), not {len(a)}")
        a += a[:1] * (2 - len(a))
    sizes = [len(v.get(k) or []) for k in ("tauQ", "A_Q", "gmaxQ", "gminQ")]
    if len(set(sizes)) != 1:
        raise ConfigError(f"size of tauQ: {sizes[0]} should be the same as A_Q: {sizes[1]}")
    if not bool(v.get("symQ", True)) and sizes[0] % 2:
        raise ConfigError(f"size of array tauQ: {sizes[0]} must be even (or single-value)")
    tauTrip = arr("tauTrip", nFF + nC > 0)
    nTrip = len(tauTrip)
    trip = {k: arr(k, False) for k in ("r_LTD", "tauLTD", "tauLTP")}
    for key, a in trip.items():
        if len(a) != nTrip:
            raise ConfigError(f"the size of {key} should be the same as tauTrip: {nTrip}")
    if nTrip == 1:
        if nE > 1 or nI > 1 or nC > 1:
            raise ConfigError(f"tauLTP, tauLTD, tauTrip have size 1, but nLearnTypeFF_E: {nE}, nLearnTypeFF_I: "
                              f"{nI}, nLearnTypeE: {nC} are inconsistent")
    elif nC + nFF > nTrip:
        raise ConfigError(f"nLearnTypeE {nC} + nLearnTypeFF {nFF} exceed the {nTrip} triplet rules")
    if nC > 0:
        for key in ("gmaxE", "gminE"):
            a = v.get(key) or []
            if len(a) > nC or 1 < len(a) < nC:
                raise ConfigError(f"{key} either has size 1 or size {nC}")
            if not a:
                raise ConfigError(f"learning = {mode} with nLearnTypeE > 0 needs '{key}'")
        if not v.get("A_V1"):
            raise ConfigError(f"learning = {mode} with nLearnTypeE > 0 needs 'A_V1'")
    gmax, gmin, A = arr("gmaxLGN", nFF > 0), arr("gminLGN", nFF > 0), arr("A_LGN", nFF > 0)
    for key, a in (("gmaxLGN", gmax), ("gminLGN", gmin)):
        if len(a) > nFF and nFF:
            raise ConfigError(f"array size of {key} cannot be bigger than nLearnTypeFF {nFF}")
        if 1 < len(a) < nFF:
            raise ConfigError(f"{key} either has size 1 or size {nFF}")
        a += a[:1] * (nFF - len(a))
    if len(A) < nFF:
        raise ConfigError(f"A_LGN needs {nFF} values")
    for key in ("r_LTD", "tauLTD", "tauLTP"):
        trip[key] += trip[key][:1] * (max(nFF, 1) - len(trip[key]))
    tauTrip = tauTrip + tauTrip[:1] * (max(nFF, 1) - len(tauTrip))
    sr = [float(x) for x in sRatioLGN]
    kw = {}
    if nE:
        kw.update(tauLTP=trip["tauLTP"][0], tauLTD=trip["tauLTD"][0], tauTrip=tauTrip[0], A_LGN=A[0],
                  r_LTD=trip["r_LTD"][0], gmaxLGN=gmax[0], gminLGN=gmin[0])
    else:
        kw.update(tauLTP=0.0, tauLTD=0.0, tauTrip=0.0, A_LGN=0.0, r_LTD=0.0, gmaxLGN=0.0, gminLGN=0.0)
    if nI:
        if len(sr) < 2:
            raise ConfigError("learning = 2 with nLearnTypeFF_I = 1 reads sRatioLGN[1]")
        k = nE
        kw.update(tauLTP_I=trip["tauLTP"][k], tauLTD_I=trip["tauLTD"][k], tauTrip_I=tauTrip[k],
                  tauAvg_I=tauAvg[1], targetFR_I=targetFR[1], A_LGN_I=A[k], r_LTD_I=trip["r_LTD"][k],
                  gmaxLGN_I=gmax[k], gminLGN_I=gmin[k], sRatioLGN_I=sr[1])
    return FFLearning(tauAvg=tauAvg[0], targetFR=targetFR[0], sRatioLGN=sr[0],
                      decayTimeHomeoFF=float(c.decayTimeHomeoFF), FF_InfRatio=float(c.FF_InfRatio),
                      applyHomeo=int(c.applyHomeo), symmetricHomeo=bool(c.symmetricHomeo),
                      rebound=bool(c.rebound), learning=mode, nLearnTypeFF_E=max(nE, 1), nLearnTypeFF_I=nI,
                      tauAvgCortical=tauAvg[0] if (mode != 3 and nC > 0) else 0.0, **kw)


def _ltd_ratio1(A_LGN, sRatio, r_LTD, tauAvg, tauTrip, tauLTD, targetFR, tauLTP):
    f = np.float32
    A_LTP = f(f(A_LGN) * f(sRatio))
    A_ratio = f(f(r_LTD) * A_LTP)
    if targetFR > 0:
        tas = f(float(f(tauAvg)) / 1000.0)
        q = f(f(tauTrip) / f(f(tauLTD) * f(tas * tas)))
        A_ratio = f(float(A_ratio) * (float(q) / 1000.0 / float(f(targetFR))))
    return float(f(A_ratio * f(tauLTP)))


def _ltd_ratio(learn, nE: int = 1, nI: int = 0):
    """A_ratio * tauLTP of each FF type, the dsLGN header's LTD ratios (src/patch.cu:4804-4811):
    learnFF_post's A_ratio (src/condShape.h:137-152) in float with its double literals."""
    out = []
    if nE:
        out.append(_ltd_ratio1(learn.A_LGN, learn.sRatioLGN, learn.r_LTD, learn.tauAvg, learn.tauTrip, learn.tauLTD,
                               learn.targetFR, learn.tauLTP))
    if nI:
        out.append(_ltd_ratio1(learn.A_LGN_I, learn.sRatioLGN_I, learn.r_LTD_I, learn.tauAvg_I, learn.tauTrip_I,
                               learn.tauLTD_I, learn.targetFR_I, learn.tauLTP_I))
    return out


def _learn_state(sim, m):
    return dict(sLGN=sim.state("sLGN"), ff_post=sim.state("ff_post"), ff_pre=sim.state("ff_pre"))


def _write_snapshot(sim, c: Config, m, history, previous, log):
    """snapShot_<time>_<output suffix>.bin in the output folder (the reference writes it in the
    working directory, src/patch.cu:6793-6912), in the reference's layout -- `history` holds the
    spike words of the last steps for its spike-word ring -- followed by this library's own
    checkpoint; the previous one is removed when delPrevSnapshot."""
    import os
    import time
    from .cfg import _prefixed
    name = _prefixed(c.outputFolder, f"snapShot_{int(time.time())}") + "_" + (c.output_suffix or "") + ".bin"
    trailer = sim.checkpoint().tobytes()        # applies the last step's delivery first
    spec, depth = m.spec, int(m.seeds.trainDepth)
    q = int(sim.step)
    ring = np.empty((depth, spec.nV1), np.float32)
    for slot in range(depth):
        # slot s holds the newest step t < q with t % depth == s (the initial v before step 0)
        t = q - 1 - ((q - 1 - slot) % depth)
        ring[slot] = history.get(t, m.init.v)
    state = {k: sim.state(k) for k in ("dep", "v", "gFF", "hFF", "gE", "gI", "hE", "hI")}
    if spec.iModel == 1:
        state["w"] = sim.state("w")
    state["gap"] = np.zeros(spec.nI * spec.nblock, np.float32)
    learning = int(c.learning)
    FM.write_reference_snapshot(
        name, m.lgn.sched.snapshot_indices(q, depth), spec.iModel, learning,
        dict(nV1=spec.nV1, nLGN=m.lgn.nLGN, ngFF=spec.ngFF, ngE=spec.ngE, ngI=spec.ngI, nType=spec.nType,
             trainDepth=depth),
        dict(ltr=sim.state("lgn_ltr"), lnl=sim.state("lgn_lnl"), rng=sim.state("lgn_rng")),
        dict(rng_cond=sim.state("v1_rng_cond"), rng_noisy=sim.state("v1_rng_noisy"), tBack=sim.state("tBack")),
        ring, state, trailer, learn=_learn_state(sim, m) if learning else None)
    if previous and previous != name and c.delPrevSnapshot and os.path.exists(previous):
        os.remove(previous)
    log(f"saved a snapshot in {name}")
    return name


def _orientation_boost(c: Config, P, nType, nV1, blockSize, ptype):
    """The orientation boost of the tonic drive and the V1 feature file (src/patch.cu:2842-2930,
    4155-4210).  readFeature is forced on by a non-empty boostOri or iOri when nOri > 0; the
    feature file is read whenever readFeature ends up on (its ocular dominance also splits the
    visual-field V1 frames, src/patch.cu:3157-3170), and the reference then asserts nOri > 0,
    iOri and boostOri (src/patch.cu:2927-2929; its build scripts do not define NDEBUG), which
    is a ConfigError here.  With boostOri given, readFeature on and nOri > 0, neuron i of type t
    is scaled by base + (1 - base) * (exp(k (cos 2 pi dOri - 1)) - 1 + A) / A, A = 1 - exp(-2k),
    (base, k) = boostOri[t], dOri its preferred orientation (feature 1) minus fOri[t] wrapped to
    [-1/2, 1/2], fOri[t] = (iOri[t] % nOri)/nOri + 1/2 (0 without iOri, when k is forced to 0);
    1 otherwise.  Returns (boost [nV1], features or None)."""
    from .cfg import _prefixed, _suffix
    nOri = int(c.values.get("nOri") or 0)
    read_feature = bool(c.readFeature)
    bo = [float(x) for x in (c.values.get("boostOri") or [])]
    io = [int(x) for x in (c.values.get("iOri") or [])]
    fOri = [f32(0.0)] * nType
    if nOri > 0:
        if bo:
            if len(bo) not in (2, 2 * nType):
                raise ConfigError("boostOri need 2 x nType elements: [baseline, std] x nType")
            read_feature = True
            if len(bo) == 2 and nType > 1:
                bo = bo * nType
            if any(bo[2 * t + 1] != 0 for t in range(nType)) and not io:
                raise ConfigError("when boostOri[std] is set, iOri needs to be set")
        if io:
            if len(io) not in (1, nType):
                raise ConfigError("iOri need 1 or nType elements")
            read_feature = True
            if len(io) == 1 and nType > 1:
                io = io * nType
            fOri = [f32(math.fmod(float(f32(io[t] % nOri) / f32(nOri)) + 0.5, 1.0)) for t in range(nType)]
        else:
            for q in range(1, len(bo), 2):
                bo[q] = 0.0
    else:
        for q in range(1, len(bo), 2):
            bo[q] = 0.0
    if not read_feature:
        return np.ones(nV1, f32), None
    feat = FM.read_v1_feature(_prefixed(c.resourceFolder, c.fV1_feature) + _suffix(c.res_suffix), nV1)
    if not (nOri > 0 and io and bo):
        raise ConfigError("readFeature = true needs nOri > 0, iOri and boostOri (the reference asserts them "
                          "after reading the feature file); set readFeature = false otherwise")
    boost = np.ones(nV1, f32)
    for i in range(nV1):
        t = int(ptype[i % blockSize])
        d = f32(feat[1, i] - fOri[t])
        if d > 0.5:
            d = f32(1 - d)
        if d < -0.5:
            d = f32(1 + d)
        base, k = f32(bo[2 * t]), f32(bo[2 * t + 1])
        amp = f32(1 - base)
        vm = f32(1 - np.exp(f32(-2 * k)))
        if vm == 0:
            boost[i] = base
        else:
            cosd = f32(math.cos(float(d) * math.pi * 2))
            boost[i] = f32(base + amp * f32(f32(f32(np.exp(f32(k * f32(cosd - 1)))) - 1 + vm) / vm))
    return boost, feat


def _sp0(c: Config, nTypeE: int, nTypeI: int):
    """Initial spike chances per step [type][2] from spE0/spI0 (Hz), src/patch.cu:810-837;
    None when every one is 0."""
    from .synth import sp0_chances
    rates = []
    for key, nt in (("spE0", nTypeE), ("spI0", nTypeI)):
        v = getattr(c, key)
        if v is None:
            v = [0.0] * (2 * nt)
        elif len(v) != 2 * nt:
            raise ConfigError(f"the size of {key} has size of {len(v)} != {nt}x 2")
        rates += list(v)
    sp0 = sp0_chances(rates, c.dt)
    return tuple(sp0) if any(x > 0 for x in sp0) else None


def _max_near_distance(conMat, delayMat, nblock, nChunk):
    """maxDistance of src/patch.cu:3808-3812: findDisConMax over each chunk of blocks, always
    over the first remainChunkSize blocks' worth of elements of the chunk (the loop keeps the
    chunk length of the last chunk), a[0] counted unconditionally."""
    nChunk = min(nChunk, nblock)
    split = nblock % nChunk
    remain = nblock // nChunk
    big = remain + (1 if split > 0 else 0)
    per_block = conMat[0].size
    n = remain * per_block
    a_all, b_all = delayMat.reshape(-1), conMat.reshape(-1)
    best = f32(0.0)
    start = 0
    for i in range(nChunk):
        a = a_all[start * per_block:start * per_block + n]
        b = b_all[start * per_block:start * per_block + n]
        m = a[0]
        sel = a[1:][b[1:] > 0]
        if sel.size:
            m = max(m, sel.max())
        best = max(best, f32(m))
        start += big if i < split else remain
    return float(best)


def build(c: Config) -> Model:
    _check_supported(c)
    P = resolve_paths(c)
    seed = int(c.values.get("seed", 0) or 0)
    nType, nTypeI, typeAcc = FM.read_connectome_cfg(P.connectome_cfg)
    nblock, blockSize, pos = FM.read_v1_allpos(P.v1_allpos)
    nV1 = nblock * blockSize
    nh = list(c.values.get("nTypeHierarchy") or [])
    if len(nh) != 2 or nh[0] + nh[1] != nType or nh[1] != nTypeI:
        raise ConfigError("nTypeHierarchy inconsistent with the connectome's nType/nTypeI")
    nTypeE = nh[0]
    nE = int(typeAcc[nTypeE - 1])
    if int(typeAcc[-1]) != blockSize:
        raise ConfigError("typeAccCount does not end at blockSize")
    synPerCon = _exact(c, "synPerCon", nType * nType)
    synPerConFF = _per_type(c, "synPerConFF", nType)
    sRatioV1 = _per_type(c, "sRatioV1", nType * nType)
    sRatioLGN = _per_type(c, "sRatioLGN", nType)
    grFF, gdFF = list(c.riseTimeFF), list(c.decayTimeFF)
    grE, gdE = list(c.riseTimeE), list(c.decayTimeE)
    grI, gdI = list(c.riseTimeI), list(c.decayTimeI)
    ngFF, ngE, ngI = len(grFF), len(grE), len(grI)
    if len(gdFF) != ngFF or len(gdE) != ngE or len(gdI) != ngI:
        raise ConfigError("rise and decay time lists differ in size")
    pFF = _exact(c, "pFF", nType * ngFF)
    pE = _exact(c, "pE", nType * ngE)
    pI = _exact(c, "pI", nType * ngI)
    gFF0 = _exact(c, "gFF0", nType * ngFF * 4)
    gE0 = _exact(c, "gE0", nType * ngE * 4)
    gI0 = _exact(c, "gI0", nType * ngI * 4)
    if c.noFarDelay and not c.noDelay:
        raise ConfigError("noFarDelay = 1 requires noDelay = 1")
    tonicDep = _per_type(c, "tonicDep", nType)
    noisyDep = _per_type(c, "noisyDep", nType)
    minTonicRatio = _per_type(c, "minTonicRatio", nType, required=False, default=[0.0] * nType)
    synFailFF = _per_type(c, "synFailFF", nType)
    synFail = [max(0.0, x) for x in _exact(c, "synFail", nType * nType)]
    vR = _per_type(c, "vR", nType)
    vThres = _per_type(c, "vThres", nType)
    vT = _per_type(c, "vT", nType) if c.iModel == 1 else list(vThres)
    Cm = _per_type(c, "C", nType)
    gL = _per_type(c, "gL", nType)
    tRef = _per_type(c, "tRef", nType)
    if c.iModel == 1:
        deltaT, tau_w = _per_type(c, "deltaT", nType), _per_type(c, "tau_w", nType)
        a, b = _per_type(c, "a", nType), _per_type(c, "b", nType)
    else:
        deltaT, tau_w, a, b = [1.0] * nType, [1.0] * nType, [0.0] * nType, [0.0] * nType
    spec = V1Spec(
        nblock=nblock, blockSize=blockSize, typeAcc=[int(x) for x in typeAcc], nTypeE=nTypeE,
        ngFF=ngFF, ngE=ngE, ngI=ngI, dt=c.dt, riseFF=grFF, decayFF=gdFF, riseE=grE, decayE=gdE,
        riseI=grI, decayI=gdI, vR=vR, vThres=vThres, gL=gL, C=Cm, tRef=tRef, vT=vT,
        deltaT=deltaT, tau_w=tau_w, a=a, b=b, pFF=pFF, pE=pE, pI=pI, synFail=synFail,
        synPerCon=synPerCon, synFailFF=synFailFF, synPerConFF=synPerConFF, noisyDep=noisyDep,
        tau_noise=c.tau_noise, noiseOnTonic=c.noiseOnTonic, iModel=c.iModel, noDelay=c.noDelay,
        noFarDelay=c.noFarDelay, speedOfThought=c.speedOfThought, hWrite=c.hWrite)
    ptype = spec.type_of(np.arange(blockSize))

    # near connectivity, scaled by sRatioV1[pre type * 2 + post type] (src/patch.cu:3655-3680)
    nnb, conMat = FM.read_mat(P.conMat, nblock, blockSize)
    nnb2, delayMat = FM.read_mat(P.delayMat, nblock, blockSize)
    if nnb2 != nnb:
        raise ConfigError("conMat and delayMat does not match")
    nNear, nbId = FM.read_neighbor_block(P.neighborBlock, nblock, nnb)
    scale = np.array(sRatioV1, f32)[ptype[:, None] * 2 + ptype[None, :]].astype(f32)
    for bb in range(nblock):
        for k in range(int(nNear[bb])):
            conMat[bb, k] = conMat[bb, k] * scale
    maxDistance = _max_near_distance(conMat, delayMat, nblock, c.nChunk)
    trainDepth = int(math.ceil(f32(f32(maxDistance) / f32(c.speedOfThought)) / f32(c.dt))) + 1

    # far connectivity (src/patch.cu:3313-3352)
    nVec, vecID, conVec, delayVec = FM.read_v1_vec(P.v1_vec, nV1)
    post = np.repeat(np.arange(nV1), nVec.astype(np.int64))
    jt = np.where(vecID % blockSize < nE, 0, 1)
    it = np.where(post % blockSize < nE, 0, 1)
    conVec = (conVec * np.array(sRatioV1, f32)[jt * 2 + it]).astype(f32)

    # LGN -> V1 (src/patch.h:30-77, src/util/util.h:162-186)
    ids = FM.read_list_of_lists(P.lgn_v1_id, u32)
    sl, maxList = FM.read_list_of_lists(P.lgn_v1_s, np.float32, with_max=True)
    if len(ids) != nV1 or len(sl) != nV1:
        raise ConfigError("LGN_V1 lists do not hold nV1 lists")
    nL = np.array([len(x) for x in ids], u32)
    lgnId = np.zeros((maxList, nV1), u32)
    sLGN = np.zeros((maxList, nV1), f32)
    rtype = spec.type_of(np.arange(nV1) % int(typeAcc[-1]))
    for i in range(nV1):
        lgnId[:len(ids[i]), i] = ids[i]
        sLGN[:len(sl[i]), i] = (sl[i] * f32(sRatioLGN[rtype[i]])).astype(f32)

    # tonic drive (src/patch.cu:4119-4220): CmoreDep scales by the feed-forward ratio
    ffRatio = FM.read_con_stats(P.conStats, nType, nV1)
    acc0 = [0] + [int(x) for x in typeAcc]
    mn = np.ones(nType, f32)
    mx = np.zeros(nType, f32)
    for bb in range(nblock):
        for j in range(nType):
            seg = ffRatio[bb * blockSize + acc0[j]:bb * blockSize + acc0[j + 1]]
            if seg.size:
                mx[j] = max(mx[j], seg.max())
                mn[j] = min(mn[j], seg.min())
    boost, feature = _orientation_boost(c, P, nType, nV1, blockSize, ptype)
    iTonic = np.zeros(nV1, f32)
    for i in range(nV1):
        t = int(ptype[i % blockSize])
        td = f32(f32(tonicDep[t]) * boost[i])
        if c.CmoreDep and mx[t] > mn[t]:
            rel = f32(1) - ffRatio[i]
            lo, hi = f32(1) - mx[t], f32(1) - mn[t]
            mr = f32(minTonicRatio[t])
            iTonic[i] = td * f32(mr + (f32(1) - mr) * ((rel - lo) / (hi - lo)))
        else:
            iTonic[i] = td
    net = V1Network(nLGNperV1=nL, lgnId=lgnId, sLGN=sLGN, nNearNB=nNear.astype(u32),
                    nbId=nbId, conMat=conMat, nVec=nVec, vecID=vecID, conVec=conVec,
                    delayVec=delayVec, tonicDep=iTonic, delayMat=None if c.noDelay else delayMat)

    # LGN cells (src/patch.cu:1523-1640, 2505-2530) and the stimulus
    stim_f = FM.read_stimulus(P.stimulus)
    # src/patch.cu:1457-1468: a flat retina reads a one-eye stimulus, a curved one two eyes
    if c.flat_retina and stim_f.neye != 1:
        raise ConfigError("flat retina shall receive one eye stimulus")
    if not c.flat_retina and stim_f.neye != 2:
        raise ConfigError("non-flat retina shall receive two eye stimulus")
    nI_, nC_, max_ecc, _, _, LGNtype = FM.read_lgn_vpos(P.lgn_vpos)
    nLGN = nI_ + nC_
    if max_ecc > stim_f.range:
        raise ConfigError(f"max_ecc: {max_ecc} must not be larger than {stim_f.range}")
    # cell order parvo_I, magno_I, parvo_C, magno_C (src/patch.cu:1723-1750)
    parvo = np.asarray(LGNtype) < 4
    nParvo_I, nParvo_C = int(parvo[:nI_].sum()), int(parvo[nI_:].sum())
    if not (np.all(parvo[:nParvo_I]) and np.all(parvo[nI_:nI_ + nParvo_C])):
        raise ConfigError("LGN_vpos: parvo cells must come before the magno cells of each eye")
    prm = FM.read_lgn_params(P.lgn, nLGN)
    geo = retina_geometry(max_ecc, stim_f.range, stim_f.buffer, bool(c.flat_retina))
    sched = make_schedule(c.dt, c.frameRate, c.tau, c.mau, c.nKernelSample, c.mKernelSample)
    lgn = LgnSpec(nParvo_I=nParvo_I, nMagno_I=nI_ - nParvo_I, nParvo_C=nParvo_C, nMagno_C=nC_ - nParvo_C,
                  mSample1D=c.mSpatialSample1D, sched=sched,
                  **{k: prm[k] for k in FM.LGN_FIELDS2 + FM.LGN_FIELDS1 + ("coneType",)},
                  normViewDistance=geo["normViewDistance"], L_x0=geo["L_x0"], L_y0=geo["L_y0"], R_x0=geo["R_x0"],
                  R_y0=geo["R_y0"], nsig=c.nsig, convolRatio=c.convolRatio, frRatio=c.frRatioLGN,
                  flat_retina=bool(c.flat_retina),
                  nSample1D=c.nSpatialSample1D, covariant=prm["covariant"])
    stim = Stimulus(frames=stim_f.frames, init_LMS=stim_f.init_LMS)

    # initial state and the seed sequence of src/patch.cu (logRand_init, host engines, init)
    s_lgn = seed
    s_init = seed + 1 + nV1
    s_sp = s_init + 1
    w0 = _exact(c, "w0", nType * 2) if c.iModel == 1 else [0.0] * (2 * nType)
    v0 = _exact(c, "v0", nType * 2) if c.use_v0 else None
    init = host_init_state(spec, s_init, iTonic, nL, v0, w0, gFF0, gE0, gI0, use_v0=c.use_v0,
                           tonicMax=float(iTonic.max()))
    seeds = Seeds(lgn=s_lgn, cond=s_sp, trainDepth=max(trainDepth, 1), sp0=_sp0(c, nTypeE, nTypeI),
                  SCsplit=int(c.SCsplit), nChunk=int(c.nChunk))
    extra = dict(nType=nType, nTypeE=nTypeE, nTypeI=nTypeI, typeAcc=typeAcc, nLGN=nLGN, feature=feature,
                 normViewDistance=geo["normViewDistance"], stimulus_filename=P.stimulus, sRatioV1=sRatioV1,
                 sRatioLGN=sRatioLGN, tonicDep=tonicDep, noisyDep=noisyDep, vR=vR,
                 vThres=vThres, gL=gL, vT=vT, C=Cm, tRef=tRef, a=a, b=b, tau_w=tau_w,
                 deltaT=deltaT, synFail=synFail, synFailFF=synFailFF, paths=P)
    return Model(spec, net, lgn, stim, init, seeds, int(c.nt), seed, extra)


def run(c: Config, chunk: int = 512, log=print) -> Model:
    """Runs the configured number of steps and writes the outputs the options ask for."""
    from . import _native as N
    from .model import Simulation
    m = build(c)
    P = m.extra["paths"]
    spec = m.spec
    sim = Simulation(m.spec, m.net, m.lgn, m.stim, m.init, m.seeds)
    try:
        learn = None
        if c.learning:
            learn = _ff_learning(c, m.extra["sRatioLGN"])
            sim.set_ff_learning(learn)
        minimal = bool(c.minimal)
        flags = (N.REC_RAW if c.rawData else 0) | (N.REC_LGN_SP if c.getLGN_sp else 0) | \
                (N.REC_LGN_FR if c.saveLGN_fr else 0)
        sample = None
        if minimal:
            # only the sample file (src/patch.cu:4916-4946): no rawData, LGN_sp, LGN_fr, frames
            flags = N.REC_RAW | N.REC_LGN_SP
            sample = _SampleWriter(c, m, P)
        raw = lsp = lfr = None
        nLGN = m.extra["nLGN"]
        if c.saveLGN_fr and not minimal:
            lfr = FM.LgnFrWriter(P.lgn_fr, m.nt, nLGN)
        if c.rawData and not minimal:
            raw = FM.RawDataWriter(P.raw, spec.dt, m.nt, spec.nV1, spec.iModel,
                                   spec.nI * spec.nblock, spec.hWrite, spec.ngFF, spec.ngE, spec.ngI)
        if c.getLGN_sp and not minimal:
            lsp = FM.LgnSpWriter(P.lgn_sp, spec.dt, m.nt, nLGN)
        frames = None
        if (c.framePhyV1output or c.frameVisV1output or c.frameVisLGNoutput) and not minimal:
            if c.framePhyV1output or c.frameVisV1output:
                flags |= N.REC_SPIKES
            if c.frameVisLGNoutput:
                flags |= N.REC_LGN_FR
            frames = _setup_frames(sim, c, m, P)
        slgn = dslgn = None
        sample_every = max(int(c.sampleInterval_LGN_V1), 1)
        if learn is not None and int(c.learnData_FF) == 1 and not minimal:
            nFE, nFI, _ = _learn_types(c)
            sr2 = (list(m.extra["sRatioLGN"]) * 2)[:2]
            gm = [float(x) for x in (c.values.get("gmaxLGN") or [])]
            gm += gm[:1] * (nFE + nFI - len(gm))
            slgn = FM.SLgnWriter(P.slgn, m.nt, sample_every, spec.dt, spec.nV1, m.net.maxLGN, sr2, nFE, nFI,
                                 gm, float(c.FF_InfRatio))
            if c.store_dsLGN:
                tfr = (list(c.values.get("targetFR")) * 2)[:2]
                dslgn = FM.DsLgnWriter(P.dslgn, m.nt, sample_every, spec.dt, spec.nV1, m.net.maxLGN, sr2, nFE, nFI,
                                       c.values.get("A_LGN") or [], _ltd_ratio(learn, nFE, nFI), tfr,
                                       int(c.learnData_FF))
        snaps = not minimal
        if snaps:
            flags |= N.REC_SPIKES          # the spike-word ring of the snapshots
        if flags:
            sim.set_record(flags, chunk + 1)
        base = 0
        if c.fSnapshot:
            base = _restore(sim, c, m)
            log(("initial state from" if c.asInit else "resumed from") + f" step {base}")
        done = 0
        interval = max(int(c.snapshotInterval), 1)
        last_snap = None
        history = {}
        depth = int(m.seeds.trainDepth)
        while done < m.nt:
            k = min(chunk, m.nt - done, interval - done % interval)
            if slgn is not None:
                k = min(k, sample_every - done % sample_every)
            sim.run(k)
            if snaps:
                first = base + done + max(0, k - depth)
                for q, row in enumerate(sim.fetch_spikes(first, min(k, depth))):
                    history[first + q] = row
                for t in [t for t in history if t < base + done + k - depth]:
                    del history[t]
            if sample is not None:
                r, sp, _ = sim.fetch_records(base + done, k, raw=True, lgn_sp=True, lgn_fr=False)
                sample.add(done, r[:, :spec.nV1], sp)
            elif flags:
                r, sp, fr = sim.fetch_records(base + done, k, raw=raw is not None, lgn_sp=lsp is not None,
                                              lgn_fr=lfr is not None)
                if raw is not None:
                    raw.write(r)
                if lsp is not None:
                    lsp.write(sp)
                if lfr is not None:
                    lfr.write(fr)
            if frames is not None:
                frames.write(sim.frames_collect(base + done, k))
            done += k
            if slgn is not None and done % sample_every == 0:
                slgn.write(sim.state("sLGN"))
                if dslgn is not None:
                    # vAvgE [nEt][2] and vAvgI follow the FF types' post traces
                    post = sim.state("ff_post")
                    nEt, nIt = spec.nE * spec.nblock, spec.nI * spec.nblock
                    a = post.size - 2 * nEt - nIt
                    dslgn.write(post[a:a + 2 * nEt], post[a + 2 * nEt:])
            if not c.minimal and (done % interval == 0 or done == m.nt):
                last_snap = _write_snapshot(sim, c, m, history, last_snap, log)
        for w in (raw, lsp, lfr, frames, sample, slgn, dslgn):
            if w is not None:
                w.close()
    finally:
        sim.close()
    e = m.extra
    if c.minimal:
        log(f"simulation for {c.output_suffix} done: {m.nt} steps of {spec.nV1} V1 neurons (minimal)")
        return m
    with open(P.patchV1_cfg, "wb") as f:
        vals = dict(c.values)
        vals.update(vR=e["vR"], vThres=e["vThres"], gL=e["gL"], vT=e["vT"], C=e["C"],
                    tRef=e["tRef"], a=e["a"], b=e["b"], tau_w=e["tau_w"], deltaT=e["deltaT"],
                    sRatioLGN=e["sRatioLGN"], sRatioV1=e["sRatioV1"], tonicDep=e["tonicDep"],
                    noisyDep=e["noisyDep"], synFail=e["synFail"], synFailFF=e["synFailFF"])
        for k in ("spE0", "spI0", "v0", "w0", "gFF0", "gE0", "gI0", "riseTimeFF",
                  "decayTimeFF", "riseTimeE", "decayTimeE", "riseTimeI", "decayTimeI", "pFF",
                  "pE", "pI"):
            vals.setdefault(k, None)
        f.write(FM.patchv1_cfg_bytes(
            vals, vL=spec.vL, vE=spec.vE, vI=spec.vI, nType=e["nType"], nTypeE=e["nTypeE"],
            nTypeI=e["nTypeI"], typeAcc=e["typeAcc"], stimulus_filename=e["stimulus_filename"],
            nLGN=e["nLGN"], nV1=spec.nV1, normViewDistance=e["normViewDistance"], L_x0=0.5,
            L_y0=0.5, R_x0=1.0, R_y0=1.0, ngFF=spec.ngFF, ngE=spec.ngE, ngI=spec.ngI,
            seed=m.seed))
    log(f"simulation for {c.output_suffix} done: {m.nt} steps of {spec.nV1} V1 neurons")
    return m


def main(argv=None):
    argv = sys.argv[1:] if argv is None else argv
    c = load(argv)
    run(c)
    return 0
