"""CPU oracle of the patchV1 hot path -- TEST INFRASTRUCTURE, not part of the product.

Only tests/, __graft_entry__.smoke() and the CPU-baseline leg of bench.py use this package,
as the oracle the GPU results are compared with.  pv1_oracle.c restates the reference's kernels on the CPU; this module builds
it with gcc and drives it in the reference's own per-step order
(src/patch.cu:5966-6880): LGN convolution -> LGN spikes -> V1 step -> near delivery -> far
delivery.  Random draws are supplied by the caller (recorded from the GPU run under test):
cuRAND is not re-derived here.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD = HERE.parent / "_build" / "oracle"
LIB = BUILD / "liboracle.so"
f32 = np.float32


def build(force: bool = False) -> Path:
    src = HERE / "pv1_oracle.c"
    hdr = HERE.parent / "include" / "patchv1_gb300.h"
    if not force and LIB.exists() and LIB.stat().st_mtime > max(src.stat().st_mtime, hdr.stat().st_mtime):
        return LIB
    BUILD.mkdir(parents=True, exist_ok=True)
    tmp = LIB.with_suffix(".tmp.so")
    cmd = ["gcc", "-O2", "-fPIC", "-shared", "-fopenmp", "-ffp-contract=off", "-std=c11",
           "-D_GNU_SOURCE", "-o", str(tmp), str(src), "-lm"]
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + res.stderr)
    os.replace(tmp, LIB)
    return LIB


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = C.CDLL(str(LIB))
        P = C.c_void_p
        FP = C.POINTER(C.c_float)
        UP = C.POINTER(C.c_uint32)
        IP = C.POINTER(C.c_int32)
        L.orc_lgn_setup.argtypes = [P, P, FP, FP, FP, FP, FP, FP, FP]
        L.orc_lgn_spatial.argtypes = [C.c_int, C.c_int, FP, FP, UP, FP, C.c_int, C.c_int, C.c_int, C.c_int, FP]
        L.orc_lgn_convol.argtypes = [P, C.c_int, C.c_int, C.c_longlong, FP, FP, FP, FP]
        L.orc_lgn_nonlinear.argtypes = [P, FP, FP, FP, FP, FP, FP, FP, FP, FP, IP, C.c_int, FP, FP]
        L.orc_lgn_nonlinear_ex.argtypes = [P, FP, FP, FP, FP, FP, FP, FP, FP, FP, IP, C.c_int, FP, FP, UP, FP]
        L.orc_lgn_ff_pre.argtypes = [C.c_int, C.c_float, C.c_float, UP, FP, FP, FP, FP, FP]
        L.orc_v1_set_ff_learning.argtypes = [P, P]
        L.orc_v1_learn_ff.argtypes = [P, FP, FP, FP]
        L.orc_ff_learning_rates.argtypes = [P, C.c_float, FP]
        L.orc_v1_learn_avg.argtypes = [P]
        L.orc_parvo_max_sample1d.argtypes = [P, P, C.c_int]
        L.orc_lgn_parvo_setup.argtypes = [P, P, P, FP, FP, FP, FP, FP]
        L.orc_lgn_parvo_spatial.argtypes = [C.c_int, C.c_int, FP, FP, UP, FP, C.c_int, C.c_int, C.c_int,
                                            C.c_int, FP]
        L.orc_lgn_parvo_convol.argtypes = [P, P, P, C.c_int, C.c_longlong, FP, FP, FP]
        L.orc_v1_create.argtypes = [P, C.c_uint32, UP, UP, FP, C.c_uint32, UP, UP, FP, UP, UP, FP, FP, FP]
        L.orc_v1_create.restype = P
        L.orc_v1_destroy.argtypes = [P]
        L.orc_v1_get.argtypes = [P, C.c_int, FP]
        L.orc_v1_put.argtypes = [P, C.c_int, FP]
        L.orc_v1_compute_v.argtypes = [P, FP, FP, FP, C.c_int]
        L.orc_v1_deliver_near.argtypes = [P, FP, C.c_int]
        L.orc_v1_deliver_far.argtypes = [P]
        L.orc_v1_set_delays.argtypes = [P, FP, C.c_int]
        F = C.c_float
        L.orc_cond_eval.argtypes = [F, F, F, F, F, F, FP]
        L.orc_adex_depc.argtypes = [F] * 6
        L.orc_adex_depc.restype = F
        L.orc_adex_rk2.argtypes = [F] * 19 + [FP, FP]
        L.orc_adex_spike.argtypes = [F] * 5 + [FP, FP]
        L.orc_logistic_ab.argtypes = [FP, FP, FP, C.c_int, FP, FP]
        L.orc_v1_deliver_near_delayed.argtypes = [P, FP, C.c_int]
        L.orc_std_normal_draws.argtypes = [C.POINTER(C.c_uint64), C.c_int, IP, C.c_int, FP]
        L.orc_v1_set_far_failure.argtypes = [P, C.c_uint64, C.c_int]
        L.orc_v1_init_spikes.argtypes = [P, FP, C.c_uint32, C.c_int, FP, UP, C.c_uint32, FP, UP, C.c_uint32, FP]
        L.orc_set_threads.argtypes = [C.c_int]
        L.orc_host_init_state.argtypes = [P, C.c_uint64, FP, UP, C.c_int, C.c_float] + [FP] * 12
        L.orc_num_threads.restype = C.c_int
        _lib = L
    return _lib


def fp(a):
    if a is None:
        return None
    assert a.dtype == np.float32 and a.flags.c_contiguous, (a.dtype, a.flags)
    return a.ctypes.data_as(C.POINTER(C.c_float))


def up(a):
    if a is None:
        return None
    assert a.dtype == np.uint32 and a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(C.c_uint32))


def ip(a):
    if a is None:
        return None
    assert a.dtype == np.int32 and a.flags.c_contiguous
    return a.ctypes.data_as(C.POINTER(C.c_int32))


ST = dict(v=0, w=1, tBack=2, dep=3, gFF=4, hFF=5, gE=6, hE=7, gI=8, hI=9, sInfo=10, sLGN=18, ff_post=19,
          total_ff=21)


def host_init_state(spec, seed: int, tonicDep, nLGNperV1, v0, w0, gFF0, gE0, gI0,
                    use_v0=False, tonicMax=None):
    """The reference's host-drawn initial state (src/patch.cu:4405-4540) restated in C
    (orc_host_init_state); same arguments and result as the library's host_init_state."""
    import ctypes as _C
    from visual_cortex_gb300.model import InitState
    n = spec.nV1
    cfg = spec.to_struct()
    td = np.ascontiguousarray(tonicDep, dtype=f32)
    nl = np.ascontiguousarray(nLGNperV1, dtype=np.uint32)
    if tonicMax is None:
        tonicMax = float(td.max())
    out = dict(v=np.empty(n, f32), w=np.empty(n, f32), gFF=np.empty(spec.ngFF * n, f32),
               hFF=np.empty(spec.ngFF * n, f32), gE=np.empty(spec.ngE * n, f32),
               hE=np.empty(spec.ngE * n, f32), gI=np.empty(spec.ngI * n, f32),
               hI=np.empty(spec.ngI * n, f32))
    w0a = np.ascontiguousarray(w0 if w0 is not None else np.zeros(2 * spec.nType), dtype=f32)
    g = [np.ascontiguousarray(x, dtype=f32) for x in (gFF0, gE0, gI0)]
    lib().orc_host_init_state(_C.byref(cfg), int(seed), fp(td), up(nl), int(bool(use_v0)), float(tonicMax),
                              fp(w0a), fp(g[0]), fp(g[1]), fp(g[2]), fp(out["v"]), fp(out["w"]),
                              fp(out["gFF"]), fp(out["hFF"]), fp(out["gE"]), fp(out["hE"]), fp(out["gI"]),
                              fp(out["hI"]))
    if spec.iModel != 1:
        out["w"] = None
    return InitState(**out)


class LgnOracle:
    """store_PM + per-frame spatial stage + per-step convolution and spikes for the magno
    and (when present) the parvo cells."""

    def __init__(self, lgn, stim, wbits: int = 8):
        self.lgn = lgn
        self.cfg = lgn.to_struct()
        self.params, self._keep = lgn.params_struct()
        nm, ns, nks = lgn.nMagno, lgn.mSample1D ** 2, lgn.sched.mKernelSample
        self.TW = np.empty((nm, nks), f32)
        self.SW = np.empty((nm, ns), f32)
        self.SC = np.empty((2, nm, ns), f32)
        self.maxConvol = np.empty(lgn.nLGN, f32)
        self.absk = np.empty(nm, f32)
        self.la = np.empty(lgn.nLGN, f32)
        self.lb = np.empty(lgn.nLGN, f32)
        L = lib()
        L.orc_lgn_setup(C.byref(self.cfg), C.byref(self.params), fp(self.TW), fp(self.SW), fp(self.SC),
                        fp(self.maxConvol), fp(self.absk), fp(self.la), fp(self.lb))
        self.nFrame = stim.frames.shape[0]
        self.stim = stim
        self.wbits = wbits
        self.S = None
        self.c50 = np.ascontiguousarray(lgn.c50, f32)
        self.sharp = np.ascontiguousarray(lgn.sharpness, f32)
        self.ltr = np.zeros(lgn.nLGN, f32)
        self.lnl = np.zeros(lgn.nLGN, f32)
        self.nParvo = lgn.nParvo
        self.PS = None
        if self.nParvo:
            self.pcfg = lgn.to_parvo_struct()
            npv, ns, pks = self.nParvo, lgn.nSample1D ** 2, lgn.sched.nKernelSample
            self.pTW = np.empty((npv, 2, pks), f32)
            self.pSW = np.empty(ns, f32)
            self.pSC = np.empty((2, npv, 2, ns), f32)
            self._cov = np.ascontiguousarray(lgn.covariant, f32)
            L.orc_lgn_parvo_setup(C.byref(self.cfg), C.byref(self.pcfg), C.byref(self.params), fp(self._cov),
                                  fp(self.pTW), fp(self.pSW), fp(self.pSC), fp(self.maxConvol))
            self.max_sample1d = L.orc_parvo_max_sample1d(C.byref(self.cfg), C.byref(self.params), lgn.nSample1D)
            ct = np.asarray(lgn.coneType, np.uint32)
            pid = lgn.parvo_ids()
            self.pcone = np.ascontiguousarray(np.concatenate([ct[pid], ct[lgn.nLGN + pid]]), np.uint32)

    def spatial(self, SW=None, SC=None):
        """S [nFrame+1][nMagno]; by default from this oracle's own SW/SC tables."""
        lgn = self.lgn
        fr = self.stim.frames
        nF, _, h, w = fr.shape
        layers = np.empty((nF + 1, 3, h, w), f32)
        layers[:nF] = fr
        for ch in range(3):
            layers[nF, ch] = self.stim.init_LMS[ch]
        SW = self.SW if SW is None else np.ascontiguousarray(SW, f32)
        SC = self.SC if SC is None else np.ascontiguousarray(SC, f32)
        cone = np.ascontiguousarray(np.asarray(lgn.coneType, np.uint32)[lgn.magno_ids()])
        S = np.empty((nF + 1, lgn.nMagno), f32)
        lib().orc_lgn_spatial(lgn.nMagno, lgn.mSample1D ** 2, fp(SW), fp(SC), up(cone), fp(layers), nF + 1,
                              h, w, self.wbits, fp(S))
        self.S = S
        if self.nParvo:
            self._layers = layers
            self.parvo_spatial()
        return S

    def parvo_spatial(self, SW=None, SC=None):
        """PS [nFrame+1][2][nParvo]; by default from this oracle's own parvo tables."""
        fr = self.stim.frames
        nF, _, h, w = fr.shape
        layers = getattr(self, "_layers", None)
        if layers is None:
            layers = np.empty((nF + 1, 3, h, w), f32)
            layers[:nF] = fr
            for ch in range(3):
                layers[nF, ch] = self.stim.init_LMS[ch]
            self._layers = layers
        SW = self.pSW if SW is None else np.ascontiguousarray(SW, f32)
        SC = self.pSC if SC is None else np.ascontiguousarray(SC, f32)
        PS = np.empty((nF + 1, 2, self.nParvo), f32)
        lib().orc_lgn_parvo_spatial(self.nParvo, self.lgn.nSample1D ** 2, fp(SW), fp(SC), up(self.pcone),
                                    fp(layers), nF + 1, h, w, self.wbits, fp(PS))
        self.PS = PS
        return PS

    def convol(self, it: int, S=None, TW=None):
        """Convolution of step it for every LGN cell, by LGN id (magno: times |k|)."""
        S = self.S if S is None else S
        TW = self.TW if TW is None else TW
        mag = np.empty(self.lgn.nMagno, f32)
        lib().orc_lgn_convol(C.byref(self.cfg), self.lgn.nMagno, self.nFrame, int(it), fp(TW), fp(S),
                             fp(self.absk), fp(mag))
        out = np.zeros(self.lgn.nLGN, f32)
        out[self.lgn.magno_ids()] = mag
        if self.nParvo:
            par = np.empty(self.nParvo, f32)
            lib().orc_lgn_parvo_convol(C.byref(self.cfg), C.byref(self.pcfg), C.byref(self.params), self.nFrame,
                                       int(it), fp(self.pTW), fp(self.PS), fp(par))
            out[self.lgn.parvo_ids()] = par
        return out

    def nonlinear(self, convol, u, ucount, cap):
        sInfo = np.zeros(self.lgn.nLGN, f32)
        fr = np.zeros(self.lgn.nLGN, f32)
        self.nsp = np.zeros(self.lgn.nLGN, np.uint32)
        self.tsp = np.zeros(self.lgn.nLGN, f32)
        mism = lib().orc_lgn_nonlinear_ex(C.byref(self.cfg), fp(convol), fp(self.maxConvol), fp(self.c50),
                                          fp(self.sharp), fp(self.la), fp(self.lb), fp(self.ltr), fp(self.lnl),
                                          fp(u), ip(ucount), int(cap), fp(sInfo), fp(fr), up(self.nsp),
                                          fp(self.tsp))
        self.last_sInfo = sInfo
        return sInfo, fr, mism

    def ff_pre(self, tauLTP: float, k: int = 0):
        """Presynaptic learning trace k (0: the FF->E type's, 1: the FF->I type's) over the step
        just computed by `nonlinear` (self.ff_vars[k] carries it): returns (trace at the step
        start, right after the spikes)."""
        n = self.lgn.nLGN
        if getattr(self, "ff_vars", None) is None:
            self.ff_vars = [np.zeros(n, f32), np.zeros(n, f32)]
        start = np.zeros(n, f32)
        at = np.zeros(n, f32)
        lib().orc_lgn_ff_pre(n, f32(self.cfg.dt), f32(tauLTP), up(self.nsp), fp(self.tsp), fp(self.last_sInfo),
                             fp(self.ff_vars[k]), fp(start), fp(at))
        return start, at

    @property
    def ff_var(self):
        return self.ff_vars[0]


class V1Oracle:
    def __init__(self, spec, net):
        self.spec = spec
        self.cfg = spec.to_struct()
        c = lambda a, t: np.ascontiguousarray(a, dtype=t)
        self._keep = [c(net.nLGNperV1, np.uint32), c(net.lgnId, np.uint32), c(net.sLGN, f32),
                      c(net.nNearNB, np.uint32), c(net.nbId, np.uint32), c(net.conMat, f32),
                      c(net.nVec, np.uint32), c(net.vecID, np.uint32), c(net.conVec, f32),
                      c(net.delayVec, f32), c(net.tonicDep, f32)]
        k = self._keep
        self.h = lib().orc_v1_create(C.byref(self.cfg), net.maxLGN, up(k[0]), up(k[1]), fp(k[2]), net.nnb,
                                     up(k[3]), up(k[4]), fp(k[5]), up(k[6]), up(k[7]), fp(k[8]), fp(k[9]),
                                     fp(k[10]))
        self.delayed = not spec.noDelay
        if self.delayed:
            # ring depth of src/patch.cu:3808-3813: the largest connected near distance
            dm = c(net.delayMat, f32)
            self._keep.append(dm)
            conn = np.asarray(net.conMat) != 0
            maxd = float(dm[conn].max()) if conn.any() else 0.0
            depth = int(np.ceil(np.float32(np.float32(maxd) / np.float32(spec.speedOfThought)) /
                                np.float32(spec.dt))) + 1
            lib().orc_v1_set_delays(self.h, fp(dm), max(depth, 2))

    def put(self, name, arr):
        lib().orc_v1_put(self.h, ST[name], fp(np.ascontiguousarray(arr, f32)))

    def get(self, name):
        s = self.spec
        n = s.nV1
        size = dict(gFF=s.ngFF * n, hFF=s.ngFF * n, gE=s.ngE * n, hE=s.ngE * n, gI=s.ngI * n,
                    hI=s.ngI * n, sLGN=self._keep[1].shape[0] * n,
                    ff_post=((0 if getattr(self, "_ff_mode", 3) == 4 else 2 * s.nE * s.nblock) + 2 * s.nE * s.nblock +
                             (1 + 2 * getattr(self, "_ff_i", 0)) * (s.blockSize - s.nE) * s.nblock),
                    total_ff=2 * n).get(name, n)
        out = np.empty(size, f32)
        lib().orc_v1_get(self.h, ST[name], fp(out))
        return out

    def set_state(self, init):
        for name in ("v", "gFF", "hFF", "gE", "hE", "gI", "hI"):
            self.put(name, getattr(init, name))
        if init.w is not None:
            self.put("w", init.w)

    def set_far_failure(self, seed, nChunk):
        lib().orc_v1_set_far_failure(self.h, int(seed), int(nChunk))

    def set_ff_learning(self, learning):
        """LGN->V1 plasticity with the parameters of a model.FFLearning."""
        self._ffl = learning.to_struct()
        self._ff_mode = int(learning.learning)
        self._ff_i = int(learning.nLearnTypeFF_I) if self._ff_mode == 2 else 0
        if lib().orc_v1_set_ff_learning(self.h, C.byref(self._ffl)) != 0:
            raise ValueError("learning modes 1-4 with nLearnTypeFF_E = 1 (0 with learning 4) are restated")

    def learn_ff(self, lgn_sInfo, pre_start, pre_spike):
        lib().orc_v1_learn_ff(self.h, fp(np.ascontiguousarray(lgn_sInfo, f32)), fp(pre_start), fp(pre_spike))

    def learn_avg(self):
        lib().orc_v1_learn_avg(self.h)

    def init_spikes(self, sp0, SCsplit, depth, rec):
        """rand_spInit with initial spikes and the delivery before the first step, from the
        device's recorded draws (`rec`: the dict Simulation keeps from pv1_v1_init_spikes).
        Returns (draw-count mismatches, spike-word history [depth][nV1])."""
        L = lib()
        if self.delayed:
            L.orc_v1_set_delays(self.h, fp(self._keep[-1]), int(depth))
        u = np.ascontiguousarray(rec["uniforms"], f32)
        nu = np.ascontiguousarray(rec["nUniform"], np.uint32)
        z = np.ascontiguousarray(rec["normals"], f32)
        nz = np.ascontiguousarray(rec["nNormal"], np.uint32)
        H = np.empty((depth, self.spec.nV1), f32)
        m = L.orc_v1_init_spikes(self.h, fp(np.ascontiguousarray(sp0, f32)), int(SCsplit), int(depth), fp(u), up(nu),
                                 u.shape[1], fp(z), up(nz), z.shape[1], fp(H))
        if m < 0:
            raise RuntimeError("orc_v1_init_spikes: the delay ring is not set up")
        return m, H

    def step(self, lgn_sInfo, noise=None, ff=None, near=None, cap=0):
        L = lib()
        nerr = L.orc_v1_compute_v(self.h, fp(np.ascontiguousarray(lgn_sInfo, f32)),
                                  fp(None if noise is None else np.ascontiguousarray(noise, f32)),
                                  fp(None if ff is None else np.ascontiguousarray(ff, f32)), int(cap))
        if self.delayed:
            L.orc_v1_deliver_near_delayed(self.h, fp(None if near is None else np.ascontiguousarray(near, f32)), int(cap))
        else:
            L.orc_v1_deliver_near(self.h, fp(None if near is None else np.ascontiguousarray(near, f32)), int(cap))
        L.orc_v1_deliver_far(self.h)
        return nerr

    def close(self):
        if self.h:
            lib().orc_v1_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
