"""LGN stage at scale on BF16 tensor cores (form c): workload, frame weights, FP64 oracle.

The whole movie is processed at once: the spatial stage S[cell][frame] (a side x side DoG
footprint on the pixel grid) is computed on the device, the temporal contraction
convol[cell][t] = sum_f S[cell][f] W[t][f] runs as tcgen05 BF16 MMAs with FP32 accumulation
(pv1_lgn_tc_*), followed by the logistic rate and the Poisson generator.  W[t][f] is the sum of
the time-reversed temporal-kernel samples that read frame f at step t, with the frame
bookkeeping of the reference's step loop (src/patch.cu:4950-5030, 5395-5422, restated in
schedule.py); it is built here in FP64 and tiled per 128 steps with a 64-frame window.
The FP64 evaluation of the same rates for the error report is test infrastructure and lives
in oracle/lgn_fp64.py.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass

import numpy as np

from . import _native as N
from .schedule import make_schedule

f32, u32, i32 = np.float32, np.uint32, np.int32
TILE_N, TILE_K, PAD = 128, 64, 64


class TcConfig(C.Structure):
    _fields_ = [(n, C.c_uint32) for n in ("nCells", "nFrame", "height", "width", "side", "nFext", "pad", "T",
                                          "frEvery", "recordRates")] + \
               [(n, C.c_float) for n in ("dt", "convolRatio", "frRatio", "meanLum")]


_FP = C.POINTER(C.c_float)
_IP = C.POINTER(C.c_int32)
for _n, (_a, _r) in {
    "pv1_lgn_tc_create": ([C.POINTER(TcConfig), _FP, _FP, _IP, _IP, _FP, _IP, _FP, _FP, _FP, _FP, _FP, _FP,
                           C.POINTER(C.c_void_p)], C.c_int),
    "pv1_lgn_tc_run": ([C.c_void_p, C.c_int, C.c_uint64, _FP], C.c_int),
    "pv1_lgn_tc_fetch": ([C.c_void_p, _FP, _FP, _FP], C.c_int),
    "pv1_lgn_tc_destroy": ([C.c_void_p], None),
    "pv1_lgn_tc_last_error": ([C.c_void_p], C.c_char_p),
}.items():
    getattr(N.lib, _n).argtypes = _a
    getattr(N.lib, _n).restype = _r


def pink_noise_frames(nFrame: int, size: int, rng, mean=0.5, rms_contrast=0.3) -> np.ndarray:
    """Frames of Gaussian noise with a 1/f^2 power spectrum, luminance mean 0.5 and RMS
    contrast 0.3 (std / mean), clipped to [0, 1]."""
    fx = np.fft.fftfreq(size)[None, :]
    fy = np.fft.fftfreq(size)[:, None]
    f = np.hypot(fx, fy)
    f[0, 0] = 1.0
    amp = 1.0 / f
    amp[0, 0] = 0.0
    out = np.empty((nFrame, size, size), f32)
    for i in range(nFrame):
        w = rng.standard_normal((size, size))
        x = np.real(np.fft.ifft2(np.fft.fft2(w) * amp))
        x = (x - x.mean()) / x.std()
        out[i] = np.clip(mean * (1 + rms_contrast * x), 0.0, 1.0).astype(f32)
    return out


def temporal_weights(sched, tauR=1.5, tauD=4.5, nR=19.0, nD=9.5, ratio=1.0, delay=14.0) -> np.ndarray:
    """Time-reversed magno temporal kernel samples, normalised by sum |K| (the kernel of
    src/discrete_input_convol.cu:8-33 and store_temporalWeight), in FP64."""
    n = sched.mKernelSample
    dts = sched.mKernelSampleDt
    t0 = sched.mKernelSampleT0f - delay
    tw = np.zeros(n)
    for j in range(n):
        t = (n - 1 - j) * dts + t0
        if t <= 0:
            continue
        a1, a2 = t / tauR, t / tauD
        tR = math.exp((nR - 1) * math.log(a1) - a1 - math.lgamma(nR)) / tauR
        tD = math.exp((nD - 1) * math.log(a2) - a2 - math.lgamma(nD)) / tauD
        tw[j] = tR - ratio * tD
    return tw / np.abs(tw).sum()


def frame_of_samples(sched, T: int) -> np.ndarray:
    """[T][nKS] absolute frame read by temporal sample j at step t (negative: before the movie)."""
    t = np.arange(T, dtype=np.int64)[:, None]
    j = np.arange(sched.mKernelSample, dtype=np.int64)[None, :]
    cf = -(-((t + 1) * sched.denorm) // sched.ntPerFrame)
    phase = (sched.magnoComp + (t + 1) * sched.denorm) % sched.ntPerFrame
    off = sched.dFrame if sched.pLongerThanM else 0
    te = off + np.where(phase <= sched.magnoComp, 2, 1)
    rel = ((sched.mKernelSampleT0 + j * sched.mKernelSampleInterval) * sched.denorm + phase) // sched.ntPerFrame
    x = te + rel
    back = (sched.maxFrame - x % sched.maxFrame) % sched.maxFrame
    return cf - 1 - back


def frame_weights(sched, tw: np.ndarray, T: int):
    """W tiles [nTiles][128][64] (FP64), window starts f0 [nTiles] (columns = frame + PAD,
    multiples of 8) and the number of frame columns."""
    F = frame_of_samples(sched, T) + PAD
    if F.min() < 0:
        raise ValueError("temporal window reaches further back than the padding")
    nTiles = -(-T // TILE_N)
    W = np.zeros((nTiles, TILE_N, TILE_K))
    f0 = np.zeros(nTiles, np.int64)
    for i in range(nTiles):
        rows = F[i * TILE_N:(i + 1) * TILE_N]
        c0 = (rows.min() // 8) * 8
        if rows.max() - c0 >= TILE_K:
            raise ValueError("a tile's frames do not fit the 64-frame window")
        f0[i] = c0
        for s in range(rows.shape[0]):
            np.add.at(W[i, s], rows[s] - c0, tw)
    nFext = int(-(-(F.max() + 1) // 8) * 8)
    nFext = max(nFext, int(f0.max()) + 8)
    return W, f0.astype(i32), nFext


@dataclass
class LgnWorkload:
    frames: np.ndarray      # [nFrame][H][W] luminance
    SW: np.ndarray          # [nCells][side*side]
    cx: np.ndarray
    cy: np.ndarray
    side: int
    k: np.ndarray           # [nCells] centre amplitude (sign: ON/OFF)
    c50: np.ndarray
    sharp: np.ndarray
    spont: np.ndarray
    la: np.ndarray
    lb: np.ndarray
    maxConvol: np.ndarray
    tw: np.ndarray          # FP64 temporal weights
    W: np.ndarray           # FP64 tiles
    f0: np.ndarray
    nFext: int
    T: int
    dt: float
    sched: object
    convolRatio: float = 1.0
    frRatio: float = 1.0
    meanLum: float = 0.5

    @property
    def nCells(self):
        return self.SW.shape[0]


def make_workload(nCells=16384, size=256, nFrame=240, side=31, T=16000, dt=0.125, seed=0,
                  sigma_c=1.2, sigma_s=3.6, jitter=0.2, amp_ratio=0.7) -> LgnWorkload:
    """ON/OFF DoG cells on a size x size 1/f^2 noise movie at 120 Hz (2 s at the defaults)."""
    rng = np.random.default_rng(seed)
    frames = pink_noise_frames(nFrame, size, rng)
    half = side // 2
    cx = rng.integers(half, size - half, nCells).astype(i32)
    cy = rng.integers(half, size - half, nCells).astype(i32)
    sc = sigma_c * (1 + jitter * rng.uniform(-1, 1, nCells))
    ss = sigma_s * (1 + jitter * rng.uniform(-1, 1, nCells))
    d = np.arange(side) - half
    r2 = (d[None, :] ** 2 + d[:, None] ** 2).reshape(-1)
    g = lambda s: np.exp(-r2[None, :] / (2 * s[:, None] ** 2)) / (2 * math.pi * s[:, None] ** 2)
    w = g(sc) - amp_ratio * g(ss)
    w = w / np.abs(w).sum(1, keepdims=True)       # sum |w| = 1: max |convol| = |k|
    on = np.arange(nCells) < nCells // 2
    k = np.where(on, 60.0, -60.0)
    sched = make_schedule(dt, 120, 250.0, 250.0, 250, 250)
    tw = temporal_weights(sched)
    W, f0, nFext = frame_weights(sched, tw, T)
    c50 = np.full(nCells, 0.25, f32)
    sharp = np.full(nCells, 3.0, f32)
    spont = np.full(nCells, 0.1, f32)
    e1 = np.exp(sharp * c50).astype(f32)
    e2 = np.exp(sharp * c50 - sharp).astype(f32)
    la = ((1 - spont) * (1 + e1) * (1 + e2) / (e1 - e2)).astype(f32)
    lb = (1 - la / (1 + e2)).astype(f32)
    return LgnWorkload(frames=frames, SW=w.astype(f32), cx=cx, cy=cy, side=side, k=k.astype(f32),
                       c50=c50, sharp=sharp, spont=spont, la=la, lb=lb,
                       maxConvol=np.abs(k).astype(f32), tw=tw, W=W, f0=f0, nFext=nFext, T=T, dt=dt,
                       sched=sched)


class LgnTensorCore:
    """The device side: spatial stage, BF16 tiles, the stepping kernels."""

    def __init__(self, wl: LgnWorkload, fr_every: int = 16, record_rates: bool = True):
        self.wl = wl
        cfg = TcConfig(nCells=wl.nCells, nFrame=wl.frames.shape[0], height=wl.frames.shape[1],
                       width=wl.frames.shape[2], side=wl.side, nFext=wl.nFext, pad=PAD, T=wl.T,
                       frEvery=fr_every, recordRates=int(record_rates), dt=wl.dt,
                       convolRatio=wl.convolRatio, frRatio=wl.frRatio, meanLum=wl.meanLum)
        self.cfg = cfg
        self._keep = [np.ascontiguousarray(a, dtype=t) for a, t in (
            (wl.frames, f32), (wl.SW, f32), (wl.cx, i32), (wl.cy, i32), (wl.W, f32), (wl.f0, i32),
            (np.abs(wl.k), f32), (wl.maxConvol, f32), (wl.c50, f32), (wl.sharp, f32), (wl.la, f32),
            (wl.lb, f32))]
        k = self._keep
        fp = lambda a: a.ctypes.data_as(_FP)
        ip = lambda a: a.ctypes.data_as(_IP)
        h = C.c_void_p()
        rc = N.lib.pv1_lgn_tc_create(C.byref(cfg), fp(k[0]), fp(k[1]), ip(k[2]), ip(k[3]), fp(k[4]), ip(k[5]),
                                     fp(k[6]), fp(k[7]), fp(k[8]), fp(k[9]), fp(k[10]), fp(k[11]), C.byref(h))
        self.h = h
        if rc != 0:
            msg = N.lib.pv1_lgn_tc_last_error(h).decode() if h.value else ""
            self.close()
            raise RuntimeError(f"pv1_lgn_tc_create failed ({N.ERRORS.get(rc, rc)}): {msg}")

    def run(self, tensor_cores: bool = True, seed: int = 1) -> float:
        ms = C.c_float()
        rc = N.lib.pv1_lgn_tc_run(self.h, int(bool(tensor_cores)), int(seed), C.byref(ms))
        if rc != 0:
            raise RuntimeError(f"pv1_lgn_tc_run failed: {N.lib.pv1_lgn_tc_last_error(self.h).decode()}")
        return float(ms.value)

    def fetch(self, S=False, spikes=False, rates=True):
        c = self.cfg
        nFr = -(-c.T // c.frEvery)
        s = np.empty((c.nCells, c.nFext), f32) if S else None
        sp = np.empty((c.T, c.nCells), f32) if spikes else None
        fr = np.empty((nFr, c.nCells), f32) if rates else None
        fp = lambda a: None if a is None else a.ctypes.data_as(_FP)
        rc = N.lib.pv1_lgn_tc_fetch(self.h, fp(s), fp(sp), fp(fr))
        if rc != 0:
            raise RuntimeError(f"pv1_lgn_tc_fetch failed: {N.lib.pv1_lgn_tc_last_error(self.h).decode()}")
        return s, sp, fr

    def device_spikes(self) -> int:
        """Device address of the last run's spike words [T][nCells] (pv1_lgn_tc_device_spikes),
        for Simulation.set_lgn_source."""
        return int(N.lib.pv1_lgn_tc_device_spikes(self.h) or 0)

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            N.lib.pv1_lgn_tc_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def main(argv=None):
    """``python -m visual_cortex_gb300.lgn_bf16 [--cells N] [--steps T] [--fp32]``: one run of the
    stage on a synthetic movie, printing the device time (used for profiling)."""
    import argparse
    ap = argparse.ArgumentParser()
    ap.add_argument("--cells", type=int, default=16384)
    ap.add_argument("--steps", type=int, default=16000)
    ap.add_argument("--fp32", action="store_true")
    a = ap.parse_args(argv)
    wl = make_workload(nCells=a.cells, T=a.steps)
    tc = LgnTensorCore(wl, fr_every=64)
    try:
        ms = tc.run(tensor_cores=not a.fp32)
    finally:
        tc.close()
    print(f"{a.cells} cells x {a.steps} steps: {ms:.3f} ms ({'FP32 CUDA cores' if a.fp32 else 'BF16 tcgen05'})")


if __name__ == "__main__":
    main()
