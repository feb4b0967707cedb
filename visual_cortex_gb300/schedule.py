"""Stimulus-frame and temporal-kernel bookkeeping of the reference's step loop.

Pure integer arithmetic restated from src/patch.cu:1342-1372 (step rate, retrace lengths),
4950-5030 (kernel sampling interval and frame phases, find_denorm in src/util/util.h:251-279)
and 5395-5412 (frame phase tails).  Shared by the GPU host driver and the CPU oracle.
"""
from __future__ import annotations

from dataclasses import dataclass


def find_denorm(u1: int, u2: int, more_dt: bool) -> tuple[int, int]:
    """Minimum number of u1-advances without phase difference to u2 (src/util/util.h:251-279).

    Returns (denorm, norm)."""
    if more_dt:
        m = u1
        if u2 % u1 == 0:
            return 1, 1
        n = u2 - u1 * (u2 // u1)
    else:
        m = u2
        if u1 % u2 == 0:
            return 1, 1
        n = u1 - u2 * (u1 // u2)
    if not m > n:
        raise ValueError("find_denorm: m <= n")
    for i in range(n, 1, -1):
        if n % i == 0 and m % i == 0:
            return m // i, n // i
    return m, 1


@dataclass
class FrameSchedule:
    dt: float
    frameRate: int
    stepRate: int
    nRetrace: int
    mRetrace: int
    nKernelSample: int
    mKernelSample: int
    kernelSampleInterval: int      # parvo, in steps
    iKernelSampleT0: int
    mKernelSampleInterval: int     # magno, in steps
    mKernelSampleT0: int
    denorm: int
    ntPerFrame: int
    maxFrame: int
    parvoFrame: int
    magnoFrame: int
    pLongerThanM: bool
    dFrame: int
    parvoComp: int
    magnoComp: int

    @property
    def kernelSampleDt(self) -> float:
        """Parvo kernel sample spacing (src/patch.cu:4962)."""
        import numpy as np
        return float(np.float32(self.kernelSampleInterval) * np.float32(self.dt))

    @property
    def kernelSampleT0f(self) -> float:
        import numpy as np
        return float(np.float32(self.iKernelSampleT0) * np.float32(self.dt))

    @property
    def mKernelSampleDt(self) -> float:
        import numpy as np
        return float(np.float32(self.mKernelSampleInterval) * np.float32(self.dt))

    @property
    def mKernelSampleT0f(self) -> float:
        import numpy as np
        return float(np.float32(self.mKernelSampleT0) * np.float32(self.dt))

    def frames_read(self, it: int) -> int:
        """Frames read from the stimulus file once step `it` started (src/patch.cu:5969)."""
        return -(-((it + 1) * self.denorm) // self.ntPerFrame)

    def snapshot_indices(self, steps_done: int, trainDepth: int) -> dict:
        """The frame bookkeeping of the step loop after steps_done steps (src/patch.cu:
        5395-5412, 5966-6057): frames read, the ring head, its previous value and wraps, the
        four phases; the next spike-word slot; iStatus 0 (no LGN switching)."""
        q = int(steps_done)
        cur = -(-(q * self.denorm) // self.ntPerFrame)
        return dict(step=q, frameCycle=cur // self.maxFrame, iFrameHead=cur % self.maxFrame,
                    oldFrameHead=(cur - 1) % self.maxFrame if cur > 0 else 0, currentFrame=cur,
                    iFramePhaseHead=(q * self.denorm) % self.ntPerFrame,
                    iFramePhaseTail=(self.parvoComp + q * self.denorm) % self.ntPerFrame,
                    mFramePhaseHead=(q * self.denorm) % self.ntPerFrame,
                    mFramePhaseTail=(self.magnoComp + q * self.denorm) % self.ntPerFrame,
                    iStatus=0, currentTimeSlot=q % int(trainDepth))

    def magno_tail(self, it: int) -> tuple[int, int]:
        """(frame tail layer offset from the newest frame's layer, phase) at step it."""
        phase = (self.magnoComp + (it + 1) * self.denorm) % self.ntPerFrame
        extra = (self.dFrame if self.pLongerThanM else 0) + (2 if phase <= self.magnoComp else 1)
        return extra, phase


def make_schedule(dt: float, frameRate: int, tau: float, mau: float, nKernelSample: int,
                  mKernelSample: int) -> FrameSchedule:
    import numpy as np
    dt32 = np.float32(dt)
    step_rate_f = 1000 / float(dt32)
    stepRate = int(round(step_rate_f))
    if round(step_rate_f) != step_rate_f:
        raise ValueError(f"stepRate = {step_rate_f} Hz must be an integer")
    if frameRate > stepRate:
        raise ValueError("frameRate > stepRate")
    nRetrace = int(round(float(np.float32(tau)) / float(dt32)))
    if round(float(np.float32(tau)) / float(dt32)) != float(np.float32(tau)) / float(dt32):
        raise ValueError("tau must be a multiple of dt")
    if nRetrace % nKernelSample:
        raise ValueError("parvo retrace must be divisible by nKernelSample")
    mRetrace = int(round(float(np.float32(mau)) / float(dt32)))
    if round(float(np.float32(mau)) / float(dt32)) != float(np.float32(mau)) / float(dt32):
        raise ValueError("mau must be a multiple of dt")
    if mRetrace % mKernelSample:
        raise ValueError("magno retrace must be divisible by mKernelSample")
    ksi = nRetrace // nKernelSample
    t0 = ksi // 2 if ksi % 2 == 0 else 0
    mksi = mRetrace // mKernelSample
    mt0 = mksi // 2 if mksi % 2 == 0 else 0
    more_dt = not (stepRate < frameRate)
    denorm, norm = find_denorm(frameRate, stepRate, more_dt)
    if (stepRate * denorm) % frameRate:
        raise ValueError("(stepRate*denorm) % frameRate != 0")
    ntPerFrame = (stepRate * denorm) // frameRate
    parvoFrame = (nRetrace * denorm + ntPerFrame - 1) // ntPerFrame + 1
    magnoFrame = (mRetrace * denorm + ntPerFrame - 1) // ntPerFrame + 1
    maxFrame = max(parvoFrame, magnoFrame)
    if maxFrame > 2048:
        raise ValueError("a layered texture allows 2048 layers")
    pLongerThanM = parvoFrame > magnoFrame
    dFrame = abs(magnoFrame - parvoFrame)
    parvoComp = (ntPerFrame - (nRetrace * denorm) % ntPerFrame) % ntPerFrame
    magnoComp = (ntPerFrame - (mRetrace * denorm) % ntPerFrame) % ntPerFrame
    return FrameSchedule(dt=float(dt32), frameRate=frameRate, stepRate=stepRate,
                         nRetrace=nRetrace, mRetrace=mRetrace, nKernelSample=nKernelSample,
                         mKernelSample=mKernelSample, kernelSampleInterval=ksi,
                         iKernelSampleT0=t0, mKernelSampleInterval=mksi, mKernelSampleT0=mt0,
                         denorm=denorm, ntPerFrame=ntPerFrame, maxFrame=maxFrame,
                         parvoFrame=parvoFrame, magnoFrame=magnoFrame,
                         pLongerThanM=pLongerThanM, dFrame=dFrame, parvoComp=parvoComp,
                         magnoComp=magnoComp)
