"""Timed CPU baseline of the hot path (test infrastructure, used by bench.py's CPU legs).

Runs the oracle's restatement of the reference's per-step sequence (LGN convolution, LGN
spikes, V1 step, near and far delivery) on the host cores with OpenMP, on a bounded number
of steps of the same synthetic workload the GPU is measured on.  The Poisson generator is
fed numpy uniforms (the point is the cost, not the draws).
"""
from __future__ import annotations

import os
import time

import numpy as np

from . import LgnOracle, V1Oracle, lib


def host_threads() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def cpu_model() -> str:
    try:
        with open("/proc/cpuinfo") as f:
            for line in f:
                if line.lower().startswith(("model name", "cpu part", "hardware")):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    return "unknown"


class CpuPatch:
    """A workload held by the oracle, ready to be stepped."""

    def __init__(self, wl, threads: int | None = None, seed: int = 1):
        self.threads = threads or host_threads()
        lib().orc_set_threads(self.threads)
        self.wl = wl
        self.lo = LgnOracle(wl.lgn, wl.stim)
        self.lo.spatial()
        self.vo = V1Oracle(wl.spec, wl.net)
        self.vo.set_state(wl.init)
        self.rng = np.random.default_rng(seed)
        self.lo.lnl[:] = -np.log(self.rng.uniform(size=wl.lgn.nLGN)).astype(np.float32)
        self.it = 0
        self.cap = 4

    def step(self, n: int) -> int:
        """Advances n steps; returns the number of V1 spikes."""
        nsp = 0
        for _ in range(n):
            conv = self.lo.convol(self.it)
            u = self.rng.uniform(size=(self.wl.lgn.nLGN, self.cap)).astype(np.float32)
            s, _, _ = self.lo.nonlinear(conv, u, None, self.cap)
            self.vo.step(s)
            nsp += int((self.vo.get("sInfo") >= 1).sum())
            self.it += 1
        return nsp

    def time_steps(self, n: int) -> float:
        t0 = time.perf_counter()
        self.step(n)
        return time.perf_counter() - t0
