"""Many trials (orientations x seeds, uneven durations and sizes) in the same launches.

The reference sweeps trials by running its `patch` executable once per orientation/seed
(src/ori.sh).  Here every trial is a Simulation (its own stimulus, seeds, initial state and
network) and a Batch steps them all together through pv1_batch_*: one batched LGN launch and
K batched V1 launches per chunk, captured as a CUDA graph, K and the V1 kernel variant picked
by the autotuner.  Each trial computes exactly what Simulation.run would compute for it.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _native as N
from .model import Simulation


class BatchError(RuntimeError):
    pass


class Batch:
    def __init__(self, sims: list[Simulation], steps: list[int], autotune: bool = True):
        if len(sims) != len(steps) or not sims:
            raise ValueError("one duration per trial")
        self.sims = list(sims)
        self.steps = [int(s) for s in steps]
        self.remaining = list(self.steps)
        arr =(C.c_void_p * len(sims))(*[s.plan.value for s in sims])
        st = (C.c_uint64 * len(sims))(*self.steps)
        h = C.c_void_p()
        rc = N.lib.pv1_batch_create(C.cast(arr, C.POINTER(C.c_void_p)), len(sims), st, C.byref(h))
        self.h = h
        if rc != 0:
            msg = N.lib.pv1_batch_last_error(h).decode() if h.value else ""
            self.close()
            raise BatchError(f"pv1_batch_create failed ({N.ERRORS.get(rc, rc)}): {msg}")
        self._check(N.lib.pv1_batch_autotune(self.h, int(bool(autotune))), "pv1_batch_autotune")

    def _check(self, rc, what):
        if rc < 0:
            raise BatchError(f"{what} failed ({N.ERRORS.get(rc, rc)}): "
                             f"{N.lib.pv1_batch_last_error(self.h).decode()}")
        return rc

    def run(self, max_steps: int = 0) -> tuple[int, float]:
        """Steps every trial to its end (or max_steps more); returns (steps the longest trial
        still has, device ms of the call)."""
        ms = C.c_float()
        before = max(self.remaining)
        left = self._check(N.lib.pv1_batch_run(self.h, int(max_steps), C.byref(ms)), "pv1_batch_run")
        done = before - int(left)      # the longest trial runs every step of the call
        for q, s in enumerate(self.sims):
            k = min(self.remaining[q], done)
            s.step += k
            self.remaining[q] -= k
        return int(left), float(ms.value)

    def sweep(self) -> float:
        """Runs the rest of every trial as one graph: the LGN stage of all remaining steps, one
        cooperative V1 launch (each slot runs its trials for all their steps, longest trials
        first), the advance (pv1_batch_sweep).  Returns the device ms."""
        ms = C.c_float()
        self._check(N.lib.pv1_batch_sweep(self.h, C.byref(ms)), "pv1_batch_sweep")
        for q, s in enumerate(self.sims):
            s.step += self.remaining[q]
            self.remaining[q] = 0
        return float(ms.value)

    def tuning(self):
        K, mb = C.c_int(), C.c_int()
        t = np.empty(12, np.float32)
        self._check(N.lib.pv1_batch_tuning(self.h, C.byref(K), C.byref(mb), N.fptr(t)), "pv1_batch_tuning")
        name = lambda b: "persistent" if b == 0 else f"minB{b}"
        cand = {f"K{k}_{name(b)}": float(t[i * 4 + b]) for i, k in enumerate((16, 32, 64))
                for b in (0, 1, 2, 3)}
        return {"K": K.value, "variant": name(mb.value), "ms_per_chunk": cand}

    def stats(self, trial: int, rates: bool = False):
        """FP64 simulated time (ms), mean rate (Hz) and optionally per-neuron rates."""
        t, m = C.c_double(), C.c_double()
        n = self.sims[trial].spec.nV1
        r = np.empty(n, np.float64) if rates else None
        self._check(N.lib.pv1_batch_stats(self.h, trial, C.byref(t),
                                          r.ctypes.data_as(C.POINTER(C.c_double)) if rates else None,
                                          C.byref(m)), "pv1_batch_stats")
        return float(t.value), float(m.value), r

    def launches(self) -> int:
        return int(N.lib.pv1_batch_launch_count(self.h))

    def close(self):
        if getattr(self, "h", None) is not None and self.h.value:
            N.lib.pv1_batch_destroy(self.h)
            self.h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def main(argv=None):
    """``python -m visual_cortex_gb300.batch``: one batched sweep of the synthetic trials,
    printing the device time and throughput (used for profiling the batched kernels)."""
    import argparse
    from . import synth
    ap = argparse.ArgumentParser()
    ap.add_argument("--trials", type=int, default=64)
    ap.add_argument("--dur-ms", type=float, nargs=2, default=(250.0, 2000.0))
    ap.add_argument("--no-autotune", action="store_true")
    ap.add_argument("--sweep", action="store_true", help="one graph with one cooperative V1 launch (pv1_batch_sweep)")
    a = ap.parse_args(argv)
    trials = synth.batch_trials(n_trials=a.trials, seed=0, dur_ms=tuple(a.dur_ms))
    sims = [Simulation(t.wl.spec, t.wl.net, t.wl.lgn, t.wl.stim, t.wl.init, t.wl.seeds) for t in trials]
    b = Batch(sims, [t.steps for t in trials], autotune=not (a.no_autotune or a.sweep))
    ms = b.sweep() if a.sweep else b.run()[1]
    work = sum(t.steps * t.wl.spec.nV1 for t in trials)
    how = "one-launch sweep" if a.sweep else f"tuning {b.tuning()}"
    print(f"{a.trials} trials, {work} neuron-steps in {ms:.2f} ms: {work / (ms * 1e-3):.4g} neuron-steps/s; {how}")
    b.close()
    for s in sims:
        s.close()


if __name__ == "__main__":
    main()
