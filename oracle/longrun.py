"""Long runs of the library next to the oracle -- TEST INFRASTRUCTURE.

`paired_raster` runs one workload for many steps on the GPU in chunks, recording every LGN
uniform of each chunk, and replays the chunk with the oracle (the reference's per-step order:
LGN convolution -> LGN spikes on the recorded uniforms -> V1 step -> near and far delivery),
keeping only the spike words.  The oracle starts from the library's LGN tables and initial LGN
integrals; those are held to the reference's own kernels separately (store_PM and
logRand_init, tests/test_ref_kernels.py), and cuRAND is not re-derived on the CPU.

`tuning_stats` reduces the rasters of a sweep over orientations to the quantities the
reference's analysis reports (oracle/tuning.py).
"""
from __future__ import annotations

import numpy as np

from . import LgnOracle, V1Oracle
from . import tuning as TU

f32 = np.float32


def paired_raster(wl, nsteps: int, chunk: int = 1000, cap: int = 8, seed_offset: int | None = None):
    """(gpu spike words [nsteps][nV1], oracle spike words [nsteps][nV1]).  The workload must
    draw no V1 noise and no synaptic failure (only the LGN uniforms are recorded)."""
    from visual_cortex_gb300 import _native as N
    from visual_cortex_gb300.model import Simulation
    s = wl.spec
    assert not any(s.noisyDep) and not any(s.synFail) and not any(s.synFailFF)
    sim = Simulation(wl.spec, wl.net, wl.lgn, wl.stim, wl.init, wl.seeds)
    n = s.nV1
    g = np.zeros((nsteps, n), f32)
    o = np.zeros((nsteps, n), f32)
    try:
        TW, SW, SC, mc = sim.lgn_tables()
        S = sim.lgn_spatial()
        lo = LgnOracle(wl.lgn, wl.stim)
        lo.TW[:] = TW
        lo.maxConvol[:] = mc
        lo.S = np.ascontiguousarray(S)
        lo.lnl[:] = sim.state("lgn_lnl")
        lo.ltr[:] = sim.state("lgn_ltr")
        vo = V1Oracle(wl.spec, wl.net)
        vo.set_state(wl.init)
        sim.set_record(N.REC_SPIKES, chunk + 1)
        for c0 in range(0, nsteps, chunk):
            k = min(chunk, nsteps - c0)
            sim.set_draw_record(k, cap)
            sim.run(k)
            g[c0:c0 + k] = sim.fetch_spikes(c0, k)
            U, Uc = sim.fetch_draws(0)
            for it in range(k):
                conv = lo.convol(c0 + it)
                sp, _, _ = lo.nonlinear(conv, np.ascontiguousarray(U[it]), np.ascontiguousarray(Uc[it]), cap)
                vo.step(sp)
                o[c0 + it] = vo.get("sInfo")
        vo.close()
    finally:
        sim.close()
    return g, o


def tuning_stats(rasters, spec, dt: float, tf_hz: float = 8.0, TFbins: int = 25):
    """rasters: [nOri] spike-word rasters of equal length.  Returns per-neuron rates
    [nOri][nV1], gOSI, OSI, preferred orientation, von Mises gOSI, and F1/F0 at each
    neuron's preferred orientation."""
    fr = np.stack([TU.rates(r, dt) for r in rasters])
    pref, osi = TU.aligned_osi(fr)
    dur = rasters[0].shape[0] * dt
    ratio = np.zeros((len(rasters), spec.nV1))
    for q, r in enumerate(rasters):
        ratio[q] = TU.f1f0(TU.spike_times(r, dt), dur, 1000.0 / tf_hz, TFbins)[2]
    return dict(fr=fr, gosi=TU.gosi(fr), osi=osi, pref=pref, vm_gosi=TU.von_mises_gosi(fr, pref),
                f1f0=ratio[pref, np.arange(spec.nV1)])
