"""Long runs: firing rates and orientation tuning of the library against the oracle.

The 1024-neuron patch (768 LIF E / 256 I, 512 LGN cells, 64 x 64 drifting grating at 8 Hz) is
run for 1 s (8000 steps) at each of 8 orientations on the GPU, and the oracle replays every
run on the same LGN uniforms (oracle/longrun.py).  Five more GPU runs per orientation start
from other initial states (the host-drawn v, w and conductances with other seeds) on the same
LGN input: they measure how far equally valid trajectories of this network drift apart (the
network is chaotic, so once a single threshold crossing differs spikes are no longer matched
one to one, and at some orientations it moves between states of different mean rate).

Criteria, following the reference's own analysis (src/plotV1_response.py:887-958 for F1/F0,
src/getTuningCurve.py:301-421 and 1709-1731 for gOSI, OSI and the von Mises fit):
* rasters identical for at least the first 50 ms at every orientation (a difference allowed
  only at a threshold crossing decided by float rounding);
* each population statistic -- mean rate per orientation and pooled over the sweep, mean
  gOSI, OSI, von Mises gOSI and F1/F0, for E and I -- within 2% of the oracle's, or, where
  the runs from other initial states spread more, within 3 standard deviations of them
  (the pooled mean rates within 2% in any case);
* per-neuron rates over the sweep: relative L2 difference within 2%, or within 1.5 times the
  mean difference between the GPU run and its replicas.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

NORI, T, NREP = 8, 8000, 5


@pytest.fixture(scope="module")
def sweep(native):
    from oracle.longrun import paired_raster, tuning_stats
    from visual_cortex_gb300 import _native as N
    from visual_cortex_gb300 import synth
    from visual_cortex_gb300.model import Simulation
    G, O, R, div = [], [], [[] for _ in range(NREP)], []
    from oracle.parity import first_divergence, knife_edge
    for q in range(NORI):
        wl = synth.config1(seed=0, orient=q * np.pi / NORI)
        g, o = paired_raster(wl, T)
        d = first_divergence(g, o)
        div.append((d, None if d is None else knife_edge(wl.spec, g, o, d)))
        G.append(g)
        O.append(o)
        for k in range(NREP):
            from visual_cortex_gb300.model import host_init_state
            s = wl.spec
            init = host_init_state(s, wl.seeds.cond + 1000 * (k + 1), wl.net.tonicDep, wl.net.nLGNperV1, None,
                                   np.tile([0.0, 0.0], s.nType).astype(np.float32),
                                   np.tile([0.01, 0.2, 0.0, 0.2], s.nType * s.ngFF).astype(np.float32),
                                   np.tile([0.005, 0.2, 0.0, 0.2], s.nType * s.ngE).astype(np.float32),
                                   np.tile([0.01, 0.2, 0.0, 0.2], s.nType * s.ngI).astype(np.float32))
            sim = Simulation(wl.spec, wl.net, wl.lgn, wl.stim, init, wl.seeds)
            try:
                sim.set_record(N.REC_SPIKES, T + 1)
                sim.run(T)
                R[k].append(sim.fetch_spikes(0, T))
            finally:
                sim.close()
    spec = wl.spec
    dt = spec.dt
    return dict(spec=spec, div=div, g=tuning_stats(G, spec, dt), o=tuning_stats(O, spec, dt),
                r=[tuning_stats(X, spec, dt) for X in R])


def _pops(spec):
    E = np.arange(spec.nV1) % spec.blockSize < spec.nE
    return (("E", E), ("I", ~E))


def test_first_50_ms_rasters_identical(sweep):
    for q, (d, edge) in enumerate(sweep["div"]):
        assert d is None or d >= 400 or edge, (q, d)


def test_population_rates_and_tuning_within_2_percent_or_replica_spread(sweep):
    g, o, r = sweep["g"], sweep["o"], sweep["r"]
    report = {}
    for pop, m in _pops(sweep["spec"]):
        stats = {}
        for q in range(NORI):
            stats[f"rate_ori{q}"] = lambda s, q=q: s["fr"][q][m].mean()
        stats["rate_pooled"] = lambda s: s["fr"][:, m].mean()
        for k in ("gosi", "osi", "vm_gosi", "f1f0"):
            stats[k] = lambda s, k=k: s[k][m][(g["fr"][:, m].max(0) > 1) & (o["fr"][:, m].max(0) > 1)].mean()
        for name, f in stats.items():
            a, b = f(g), f(o)
            sd = np.array([f(g)] + [f(x) for x in r]).std(ddof=1)
            report[f"{pop}_{name}"] = (float(a), float(b), float(sd), bool(abs(a - b) <= max(0.02 * abs(b), 3 * sd)))
        pooled = stats["rate_pooled"]
        report[f"{pop}_pooled_within_2pct"] = bool(abs(pooled(g) - pooled(o)) <= 0.02 * pooled(o))
    print(report)
    bad = {k: v for k, v in report.items() if (v is False or (isinstance(v, tuple) and not v[-1]))}
    assert not bad, bad


def test_per_neuron_rates(sweep):
    g, o, r = sweep["g"], sweep["o"], sweep["r"]
    for pop, m in _pops(sweep["spec"]):
        a, b = g["fr"][:, m].mean(0), o["fr"][:, m].mean(0)
        d = np.linalg.norm(a - b) / np.linalg.norm(b)
        base = np.mean([np.linalg.norm(a - x["fr"][:, m].mean(0)) / np.linalg.norm(a) for x in r])
        assert d <= max(0.02, 1.5 * base), (pop, d, base)
        assert np.corrcoef(a, b)[0, 1] > 0.99, pop
