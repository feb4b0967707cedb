"""GPU-vs-oracle parity runs (test infrastructure).

`run_parity` steps one synthetic workload on the GPU with every random draw recorded, then
replays the same steps with the CPU oracle in the reference's order, feeding it the recorded
draws, and returns both sides' per-step records for comparison.

Two modes for the LGN tables: `own_tables=True` makes the oracle use its own restated
store_PM tables and its own emulation of the texture sampling (an end-to-end check, where the
9-bit texture weights can move a few LGN spikes); `own_tables=False` feeds it the GPU's
tables after they were compared separately, so that the V1 dynamics can be compared spike for
spike.
"""
from __future__ import annotations

import numpy as np

from . import LgnOracle, V1Oracle

f32 = np.float32


def record_layout(spec):
    """Offsets of the fields inside one rawData record."""
    n = spec.nV1
    h = 1 if spec.hWrite else 0
    o = {"sInfo": 0, "dep": n}
    off = 2 * n
    if spec.iModel == 1:
        o["w"] = off
        off += n
    o["v"] = off
    off += n
    o["gFF"] = off
    off += spec.ngFF * n
    if h:
        o["hFF"] = off
        off += spec.ngFF * n
    o["gE"] = off
    off += spec.ngE * n
    o["gI"] = off
    off += spec.ngI * n
    if h:
        o["hE"] = off
        off += spec.ngE * n
        o["hI"] = off
        off += spec.ngI * n
    return o


def split_record(spec, rec):
    o = record_layout(spec)
    n = spec.nV1
    sizes = dict(sInfo=n, dep=n, w=n, v=n, gFF=spec.ngFF * n, hFF=spec.ngFF * n, gE=spec.ngE * n,
                 gI=spec.ngI * n, hE=spec.ngE * n, hI=spec.ngI * n)
    return {k: rec[..., v:v + sizes[k]] for k, v in o.items()}


LEARN_KEYS = ("sLGN", "ff_post", "total_ff")


def run_parity(wl, nsteps: int, cap: int = 8, own_tables: bool = False, sim=None, learning=None):
    """learning: a model.FFLearning to run with LGN->V1 plasticity on both sides; the final
    weights, post variables, homeostasis totals and presynaptic traces come back under
    gpu/oracle "learn"."""
    from visual_cortex_gb300.model import Simulation
    from visual_cortex_gb300 import _native as N

    close = sim is None
    if sim is None:
        sim = Simulation(wl.spec, wl.net, wl.lgn, wl.stim, wl.init, wl.seeds,
                         record_init=4 * cap if wl.seeds.has_sp0() else 0)
    init_rec = sim.init_record
    if wl.seeds.has_sp0() and init_rec is None:
        raise ValueError("initial spikes: the Simulation must be made with record_init > 0")
    try:
        if learning is not None:
            sim.set_ff_learning(learning)
        gpu_tables = sim.lgn_tables()
        gpu_S = sim.lgn_spatial()
        gpu_parvo = (sim.lgn_parvo_tables(), sim.lgn_parvo_spatial()) if wl.lgn.nParvo else None
        lnl0 = sim.state("lgn_lnl")
        ltr0 = sim.state("lgn_ltr")
        sim.set_record(N.REC_RAW | N.REC_LGN_SP | N.REC_LGN_FR, nsteps + 1)
        sim.set_draw_record(nsteps, cap)
        sim.run(nsteps)
        raw, lsp, lfr = sim.fetch_records(0, nsteps, raw=True, lgn_sp=True, lgn_fr=True)
        U, Uc = sim.fetch_draws(0)
        noise, _ = sim.fetch_draws(1)
        ff, _ = sim.fetch_draws(2)
        near, _ = sim.fetch_draws(3)
        final = {k: sim.state(k) for k in ("v", "gE", "gI", "gFF", "tBack")}
        learn = None
        if learning is not None:
            learn = {k: sim.state(k) for k in LEARN_KEYS}
            learn["ff_pre"] = sim.state("ff_pre")
        launches = sim.launches()
    finally:
        if close:
            sim.close()

    lo = LgnOracle(wl.lgn, wl.stim)
    ora_tables = (lo.TW.copy(), lo.SW.copy(), lo.SC.copy(), lo.maxConvol.copy())
    ora_S = lo.spatial()
    if not own_tables:
        TW, SW, SC, mc = gpu_tables
        lo.TW[:] = TW
        lo.maxConvol[:] = mc
        lo.S = np.ascontiguousarray(gpu_S)
        if gpu_parvo is not None:
            (pTW, _, _), PS = gpu_parvo
            lo.pTW[:] = pTW
            lo.PS = np.ascontiguousarray(PS)
    # the initial carried integrals come from the library's LGN generators (the oracle does
    # not re-derive cuRAND); those generators and lastNegLogRand are held byte for byte to the
    # reference's own logRand_init (tests/test_ref_kernels.py), so the copy carries no
    # unchecked state into the comparison
    lo.lnl[:] = lnl0
    lo.ltr[:] = ltr0
    vo = V1Oracle(wl.spec, wl.net)
    vo.set_state(wl.init)
    vo.set_far_failure(wl.seeds.far_engine_seed, wl.seeds.nChunk)
    if learning is not None:
        vo.set_ff_learning(learning)
        mode = int(learning.learning)
        n_types = 0 if mode == 4 else 1 + (int(learning.nLearnTypeFF_I) if mode == 2 else 0)
    mism = 0
    o_hist = None
    if wl.seeds.has_sp0():
        m0, o_hist = vo.init_spikes(wl.seeds.sp0, wl.seeds.SCsplit, wl.seeds.trainDepth, init_rec)
        mism += m0
    nV1 = wl.spec.nV1
    o_raw = np.zeros_like(raw)
    o_lsp = np.zeros_like(lsp)
    o_lfr = np.zeros_like(lfr)
    lay = record_layout(wl.spec)
    for it in range(nsteps):
        conv = lo.convol(it)
        s, fr, m = lo.nonlinear(conv, np.ascontiguousarray(U[it]), np.ascontiguousarray(Uc[it]), cap)
        mism += m
        o_lsp[it] = s
        o_lfr[it] = fr
        if learning is not None and mode != 4:
            pre_start, pre_spike = lo.ff_pre(learning.tauLTP, 0)
            if n_types > 1:
                lo.ff_pre(learning.tauLTP_I, 1)
        vo.step(s, noise=noise[it], ff=np.ascontiguousarray(ff[it]), near=np.ascontiguousarray(near[it]), cap=cap)
        if learning is not None:
            if mode != 4:
                vo.learn_ff(s, pre_start, pre_spike)
            if mode != 3:
                vo.learn_avg()
        r = o_raw[it]
        r[lay["sInfo"]:lay["sInfo"] + nV1] = vo.get("sInfo")
        r[lay["dep"]:lay["dep"] + nV1] = vo.get("dep")
        if "w" in lay:
            r[lay["w"]:lay["w"] + nV1] = vo.get("w")
        r[lay["v"]:lay["v"] + nV1] = vo.get("v")
        for k in ("gFF", "hFF", "gE", "gI", "hE", "hI"):
            if k in lay:
                a = vo.get(k)
                r[lay[k]:lay[k] + a.size] = a
    o_final = {k: vo.get(k) for k in ("v", "gE", "gI", "gFF", "tBack")}
    o_learn = None
    if learning is not None:
        o_learn = {k: vo.get(k) for k in LEARN_KEYS}
        o_learn["ff_pre"] = (np.concatenate([lo.ff_vars[k] for k in range(n_types)]) if n_types
                             else np.zeros(0, f32))
    vo.close()
    return dict(gpu=dict(raw=raw, lsp=lsp, lfr=lfr, tables=gpu_tables, S=gpu_S, final=final,
                         history=None if init_rec is None else init_rec["history"], learn=learn),
                ora=dict(raw=o_raw, lsp=o_lsp, lfr=o_lfr, tables=ora_tables, S=ora_S, final=o_final,
                         history=o_hist, learn=o_learn),
                draw_count_mismatch=mism, launches=launches)


def first_divergence(a_sinfo, b_sinfo):
    """First step at which the spike rasters (sInfo >= 1) differ, or None."""
    sa = a_sinfo >= 1
    sb = b_sinfo >= 1
    diff = np.nonzero((sa != sb).any(axis=1))[0]
    return int(diff[0]) if diff.size else None


def knife_edge(spec, a_sinfo, b_sinfo, step, eps_mv=1e-3):
    """True if every raster difference at `step` is a threshold crossing decided by float
    rounding: on the side that did not spike the membrane sits within eps_mv of vThres."""
    sa, sb = a_sinfo[step] >= 1, b_sinfo[step] >= 1
    idx = np.nonzero(sa != sb)[0]
    vthr = np.asarray(spec.vThres, dtype=np.float64)[spec.type_of(idx % spec.blockSize)]
    v_other = np.where(sa[idx], b_sinfo[step][idx], a_sinfo[step][idx])
    return bool(np.all(np.abs(v_other - vthr) < eps_mv))


def first_spike_time_divergence(a_v1, b_v1, a_lgn, b_lgn, tol_tsp):
    """First step at which a V1 or LGN spike present on both sides differs in its time by
    more than tol_tsp (in units of dt), or the rasters differ; None if never."""
    n = a_v1.shape[0]
    for t in range(n):
        for a, b in ((a_v1[t], b_v1[t]), (a_lgn[t], b_lgn[t])):
            sa, sb = a >= 1, b >= 1
            if (sa != sb).any():
                return t
            if sa.any() and np.max(np.abs(a[sa] - b[sa])) > tol_tsp:
                return t
    return None


def avg_floor_flips(spec, words_a, words_b):
    """Per excitatory neuron (E ids, block-major), the number of steps at which floor() of the
    two runs' spike words differ.  With learning != 3 the delivery adds floor(word) to vAvgE
    every step (src/coredynamics.cu:2548-2560), and a word that holds the membrane potential
    (no spike) within an ulp of an integer floors to neighbouring integers on the two sides:
    each such step moves vAvgE by 1 (decayed since)."""
    a = np.floor(np.asarray(words_a, np.float32)).reshape(len(words_a), spec.nblock, spec.blockSize)
    b = np.floor(np.asarray(words_b, np.float32)).reshape(len(words_b), spec.nblock, spec.blockSize)
    return (a != b)[:, :, :spec.nE].sum(axis=0).reshape(-1)


def compare_avg(got, want, flips, rtol=1e-5):
    """vAvgE [nEt][2] of two runs: entries of neurons without floor flips within rtol of the
    largest value; a neuron with k flips differs by at most k (+ rtol).  Returns the largest
    relative error over the neurons without flips."""
    got = np.asarray(got, np.float64).reshape(-1, 2)
    want = np.asarray(want, np.float64).reshape(-1, 2)
    scale = max(np.abs(want).max(), 1e-30)
    d = np.abs(got - want).max(axis=1)
    ok = flips == 0
    assert np.all(d[~ok] <= flips[~ok] + rtol * scale), (d[~ok], flips[~ok])
    return float(d[ok].max() / scale) if ok.any() else 0.0


def compare(res, spec, tol_tsp=1e-5):
    """Summary numbers of a parity run (all assertions are left to the caller).

    Traces are compared up to the first spike-time divergence: the first step at which a
    spike (V1 or LGN) present in both runs differs in time by more than tol_tsp of a step,
    or a spike is present in only one run.

    Membrane traces are compared relative to |v|; conductance traces relative to the
    largest value of that conductance over the population at the same step (a conductance
    that is decaying towards 0 has no meaningful relative error of its own)."""
    g, o = res["gpu"], res["ora"]
    G = split_record(spec, g["raw"])
    O = split_record(spec, o["raw"])
    nsteps = g["raw"].shape[0]
    div = first_divergence(G["sInfo"], O["sInfo"])
    tdiv = first_spike_time_divergence(G["sInfo"], O["sInfo"], g["lsp"], o["lsp"], tol_tsp)
    upto = nsteps if tdiv is None else tdiv
    out = {"first_raster_divergence": div, "first_spike_time_divergence": tdiv, "steps": nsteps,
           "divergence_is_knife_edge": None if div is None else knife_edge(spec, G["sInfo"], O["sInfo"], div)}
    full_v = np.abs(G["v"].astype(np.float64) - O["v"]) / np.maximum(np.abs(O["v"]), 1.0)
    out["max_rel_v_to_raster_divergence"] = float(full_v[:nsteps if div is None else div].max()) if (div is None or div) else 0.0
    for k in ("v", "gE", "gI", "gFF"):
        a, b = G[k][:upto].astype(np.float64), O[k][:upto].astype(np.float64)
        if not upto:
            out[f"max_rel_{k}"] = 0.0
            continue
        if k == "v":
            scale = np.maximum(np.abs(b), 1.0)
        else:
            scale = np.maximum(np.abs(b).max(axis=1, keepdims=True), 1e-12)
        out[f"max_rel_{k}"] = float(np.max(np.abs(a - b) / scale))
    both = (G["sInfo"][:upto] >= 1) & (O["sInfo"][:upto] >= 1)
    out["v1_tsp_maxdiff"] = float(np.max(np.abs(G["sInfo"][:upto][both] - O["sInfo"][:upto][both]))) if both.any() else 0.0
    lg = g["lsp"] >= 1
    lo_ = o["lsp"] >= 1
    out["lgn_spike_mismatch"] = int((lg != lo_).sum())
    out["lgn_spikes"] = int(lg.sum())
    out["v1_spikes_gpu"] = int((G["sInfo"] >= 1).sum())
    out["v1_spikes_ora"] = int((O["sInfo"] >= 1).sum())
    both = lg & lo_
    out["lgn_tsp_maxdiff"] = float(np.max(np.abs(g["lsp"][both] - o["lsp"][both]))) if both.any() else 0.0
    out["lgn_fr_maxrel"] = float(np.max(np.abs(g["lfr"] - o["lfr"]) / np.maximum(np.abs(o["lfr"]), 1e-3)))
    return out
