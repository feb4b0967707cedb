#!/usr/bin/env python3
"""Benchmark: V1 neuron-steps/s of the patchV1 hot path on GB300.

Workload (the full-patch configuration): 32 blocks x 1024 = 32,768 V1 neurons (80% LIF E /
20% AdEx I), 16,384 ON/OFF magno LGN cells on 128x128 drifting-grating frames at 120 Hz,
~400 far partners per neuron with distance delays, dense within-block connectivity,
dt = 0.125 ms, fp32, seeded synthetic data.

One bench step = `--sim-steps` simulation steps (default 800 = 100 ms simulated) of the whole
loop (LGN convolution + LGN spikes + V1 step + near and far delivery).  Between timed bench
steps L2 is flushed by writing a 512 MiB buffer.  `value` is device time (CUDA events on the
plan's stream); `e2e` runs the same bench step through the public API from host buffers:
stimulus upload (H2D) + the steps + spike-raster download (D2H), wall-clock timed.

`--impl reference` times the CPU implementation of the path (the oracle's restatement of the
reference's kernels and host far delivery, OpenMP on all host cores) on the same workload.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import tempfile
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "V1 neuron-steps/s fwd and fwd+adjoint, batched vs plain on one GB300 at tol"
UNIT = "neuron-steps/s"
L2_FLUSH = 512 << 20


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class Clocks:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        # the raw samples: PV1_CLOCKS_DIR if set (to keep them), else a temporary folder
        folder = os.environ.get("PV1_CLOCKS_DIR") or tempfile.mkdtemp(prefix="pv1_clocks_")
        self.path = os.path.join(folder, f"clocks_dev{device}.csv")

    def __enter__(self):
        try:
            os.makedirs(os.path.dirname(self.path), exist_ok=True)
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"], stdout=self.f,
                stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None
        time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()
            self.f.close()

    def summary(self):
        if self.proc is None or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        sm, smax, reasons = [], [], set()
        names = ["active", "hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            parts = [x.strip() for x in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names[1:], parts[5:9]):
                if v.lower() in ("active", "1", "0x1"):
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": float(max(smax)),
                "reasons": sorted(reasons), "samples": len(sm)}


def load_peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def load_traffic(kernel: str):
    path = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(path):
        with open(path) as f:
            t = json.load(f)
        return t.get(kernel)
    return None


def algorithmic_bytes_per_neuron_step(wl, rate_hz: float) -> float:
    """Bytes per V1 neuron-step the step kernel must move (state read+write, LGN synapses,
    LGN spike words, and the per-spike conMat column and far fan-out)."""
    s = wl.spec
    S = 3 + 2 * (s.ngFF + s.ngE + s.ngI)
    m = float(np.mean(wl.net.nLGNperV1))
    nlgn_over_n = wl.lgn.nLGN / s.nV1
    k_far = float(np.mean(wl.net.nVec)) if wl.net.nVec.size else 0.0
    n_nb = float(np.mean(wl.net.nNearNB))
    r_dt = rate_hz * s.dt * 1e-3
    return 8 * S + 12 + 8 * m + 8 * nlgn_over_n + r_dt * (4 * s.blockSize * n_nb + 16 * k_far)


def build_workload(name: str, host_init=None):
    """The seeded synthetic workload.  host_init: who draws the initial state (the library by
    default; the reference arm passes the oracle's restatement, so it maps no product code)."""
    from visual_cortex_gb300 import synth
    if name == "C1":
        return synth.config1(seed=0, host_init=host_init)
    return synth.config2(seed=0, host_init=host_init)


def bench_config(name: str, wl) -> dict:
    """The `config` object of both arms' JSON lines (identical by construction)."""
    return {"workload": ("32x1024 V1 (80% LIF E / 20% AdEx I), 16384 magno LGN, 128x128 grating "
                         "120 Hz, ~400 far partners/neuron, dt 0.125 ms") if name == "C2"
            else "1x1024 V1, 512 LGN, 64x64 grating, dt 0.125 ms",
            "nV1": wl.spec.nV1, "nLGN": wl.lgn.nLGN, "seed": 0, "mode": "plain forward",
            "unit_of_work": "one V1 neuron advanced by one 0.125 ms step (LGN, V1 step, near and far delivery)",
            "l2": "GPU arm: L2 flushed (512 MiB write) before each timed bench step; CPU arm: not applicable"}


def run_gb300(args):
    rank, world, local = dist_env()
    from visual_cortex_gb300.build import build_native
    build_native()
    from visual_cortex_gb300 import _native as N
    from visual_cortex_gb300.model import Simulation, Stimulus

    N.check(None, N.lib.pv1_set_device(local), "pv1_set_device")
    dist = None
    if world > 1:
        import torch
        import torch.distributed as td
        torch.cuda.set_device(local)
        td.init_process_group("nccl")
        dist = td

    wl = build_workload(args.config)
    S = args.sim_steps
    sim = Simulation(wl.spec, wl.net, wl.lgn, wl.stim, wl.init, wl.seeds)
    for _ in range(args.warmup):
        sim.run_timed(S, L2_FLUSH)
    if dist:
        dist.barrier()
    times = []
    launches = 0
    with Clocks(local) as clk:
        for _ in range(args.steps):
            times.append(sim.run_timed(S, L2_FLUSH))
            launches += sim.launches()
    total_ms = float(np.sum(times))
    if dist:
        import torch
        t = torch.tensor([total_ms], device=f"cuda:{local}")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        total_ms = float(t.item())
    neuron_steps = wl.spec.nV1 * S * args.steps * world
    value = neuron_steps / (total_ms * 1e-3)

    # per-kernel device time (direct launches, events around each launch)
    v1_ms, lgn_ms, chunk = sim.time_kernels(320)
    persistent = sim.persistent()

    # end to end through the public API from page-locked host buffers: the stimulus movie in
    # (and its per-frame spatial stage), the spike raster of every step out
    sim.set_record(N.REC_SPIKES, S + 1)
    frames = N.pinned_empty(wl.stim.frames.shape, np.float32)
    frames[...] = wl.stim.frames
    stim = Stimulus(frames=frames, init_LMS=wl.stim.init_LMS)
    raster = N.pinned_empty((S, wl.spec.nV1), np.float32)
    e2e_times, spikes = [], 0
    for q in range(max(1, args.steps)):
        t0 = time.perf_counter()
        sim.load_stimulus(stim)
        sp = sim.run_spikes_to_host(S, raster)
        e2e_times.append(time.perf_counter() - t0)
        spikes += int((sp >= 1).sum())
    e2e_s = float(np.sum(e2e_times))
    e2e_value = wl.spec.nV1 * S * len(e2e_times) * world / e2e_s
    rate_hz = spikes / (wl.spec.nV1 * S * len(e2e_times) * wl.spec.dt * 1e-3)
    sim.close()

    peak, peak_kind = load_peaks()
    bpn = algorithmic_bytes_per_neuron_step(wl, rate_hz)
    # the dominant kernel: one cooperative launch per chunk of steps, or one launch per step
    kernel = "v1_persistent_kernel" if persistent else "v1_step_kernel"
    steps_per_launch = chunk if persistent else 1
    bytes_per_launch = bpn * wl.spec.nV1 * steps_per_launch
    launch_ms = v1_ms * steps_per_launch
    achieved = bytes_per_launch / (launch_ms * 1e-3) / 1e9
    traffic = load_traffic(kernel)

    out = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": total_ms / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded)",
        "config": bench_config(args.config, wl),
        "sim_steps_per_bench_step": S, "v1_rate_hz": rate_hz,
        "e2e": {"value": e2e_value, "unit": UNIT,
                "h2d_bytes_per_step": int(wl.stim.frames.nbytes),
                "d2h_bytes_per_step": int(S * wl.spec.nV1 * 4)},
        "gpu_launches": int(launches),
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                     "frac": achieved / peak, "traffic": traffic,
                     "kernel": kernel, "peak_source": f"{peak_kind} hbm_gbs",
                     "algorithmic_bytes_per_launch": bytes_per_launch, "steps_per_launch": steps_per_launch,
                     "algorithmic_bytes_per_neuron_step": bpn,
                     "launch_ms": launch_ms, "lgn_chunk_ms": lgn_ms, "lgn_chunk_steps": chunk},
        "clocks": clk.summary(),
    }
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(wl, args.cpu_sample_steps)
    if rank == 0 and not args.no_forms:
        del wl, sim
        forms = {"batched": bench_batched(args.batch_trials)}
        forms["batched"]["vs_plain"] = forms["batched"]["value"] / value
        bound = out.get("cpu_baseline", {}).get("reference_plain_gpu_bound")
        if bound:
            forms["batched"]["vs_reference_plain_gpu_bound"] = forms["batched"]["value"] / bound["value"]
        forms["adjoint"] = bench_adjoint()
        forms["lgn_bf16"] = bench_lgn_bf16()
        out["forms"] = forms
    if dist:
        dist.barrier()
        dist.destroy_process_group()
    return out if rank == 0 else None


def bench_batched(n_trials: int):
    """The batched sweep: n_trials instances of an 8 x 1024 patch, 12 orientations, contrast
    U[0.1, 1], durations U[250, 2000] ms, all run to their ends by one Batch, twice: in
    autotuned chunks, and as one graph with one cooperative V1 launch (pv1_batch_sweep, the
    line's value).  Value = sum over trials of neurons x steps / device time of the sweep."""
    from visual_cortex_gb300 import synth
    from visual_cortex_gb300.batch import Batch
    from visual_cortex_gb300.model import Simulation
    trials = synth.batch_trials(n_trials=n_trials, seed=0)
    t0 = time.perf_counter()
    sims = [Simulation(t.wl.spec, t.wl.net, t.wl.lgn, t.wl.stim, t.wl.init, t.wl.seeds) for t in trials]
    b = Batch(sims, [t.steps for t in trials], autotune=True)
    _, ms = b.run()
    rates = [b.stats(q)[1] for q in range(len(trials))]
    e2e_s = time.perf_counter() - t0
    launches = b.launches()
    tuning = b.tuning()
    b.close()
    for s in sims:
        s.close()
    work = sum(t.steps * t.wl.spec.nV1 for t in trials)
    # the same trials as one graph of three launches (pv1_batch_sweep): the LGN stage of every
    # step, ONE cooperative V1 launch (slots run their trials longest first), the advance
    t0 = time.perf_counter()
    sims = [Simulation(t.wl.spec, t.wl.net, t.wl.lgn, t.wl.stim, t.wl.init, t.wl.seeds) for t in trials]
    b = Batch(sims, [t.steps for t in trials], autotune=False)
    sweep_ms = b.sweep()
    sweep_rates = [b.stats(q)[1] for q in range(len(trials))]
    sweep_e2e_s = time.perf_counter() - t0
    sweep_launches = b.launches()
    b.close()
    for s in sims:
        s.close()
    sweep = {"value": work / (sweep_ms * 1e-3), "unit": UNIT, "device_ms": sweep_ms,
             "gpu_launches": sweep_launches, "e2e": {"value": work / sweep_e2e_s, "unit": UNIT},
             "mean_rate_hz": float(np.mean(sweep_rates)),
             "same_rates_as_chunked": bool(np.array_equal(np.float64(rates), np.float64(sweep_rates)))}
    chunked = {"value": work / (ms * 1e-3), "unit": UNIT, "device_ms": ms, "gpu_launches": launches,
               "tuning": tuning, "e2e": {"value": work / e2e_s, "unit": UNIT}}
    return {"value": sweep["value"], "unit": UNIT, "device_ms": sweep_ms,
            "e2e": {"value": work / sweep_e2e_s, "unit": UNIT,
                    "note": "plan creation with all host->device uploads, the sweep and the FP64 rate read-back"},
            "workload": f"{n_trials} trials x 8x1024 V1 / 4096 LGN, 128x128 gratings at 12 orientations, "
                        "contrast U[0.1,1], durations U[250,2000] ms, dt 0.125 ms",
            "neuron_steps": work, "trial_steps": [t.steps for t in trials], "gpu_launches": sweep_launches,
            "one_launch_sweep": sweep, "chunked_autotuned": chunked, "mean_rate_hz": float(np.mean(rates))}


def bench_adjoint(reps: int = 3):
    """The differentiable form: 4096 neurons x batch 16 x 4000 steps (0.125 ms), 30 LGN weights
    per neuron, fast-sigmoid surrogate (slope 5/mV), loss = MSE of 20 ms-window rates against a
    teacher with perturbed weights.  Forward alone vs forward + adjoint (checkpoints every 64
    steps), device time with CUDA events on torch's stream."""
    import torch
    from visual_cortex_gb300.adjoint import make_patch, rate_loss
    patch, W0 = make_patch(B=16, nblock=4, T=4000, K=30, seed=0)
    c = patch.cfg
    rng = np.random.default_rng(1)
    W = torch.tensor(W0, device="cuda")
    WT = torch.tensor(np.maximum(W0 * (1 + 0.2 * rng.standard_normal(W0.shape)), 0).astype(np.float32),
                      device="cuda")
    tE = torch.tensor(5.0, dtype=torch.float64, device="cuda", requires_grad=True)
    tI = torch.tensor(7.0, dtype=torch.float64, device="cuda", requires_grad=True)
    with torch.no_grad():
        target, _ = patch.forward(WT, tE.detach(), tI.detach())
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]

    def fwd():
        with torch.no_grad():
            return patch.forward(W, tE.detach(), tI.detach())

    def fwd_bwd():
        Wg = W.clone().requires_grad_(True)
        r, _ = patch.forward(Wg, tE, tI)
        loss = rate_loss(r, target)
        loss.backward()
        return loss, Wg.grad

    fwd(); fwd_bwd()
    torch.cuda.synchronize()
    ev[0].record()
    for _ in range(reps):
        rates, _ = fwd()
    ev[1].record()
    ev[2].record()
    for _ in range(reps):
        loss, g = fwd_bwd()
    ev[3].record()
    torch.cuda.synchronize()
    f_ms = ev[0].elapsed_time(ev[1]) / reps
    fb_ms = ev[2].elapsed_time(ev[3]) / reps
    work = c.B * c.N * c.T
    return {"fwd": {"value": work / (f_ms * 1e-3), "unit": UNIT, "ms": f_ms},
            "fwd_adjoint": {"value": work / (fb_ms * 1e-3), "unit": UNIT, "ms": fb_ms},
            "fwd_adjoint_over_fwd_time": fb_ms / f_ms,
            "workload": "4096 neurons (4x1024) x batch 16 x 4000 steps, 30 LGN weights/neuron, "
                        "checkpoint every 64 steps, grads wrt W and AMPA/GABA decay",
            "mean_rate_hz": float(rates.mean()), "loss": float(loss.detach()),
            "grad_norm_W": float(g.norm()), "grad_tauE": float(tE.grad), "grad_tauI": float(tI.grad)}


def bench_lgn_bf16():
    """LGN convolution at scale: 16384 ON/OFF cells, 31x31-pixel DoG footprints (sigma +-20%),
    250-tap temporal kernel, 256x256 1/f^2 noise frames at 120 Hz for 2 s (16000 steps).  The
    temporal contraction as tcgen05 BF16 MMAs (FP32 accumulate) vs the same tiles in FP32 on CUDA
    cores, each followed by the logistic rate and Poisson spikes; rates against an FP64 oracle
    on 1024 cells x 250 steps."""
    from visual_cortex_gb300 import lgn_bf16 as L
    from visual_cortex_gb300 import _native as N
    from visual_cortex_gb300.model import Simulation
    wl = L.make_workload(seed=0)
    tc = L.LgnTensorCore(wl, fr_every=64)
    try:
        tc.run(tensor_cores=True)
        tc.run(tensor_cores=False)
        ms32 = float(np.median([tc.run(tensor_cores=False) for _ in range(3)]))
        _, _, fr32 = tc.fetch()
        ms16 = float(np.median([tc.run(tensor_cores=True) for _ in range(3)]))
        _, _, fr16 = tc.fetch()
        # the full-patch V1 (16384 LGN cells, as the stage) driven by the BF16 stage's spike
        # words for the whole 2 s (pv1_set_lgn_source)
        v1 = build_workload("C2")
        sim = Simulation(v1.spec, v1.net, v1.lgn, v1.stim, v1.init, v1.seeds)
        try:
            sim.set_lgn_source(tc.device_spikes(), 0, wl.T)
            sim.set_record(N.REC_SPIKES, 4097)
            drv_ms = sim.run_timed(4000, 0)
            counts = sim.fetch_spikes(0, 4000)
            sim.set_record(0, 2)
            drv_ms += sim.run_timed(wl.T - 4000, 0)
            driven = {"value": v1.spec.nV1 * wl.T / (drv_ms * 1e-3), "unit": UNIT, "ms": drv_ms,
                      "v1_rate_hz_first_500ms": float(np.floor(np.where(counts >= 1, counts, 0)).sum()) /
                      (v1.spec.nV1 * 4000 * wl.dt * 1e-3),
                      "e2e_stage_plus_v1_ms": ms16 + drv_ms,
                      "what": "the 32x1024 V1 of the headline workload stepped for the stage's 16000 steps on its "
                              "BF16 spike words (one device-to-device copy of each chunk's rows into the LGN ring)"}
        finally:
            sim.close()
    finally:
        tc.close()
    rng = np.random.default_rng(0)
    cells = np.sort(rng.choice(wl.nCells, 1024, replace=False))
    steps = np.arange(0, wl.T, 64)
    from oracle.lgn_fp64 import oracle_rates, rate_errors
    ref = oracle_rates(wl, cells, steps)
    work = wl.nCells * wl.T
    peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json"))) if os.path.exists(
        os.path.join(ROOT, "MEASURED_PEAKS.json")) else {}
    bf16_peak = peaks.get("bf16_tflops", 1900.0)
    flops = 2.0 * L.TILE_K * wl.T * wl.nCells          # MMA work as issued (K = 64 window)
    kf = 2.0 * 32 * wl.T * wl.nCells                    # algorithmic: ~32 frames per window
    out_bytes = 4.0 * wl.T * wl.nCells + 4.0 * len(range(0, wl.T, 64)) * wl.nCells
    return {"bf16_tensor": {"value": work / (ms16 * 1e-3), "unit": "LGN cell-steps/s", "ms": ms16,
                            "err_vs_fp64": rate_errors(fr16[:, cells], ref),
                            "tensor_tflops": kf / (ms16 * 1e-3) / 1e12,
                            "tensor_frac_of_measured_bf16": kf / (ms16 * 1e-3) / 1e12 / bf16_peak,
                            "mma_tflops_issued": flops / (ms16 * 1e-3) / 1e12,
                            "hbm_gbs_outputs": out_bytes / (ms16 * 1e-3) / 1e9},
            "fp32_cuda_cores": {"value": work / (ms32 * 1e-3), "unit": "LGN cell-steps/s", "ms": ms32,
                                "err_vs_fp64": rate_errors(fr32[:, cells], ref)},
            "speedup_bf16_over_fp32": ms32 / ms16,
            "v1_driven_by_bf16_stage": driven,
            "workload": "16384 ON/OFF cells, 31x31 px DoG (sigma +-20%), 250 taps, 256x256 1/f^2 noise, "
                        "120 Hz, 2 s (16000 steps at 0.125 ms)"}


def cpu_baseline(wl, nsteps: int):
    import oracle
    from oracle.baseline import CpuPatch, cpu_model, host_threads
    oracle.build()
    cp = CpuPatch(wl)
    cp.step(2)
    dt = cp.time_steps(nsteps)
    out = {"value": wl.spec.nV1 * nsteps / dt, "unit": UNIT, "cores": cp.threads, "kind": "port",
           "sample": f"{nsteps} steps of the same workload ({wl.spec.nV1} neurons), "
                     f"CPU restatement with OpenMP on {cp.threads} threads ({cpu_model()})",
           "seconds": dt}
    out["reference_plain_gpu_bound"] = reference_plain_bound(cp, wl)
    return out


def reference_plain_bound(cp, wl, nsteps: int = 12):
    """An upper bound on the reference's own plain-GPU rate for this workload: its step loop
    runs the far delivery (fill_fSpikeTrain + recal_G_vec, src/patch.cu:6597-6620) on one host
    thread every step, over every far synapse, whatever the GPU does meanwhile.  Timed here
    with the oracle's C restatement of that loop on one thread (contiguous arrays, so no
    slower than the reference's nested vectors), on the spike words of the CPU run above."""
    import time
    import oracle
    L = oracle.lib()
    L.orc_set_threads(1)
    vo = cp.vo
    sI = vo.get("sInfo")
    L.orc_v1_deliver_far(vo.h)
    t0 = time.perf_counter()
    for _ in range(nsteps):
        vo.put("sInfo", sI)
        L.orc_v1_deliver_far(vo.h)
    per = (time.perf_counter() - t0) / nsteps
    L.orc_set_threads(cp.threads)
    return {"value": wl.spec.nV1 / per, "unit": UNIT, "host_far_ms_per_step": per * 1e3,
            "far_synapses": int(np.sum(wl.net.nVec)),
            "how": "neurons / (time of the reference's per-step host far delivery, restated in C, one thread); "
                   "the reference's GPU work and its per-step host<->device copies only add to its step time"}


def run_reference(args):
    rank, world, local = dist_env()
    if rank != 0:
        return None
    import oracle
    from oracle.baseline import CpuPatch, cpu_model
    oracle.build()
    wl = build_workload(args.config, host_init=oracle.host_init_state)
    from visual_cortex_gb300 import _native
    assert not _native.loaded(), "the reference arm must not map the product library"
    cp = CpuPatch(wl)
    n = args.cpu_sample_steps
    for _ in range(args.warmup):
        cp.step(max(1, n // 4))
    times = [cp.time_steps(n) for _ in range(args.steps)]
    total = float(np.sum(times))
    value = wl.spec.nV1 * n * args.steps / total
    return {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": total / args.steps * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded)",
        "config": bench_config(args.config, wl),
        "sim_steps_per_bench_step": n,
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cp.threads, "kind": "port",
                         "sample": f"{n} simulation steps of the same workload per bench step (a bounded "
                                   f"sample; the GB300 arm runs 800), CPU restatement of the reference "
                                   f"kernels + host far delivery, OpenMP ({cpu_model()})"},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--config", default="C2", choices=["C1", "C2"])
    ap.add_argument("--sim-steps", type=int, default=800)
    ap.add_argument("--cpu-sample-steps", type=int, default=40)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-forms", action="store_true", help="skip the batched / adjoint / BF16 lines")
    ap.add_argument("--batch-trials", type=int, default=64)
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    out = run_reference(args) if args.impl == "reference" else run_gb300(args)
    if out is not None:
        print(json.dumps(out))


if __name__ == "__main__":
    main()
