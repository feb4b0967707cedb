"""Writes tests/golden/ref_kernels.npz: outputs of the reference's OWN GPU kernels on the seeded
cases of oracle/ref_cases.py (plus the inputs that cannot be rebuilt from seeds).

The kernels come from oracle/_ref/ref_kernels.cubin, which oracle/ref/build_ref_kernels.sh
compiles from the reference's sources where they lie; oracle/ref/ref_kernel_runner.cu (built
here with nvcc) loads that module and launches the kernels as the reference's step loop does.
Run from the repository root on a machine with a GPU:

  REFERENCE_SRC=<reference checkout>/src bash oracle/ref/build_ref_kernels.sh   # where the sources are
  python tests/golden/make_ref_kernel_golden.py [out.npz]                        # on the GPU machine
  python tests/golden/make_ref_kernel_golden.py --learning [out.npz]             # ref_learning.npz

Cases:
  lgn_*    logRand_init + 48 steps of LGN_nonlinear (512 cells, seeded drive)
  magno_*  store_PM (magno cells) + 400 steps of LGN_convol_magno (128 cells, grating movie)
  init0_*  rand_spInit without initial spikes (2 x 1024 neurons)
  init1_*  rand_spInit with initial spikes (spE0/spI0 > 0)
  run_*    rand_spInit, then 160 steps of compute_V_collect_spike_learnFF_fast +
           recal_G_mat_nd_fast on the LGN spike words of the library's own run of the workload
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

from oracle import ref_cases as RC  # noqa: E402

REF = os.path.join(ROOT, "oracle", "_ref")
CUBIN = os.path.join(REF, "ref_kernels.cubin")
RUNNER = os.path.join(REF, "ref_kernel_runner")


def build_runner():
    src = os.path.join(ROOT, "oracle", "ref", "ref_kernel_runner.cu")
    subprocess.run(["nvcc", "-O2", "-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a", "-o", RUNNER,
                    src, "-lcuda"], check=True)


def run(mode, inputs):
    with tempfile.TemporaryDirectory() as d:
        fi, fo = os.path.join(d, "in.bin"), os.path.join(d, "out.bin")
        RC.write_bundle(fi, inputs)
        subprocess.run([RUNNER, CUBIN, mode, fi, fo], check=True)
        return RC.read_bundle(fo)


def learning(out_path):
    """ref_learning.npz: LGN_nonlinear with learning = 3 (the presynaptic trace of each cell per
    step: at the end, at the start, right after its spikes) on the LGN case, and 120 V1 steps of
    compute_V_collect_spike_learnFF_fast + recal_G_mat_nd_fast with learning = 3 (v1_*), learning = 2
    (v2_*) and learning = 4 (v4_*) on the LGN spike words of the library's own run, the presynaptic traces
    given per step."""
    res = {}
    lo = run("lgnlearn", RC.lgn_learn_case())
    for k, v in lo.items():
        res["lgn_" + k] = v
    wl = RC.v1_workload(sp=False)
    from visual_cortex_gb300 import _native as N
    from visual_cortex_gb300.model import Simulation
    sim = Simulation(wl.spec, wl.net, wl.lgn, wl.stim, wl.init, wl.seeds)
    try:
        sim.set_record(N.REC_LGN_SP, RC.LEARN_T + 1)
        sim.run(RC.LEARN_T)
        _, lsp, _ = sim.fetch_records(0, RC.LEARN_T, raw=False, lgn_sp=True, lgn_fr=False)
    finally:
        sim.close()
    vi = RC.v1_learn_inputs(wl, np.asarray(lsp, np.float32), RC.LEARN_T)
    o = run("v1learn", vi)
    res["v1_lgnSInfo"] = np.asarray(lsp, np.float32)
    res["v1_preStart"] = vi["preStart"].reshape(RC.LEARN_T, -1)
    res["v1_preSpk"] = vi["preSpk"].reshape(RC.LEARN_T, -1)
    for k in RC.STATE_KEYS:
        res["v1_in_" + k] = vi[k]
    for k, v in o.items():
        res["v1_" + k] = v
    # learning = 2: both FF types, vAvgE through the delivery with a cortical E type's tauAvg
    v2 = RC.v1_learn_inputs(wl, np.asarray(lsp, np.float32), RC.LEARN_T, RC.learning_params2())
    o2 = run("v1learn", v2)
    for k, v in o2.items():
        res["v2_" + k] = v
    # learning = 4: no FF learning, vAvgE through the delivery only
    o4 = run("v1learn", RC.v1_learn_inputs(wl, np.asarray(lsp, np.float32), RC.LEARN_T, RC.learning_params4()))
    for k, v in o4.items():
        res["v4_" + k] = v
    np.savez_compressed(out_path, **res)
    print(f"wrote {out_path}: {len(res)} arrays; v1: {(o['raster'] >= 1).sum()} V1 spikes, "
          f"max |dw| {np.abs(o['sLGN'] - wl.net.sLGN.reshape(-1)).max():.3g}")


def main():
    if len(sys.argv) > 1 and sys.argv[1] == "--learning":
        if not os.path.exists(CUBIN):
            raise SystemExit(f"{CUBIN} is missing: run oracle/ref/build_ref_kernels.sh where the reference's sources are")
        build_runner()
        learning(sys.argv[2] if len(sys.argv) > 2 else os.path.join(ROOT, "tests", "golden", "ref_learning.npz"))
        return
    out_path = sys.argv[1] if len(sys.argv) > 1 else os.path.join(ROOT, "tests", "golden", "ref_kernels.npz")
    if not os.path.exists(CUBIN):
        raise SystemExit(f"{CUBIN} is missing: run oracle/ref/build_ref_kernels.sh where the reference's sources are")
    build_runner()
    res = {}

    # LGN generators and LGN_nonlinear
    li = RC.lgn_case()
    lo = run("lgn", li)
    for k, v in lo.items():
        res["lgn_" + k] = v

    # store_PM (magno) and LGN_convol_magno over a grating movie
    mo = run("magno", RC.magno_inputs(RC.magno_workload()))
    for k, v in mo.items():
        res["magno_" + k] = v

    # rand_spInit without and with initial spikes
    wl0 = RC.v1_workload(sp=False)
    o = run("v1init", RC.v1_inputs(wl0))
    for k in ("rGenCond", "rNoisy", "spikeTrain", "v", "w", "tBack", "npre"):
        res["init0_" + k] = o[k]
    wl1 = RC.v1_workload(sp=True)
    i1 = RC.v1_inputs(wl1, sp0=wl1.seeds.sp0)
    o = run("v1init", i1)
    for k in ("rGenCond", "rNoisy", "spikeTrain", "v", "w", "tBack", "npre"):
        res["init1_" + k] = o[k]
    for k in RC.STATE_KEYS:
        res["init1_in_" + k] = i1[k] if k in i1 else np.zeros(0, np.float32)

    # the V1 steps on the LGN spike words of the library's own run of the same workload
    from visual_cortex_gb300 import _native as N
    from visual_cortex_gb300.model import Simulation
    sim = Simulation(wl0.spec, wl0.net, wl0.lgn, wl0.stim, wl0.init, wl0.seeds)
    try:
        sim.set_record(N.REC_LGN_SP, RC.V1_T + 1)
        sim.run(RC.V1_T)
        _, lsp, _ = sim.fetch_records(0, RC.V1_T, raw=False, lgn_sp=True, lgn_fr=False)
    finally:
        sim.close()
    ri = RC.v1_inputs(wl0, lgn_rows=lsp, T=RC.V1_T)
    o = run("v1run", ri)
    res["run_lgnSInfo"] = np.asarray(lsp, np.float32)
    for k in RC.STATE_KEYS:
        res["run_in_" + k] = ri[k]
    for k, v in o.items():
        res["run_" + k] = v
    np.savez_compressed(out_path, **res)
    sp = (o["raster"] >= 1).sum()
    print(f"wrote {out_path}: {len(res)} arrays; run: {sp} V1 spikes in {RC.V1_T} steps; "
          f"lgn: {(lo['sInfo'] >= 1).sum()} LGN spikes")


if __name__ == "__main__":
    main()
