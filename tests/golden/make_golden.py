"""Writes tests/golden/ref_golden.npz: inputs and the reference's own outputs for them.

The outputs come from oracle/_ref/ref_golden, built by oracle/ref/build_ref.sh from the
reference's sources (ConductanceShape, the AdEx struct, hStatic_nonlinear, find_denorm,
fill_fSpikeTrain + recal_G_vec, with and without synaptic failure, learnFF_pre/learnFF_post).  Run from the repository root, where the reference's
sources are readable:
  REFERENCE_SRC=<reference checkout>/src bash oracle/ref/build_ref.sh && python tests/golden/make_golden.py
"""
import os
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
BIN = os.path.join(ROOT, "oracle", "_ref", "ref_golden")
f32, u32, i32 = np.float32, np.uint32, np.int32


def run(mode, arr_in, dtype_out):
    with tempfile.TemporaryDirectory() as d:
        fi, fo = os.path.join(d, "in"), os.path.join(d, "out")
        with open(fi, "wb") as f:
            for a in (arr_in if isinstance(arr_in, (list, tuple)) else [arr_in]):
                f.write(np.ascontiguousarray(a).tobytes())
        subprocess.run([BIN, mode, fi, fo], check=True, stdout=subprocess.DEVNULL)
        return np.fromfile(fo, dtype=dtype_out)


def main():
    rng = np.random.default_rng(20261203)
    out = {}
    # ConductanceShape: rise, decay, g, h, f, dt
    n = 512
    cond = np.stack([rng.uniform(0.5, 3, n), rng.uniform(4, 90, n), rng.uniform(0, 2, n),
                     rng.uniform(0, 2, n), rng.uniform(0, 3, n), rng.uniform(0, 0.125, n)], 1).astype(f32)
    out["cond_in"] = cond
    out["cond_out"] = run("cond", cond, f32).reshape(n, 4)
    # AdEx: w0 tau_w a b v0 vR vThres gL C tRef vT deltaT dep gE0 gI0 gE1 gI1 dt
    ad = np.stack([rng.uniform(0, 0.5, n), rng.uniform(50, 200, n), rng.uniform(0, 0.05, n),
                   rng.uniform(0, 0.5, n), rng.uniform(-70, -49, n), np.full(n, -60.0), np.full(n, -50.0),
                   rng.uniform(0.03, 0.08, n), rng.uniform(0.8, 1.2, n), np.full(n, 2.0),
                   rng.uniform(-52, -48, n), rng.uniform(0.5, 2, n), rng.uniform(0, 1, n),
                   rng.uniform(0, 0.3, n), rng.uniform(0, 0.3, n), rng.uniform(0, 0.3, n),
                   rng.uniform(0, 0.3, n), rng.uniform(0.02, 0.125, n)], 1).astype(f32)
    out["adex_in"] = ad
    out["adex_out"] = run("adex", ad, f32).reshape(n, 5)
    # logistic a, b
    spont = rng.uniform(0, 0.3, n).astype(f32)
    c50 = rng.uniform(0.05, 0.6, n).astype(f32)
    sharp = rng.uniform(1, 10, n).astype(f32)
    out["logistic_in"] = np.stack([spont, c50, sharp])
    out["logistic_out"] = run("logistic", [spont, c50, sharp], f32).reshape(2, n)
    # find_denorm: (frame rate, step rate, MorN) pairs of common settings
    pairs = [(fr, int(round(1000 / dt)), 1) for fr in (24, 30, 60, 96, 100, 120, 144, 240)
             for dt in (0.0625, 0.1, 0.125, 0.25, 0.5, 1.0)]
    pairs += [(8000, 120, 0), (1000, 120, 0), (4000, 96, 0)]
    den = np.array(pairs, u32).reshape(-1)
    out["denorm_in"] = den.reshape(-1, 3)
    out["denorm_out"] = run("denorm", den, u32).reshape(-1, 2)
    # far delivery over a spike sequence: 2 blocks x 64 (48 E), ngE 2, ngI 1
    nV1, bs, nE, ngE, ngI, T = 128, 64, 48, 2, 1, 120
    nVec = rng.integers(0, 25, nV1).astype(u32)
    ids, strs, dels = [], [], []
    for i in range(nV1):
        other = np.setdiff1d(np.arange(nV1), np.arange((i // bs) * bs, (i // bs + 1) * bs))
        c = rng.choice(other, int(nVec[i]), replace=False)
        ids.append(c)
        strs.append(rng.lognormal(0, 0.5, len(c)) * np.where(c % bs < nE, 0.01, 0.04))
        dels.append(rng.uniform(0.0, 1.5, len(c)))
    vecID = np.concatenate(ids).astype(u32)
    conVec = np.concatenate(strs).astype(f32)
    delayVec = np.concatenate(dels).astype(f32)
    spk = rng.random((T, nV1)) < 0.03
    sInfo = np.where(spk, 1.0 + rng.random((T, nV1)), rng.uniform(-70, -51, (T, nV1)))
    sInfo[rng.random((T, nV1)) < 0.002] += 1.0            # a few double spikes
    sInfo = sInfo.astype(f32)
    hdr = np.array([nV1, bs, nE, ngE, ngI, T, len(vecID), 0], i32)
    prm = np.array([0.125, 1.0, 1.0, 2.0, 5.0, 80.0, 1.0, 1.0, 7.0, 7.0,
                    0.8, 0.2, 0.8, 0.2, 1.0, 1.0, 0.0, 0.0], f32)   # pE [type][ngE], pI [type][ngI]
    res = run("far", [hdr, prm, nVec, vecID, conVec, delayVec, sInfo], f32)
    out["far_hdr"], out["far_prm"] = hdr, prm
    out["far_nVec"], out["far_vecID"], out["far_conVec"], out["far_delayVec"] = nVec, vecID, conVec, delayVec
    out["far_sInfo"] = sInfo
    out["far_out"] = res.reshape(T, (ngE + ngI) * 2, nV1)
    # far delivery with synaptic failure: 3 blocks x 64 in 2 chunks (2 + 1 blocks), host engines
    nV1 = 192
    nVec = rng.integers(0, 25, nV1).astype(u32)
    ids, strs, dels = [], [], []
    for i in range(nV1):
        other = np.setdiff1d(np.arange(nV1), np.arange((i // bs) * bs, (i // bs + 1) * bs))
        c = rng.choice(other, int(nVec[i]), replace=False)
        ids.append(c)
        strs.append(rng.lognormal(0, 0.5, len(c)) * np.where(c % bs < nE, 0.01, 0.04))
        dels.append(rng.uniform(0.0, 1.5, len(c)))
    vecID = np.concatenate(ids).astype(u32)
    conVec = np.concatenate(strs).astype(f32)
    delayVec = np.concatenate(dels).astype(f32)
    spk = rng.random((T, nV1)) < 0.03
    sInfo = np.where(spk, 1.0 + rng.random((T, nV1)), rng.uniform(-70, -51, (T, nV1))).astype(f32)
    hdr = np.array([nV1, bs, nE, ngE, ngI, T, len(vecID), 2], i32)
    seed0 = np.array([987654], np.uint64)
    fail = np.array([0.2, 0.3, 0.25, 0.1, 5.0, 7.5, 4.26, 7.88], f32)    # synFail[4], synPerCon[4]
    res = run("farfail", [hdr, seed0, fail, prm, nVec, vecID, conVec, delayVec, sInfo], f32)
    out["farfail_hdr"], out["farfail_seed"], out["farfail_fail"] = hdr, seed0, fail
    out["farfail_nVec"], out["farfail_vecID"] = nVec, vecID
    out["farfail_conVec"], out["farfail_delayVec"], out["farfail_sInfo"] = conVec, delayVec, sInfo
    out["farfail_out"] = res.reshape(T, (ngE + ngI) * 2, nV1)
    # LGN->V1 learning constants: learnFF_pre/learnFF_post and exp_homeo for parameter rows
    # {tauLTP, tauLTD, tauTrip, tauAvg, targetFR, A_LGN, r_LTD, gmaxLGN, gminLGN, sRatioLGN, dt,
    # decayTimeHomeoFF}
    m = 64
    lf = np.stack([rng.uniform(5, 40, m), rng.uniform(10, 60, m), rng.uniform(50, 200, m),
                   rng.uniform(200, 3000, m), np.where(rng.random(m) < 0.3, 0.0, rng.uniform(0.5, 20, m)),
                   rng.uniform(1e-4, 5e-2, m), rng.uniform(0.2, 2, m), rng.uniform(0.1, 2, m),
                   rng.uniform(0, 0.05, m), rng.uniform(0.5, 3, m), rng.choice([0.0625, 0.1, 0.125, 0.25], m),
                   rng.uniform(50, 1000, m)], 1).astype(f32)
    out["learnff_in"] = lf
    out["learnff_out"] = run("learnff", lf, np.uint8).reshape(m, -1)
    np.savez_compressed(os.path.join(ROOT, "tests", "golden", "ref_golden.npz"), **out)
    print({k: v.shape for k, v in out.items()})


if __name__ == "__main__":
    sys.exit(main())
