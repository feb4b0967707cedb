"""The cfg-driven run: reference-format inputs in, reference-format outputs out."""
import tempfile

import numpy as np
import pytest

from visual_cortex_gb300 import cfg, driver, formats as FM, synth


@pytest.fixture(scope="module")
def written():
    wl = synth.make_workload("drv", seed=2, nblock=2, n_lgn=512, m=20, width=64, height=64,
                             nt=96, far_partners=50, adex_inh=True, nFrame=60)
    d = tempfile.mkdtemp()
    fn = synth.write_reference_files(wl, d, seed=2, nt=96)
    return wl, fn


def test_build_reads_back_the_workload(written):
    wl, fn = written
    m = driver.build(cfg.load(["-c", fn]))
    assert m.spec == wl.spec
    for k in ("nLGNperV1", "lgnId", "sLGN", "nNearNB", "nbId", "conMat", "nVec", "vecID",
              "conVec", "delayVec"):
        assert np.array_equal(getattr(m.net, k), getattr(wl.net, k)), k
    assert np.array_equal(m.stim.frames, wl.stim.frames)
    assert m.lgn.sched == wl.lgn.sched
    # CmoreDep tonic drive: tonicDep * (minTonicRatio + (1 - minTonicRatio) * scaled ratio)
    t = m.spec.type_of(np.arange(m.spec.nV1) % m.spec.blockSize)
    assert np.all(m.net.tonicDep[t == 0] <= np.float32(0.6) + 1e-6)
    assert np.all(m.net.tonicDep[t == 0] >= np.float32(0.3) - 1e-6)
    # trainDepth from the largest connected within-block distance
    assert m.seeds.trainDepth >= 2


def test_scaling_rules(written):
    wl, fn = written
    m = driver.build(cfg.load(["-c", fn, "--sRatioV1", "0.5,2,3,4", "--sRatioLGN", "2"]))
    bs, nE = m.spec.blockSize, m.spec.nE
    c = m.net.conMat[0, 0]
    c0 = wl.net.conMat[0, 0]
    np.testing.assert_array_equal(c[:nE, :nE], (c0[:nE, :nE] * np.float32(0.5)).astype(np.float32))
    np.testing.assert_array_equal(c[:nE, nE:], (c0[:nE, nE:] * np.float32(2)).astype(np.float32))
    np.testing.assert_array_equal(c[nE:, :nE], (c0[nE:, :nE] * np.float32(3)).astype(np.float32))
    np.testing.assert_array_equal(m.net.sLGN, (wl.net.sLGN * np.float32(2)).astype(np.float32))


def test_unsupported_keys_fail_loudly(written):
    _, fn = written
    with pytest.raises(cfg.ConfigError, match="learning"):
        driver.build(cfg.load(["-c", fn, "--learning", "1", "--learnData_FF", "2"]))
    with pytest.raises(cfg.ConfigError, match="noFarDelay"):
        driver.build(cfg.load(["-c", fn, "--noDelay", "0", "--noFarDelay", "1"]))
    m = driver.build(cfg.load(["-c", fn, "--noDelay", "0", "--noFarDelay", "0"]))
    assert m.spec.noDelay == 0 and m.net.delayMat is not None


@pytest.mark.gpu
def test_run_writes_reference_outputs(written, native):
    from visual_cortex_gb300.model import Simulation
    from visual_cortex_gb300 import _native as N
    wl, fn = written
    c = cfg.load(["-c", fn])
    m = driver.run(c, chunk=40, log=lambda *_: None)
    P = cfg.resolve_paths(c)
    h, raw = FM.read_raw(P.raw)
    assert h["nt"] == 96 and h["nV1"] == m.spec.nV1 and h["mI"] == m.spec.nI * m.spec.nblock
    dt, sp = FM.read_lgn_sp(P.lgn_sp)
    fr = FM.read_lgn_fr(P.lgn_fr)
    sim = Simulation(m.spec, m.net, m.lgn, m.stim, m.init, m.seeds)
    try:
        sim.set_record(N.REC_RAW | N.REC_LGN_SP | N.REC_LGN_FR, 97)
        sim.run(96)
        r2, sp2, fr2 = sim.fetch_records(0, 96, raw=True, lgn_sp=True, lgn_fr=True)
    finally:
        sim.close()
    np.testing.assert_array_equal(raw, r2)
    np.testing.assert_array_equal(sp, sp2)
    np.testing.assert_array_equal(fr, fr2)
    assert (raw[:, :m.spec.nV1] >= 1).sum() > 0 or (sp >= 1).sum() > 0
    b = open(P.patchV1_cfg, "rb").read()
    assert np.frombuffer(b[:4], np.uint32)[0] == 4
    assert np.frombuffer(b[4:16], np.float32).tolist() == [m.spec.vL, m.spec.vE, m.spec.vI]


def test_parvo_cells_read_back():
    """Parvo cells (LGN types 0-3 before the magno cells) go through the reference's files:
    counts, component parameters, cone types, covariant and the parvo kernel grid."""
    wl = synth.make_workload("parvo", seed=9, nblock=1, n_lgn=256, m=20, width=64, height=64, nt=48,
                             nFrame=40, n_parvo=64, tau=300.0, nKernelSample=150)
    d = tempfile.mkdtemp()
    fn = synth.write_reference_files(wl, d, seed=3, nt=48)
    m = driver.build(cfg.load(["-c", fn]))
    L, L0 = m.lgn, wl.lgn
    assert (L.nParvo_I, L.nMagno_I, L.nParvo_C, L.nMagno_C) == (64, 256, 0, 0)
    assert L.nSample1D == L0.nSample1D and L.sched == L0.sched
    assert L.sched.kernelSampleInterval == 16 and L.sched.pLongerThanM
    for k in ("polar", "ecc", "rw", "rh", "orient", "k", "tauR", "tauD", "delay", "coneType", "covariant",
              "c50", "sharpness"):
        assert np.array_equal(getattr(L, k), getattr(L0, k)), k


def test_curved_retina_reads_back():
    """flat_retina = false: a two-eye stimulus file, the curved geometry of src/patch.cu:
    1609-1622 (visual centre of the left eye at buffer / (2 extent), view distance from
    tan(max_ecc))."""
    import math
    wl = synth.make_workload("curved", seed=4, nblock=1, n_lgn=256, m=20, width=64, height=64, nt=48,
                             nFrame=40, flat_retina=False)
    d = tempfile.mkdtemp()
    fn = synth.write_reference_files(wl, d, seed=3, nt=48)
    m = driver.build(cfg.load(["-c", fn]))
    L = m.lgn
    assert not L.flat_retina and L.L_y0 == 0.5 and 0 < L.L_x0 < 0.25
    assert L.R_x0 == np.float32(0.5) + np.float32(L.L_x0)
    stim = FM.read_stimulus(cfg.resolve_paths(cfg.load(["-c", fn])).stimulus)
    ext = stim.range + 2 * stim.buffer
    max_ecc = float(np.max(np.hypot(wl.lgn.xy[:, 0], wl.lgn.xy[:, 1])))
    assert L.normViewDistance == pytest.approx((max_ecc / (2 * ext)) / math.tan(max_ecc * math.pi / 180), rel=1e-5)
    assert stim.neye == 2
    with pytest.raises(cfg.ConfigError, match="one eye"):
        driver.build(cfg.load(["-c", fn, "--flat_retina", "1"]))


def test_two_eye_parvo_reads_back():
    """Parvo and magno cells in both eyes (LGN_vpos nI / nC, cells ordered parvo_I, magno_I,
    parvo_C, magno_C): the driver splits them as the reference does."""
    wl = synth.make_workload("twoeye", seed=5, nblock=1, n_lgn=256, m=20, width=64, height=64, nt=48,
                             nFrame=40, flat_retina=False, n_parvo=32, tau=300.0, nKernelSample=150,
                             contra=True)
    d = tempfile.mkdtemp()
    fn = synth.write_reference_files(wl, d, seed=3, nt=48)
    m = driver.build(cfg.load(["-c", fn]))
    L = m.lgn
    assert (L.nParvo_I, L.nMagno_I, L.nParvo_C, L.nMagno_C) == (16, 128, 16, 128)
    np.testing.assert_array_equal(L.coneType, wl.lgn.coneType)
    np.testing.assert_allclose(L.polar, wl.lgn.polar, rtol=1e-6)


@pytest.mark.gpu
def test_snapshot_resume_continues_the_run(written, native):
    """A run of 96 steps leaves a snapshot; a second run resumed from it (fSnapshot, asInit =
    false) for 40 more steps writes the same records as one straight run of 136 steps."""
    import glob
    import os
    import shutil
    wl, fn = written
    d = os.path.dirname(fn)
    out1, out2, out3 = (os.path.join(d, x) + "/" for x in ("o1", "o2", "o3"))
    lgn = cfg.resolve_paths(cfg.load(["-c", fn])).lgn     # read from the output folder
    for o in (out1, out2, out3):
        os.makedirs(o, exist_ok=True)
        shutil.copy(lgn, o + os.path.basename(lgn))
    driver.run(cfg.load(["-c", fn, "--outputFolder", out1, "--output_suffix", "s"]), chunk=40, log=lambda *_: None)
    snaps = glob.glob(out1 + "snapShot_*_s.bin")
    assert len(snaps) == 1      # the earlier ones of the run were removed (delPrevSnapshot)
    name = os.path.basename(snaps[0])[:-len("_s.bin")]
    c2 = cfg.load(["-c", fn, "--outputFolder", out2, "--output_suffix", "s", "--nt", "40",
                   "--fSnapshot", "!" + out1 + name, "--snapshot_suffix", "s", "--asInit", "false"])
    driver.run(c2, chunk=40, log=lambda *_: None)
    driver.run(cfg.load(["-c", fn, "--outputFolder", out3, "--output_suffix", "s", "--nt", "136"]), chunk=40,
               log=lambda *_: None)
    _, r2 = FM.read_raw(cfg.resolve_paths(c2).raw)
    _, r3 = FM.read_raw(cfg.resolve_paths(cfg.load(["-c", fn, "--outputFolder", out3, "--output_suffix", "s"])).raw)
    np.testing.assert_array_equal(r2, r3[96:])


@pytest.mark.gpu
def test_reference_layout_snapshot(native):
    """Snapshots in the reference's layout (src/patch.cu:6793-6912): the indices, sizes and the
    newest slot of the spike-word ring are where the reference writes them; a snapshot cut to
    the reference's own fields (as the reference writes it) resumes a run without far synapses
    bit for bit (src/patch.cu:5489-5685, asInit = false), and with asInit = true it is the
    initial state of a new run at step 0."""
    import glob
    import os
    from visual_cortex_gb300.model import Simulation
    wl = synth.make_workload("snap", seed=4, nblock=1, n_lgn=512, m=20, width=64, height=64, nt=64,
                             adex_inh=True, nFrame=40)
    d = tempfile.mkdtemp()
    fn = synth.write_reference_files(wl, d, seed=4, nt=64)
    outs = [os.path.join(d, x) + "/" for x in ("a", "b", "c")]
    lgn = cfg.resolve_paths(cfg.load(["-c", fn])).lgn
    import shutil
    for o in outs:
        os.makedirs(o, exist_ok=True)
        shutil.copy(lgn, o + os.path.basename(lgn))
    quiet = dict(chunk=16, log=lambda *_: None)
    driver.run(cfg.load(["-c", fn, "--outputFolder", outs[0], "--output_suffix", "s", "--nt", "32"]), **quiet)
    snap_fn = glob.glob(outs[0] + "snapShot_*_s.bin")[0]
    m = driver.build(cfg.load(["-c", fn]))
    snap, trailer = FM.read_reference_snapshot(snap_fn, m.spec.nI * m.spec.nblock)
    assert trailer[:8] == b"PV1CKPT\0"
    depth = int(m.seeds.trainDepth)
    assert snap["idx"]["step"] == 32 and snap["idx"]["currentTimeSlot"] == 32 % depth
    assert snap["sizes"]["nV1"] == m.spec.nV1 and snap["sizes"]["trainDepth"] == depth
    _, raw = FM.read_raw(cfg.resolve_paths(cfg.load(["-c", fn, "--outputFolder", outs[0], "--output_suffix", "s"])).raw)
    np.testing.assert_array_equal(snap["spike_train"][31 % depth], raw[31, :m.spec.nV1])
    # the reference's own fields only
    ref_only = outs[0] + "refsnap_s.bin"
    with open(snap_fn, "rb") as f:
        data = f.read()
    with open(ref_only, "wb") as f:
        f.write(data[:len(data) - len(trailer)])
    c2 = cfg.load(["-c", fn, "--outputFolder", outs[1], "--output_suffix", "s", "--nt", "32",
                   "--fSnapshot", "!" + outs[0] + "refsnap", "--snapshot_suffix", "s", "--asInit", "false"])
    driver.run(c2, **quiet)
    driver.run(cfg.load(["-c", fn, "--outputFolder", outs[2], "--output_suffix", "s", "--nt", "64"]), **quiet)
    _, r2 = FM.read_raw(cfg.resolve_paths(c2).raw)
    _, r3 = FM.read_raw(cfg.resolve_paths(cfg.load(["-c", fn, "--outputFolder", outs[2], "--output_suffix", "s"])).raw)
    np.testing.assert_array_equal(r2, r3[32:])
    # asInit = true: the snapshot's state at step 0
    c4 = cfg.load(["-c", fn, "--fSnapshot", "!" + outs[0] + "refsnap", "--snapshot_suffix", "s", "--asInit", "true"])
    m4 = driver.build(c4)
    sim = Simulation(m4.spec, m4.net, m4.lgn, m4.stim, m4.init, m4.seeds)
    try:
        assert driver._restore(sim, c4, m4) == 0 and sim.step == 0
        for k in ("v", "gE", "gI", "gFF", "hFF"):
            np.testing.assert_array_equal(sim.state(k), snap["state"][k], err_msg=k)
        np.testing.assert_array_equal(sim.state("tBack"), snap["v1"]["tBack"])
        np.testing.assert_array_equal(sim.state("v1_rng_cond"), snap["v1"]["rng_cond"])
        np.testing.assert_array_equal(sim.state("lgn_rng"), snap["lgn"]["rng"])
        sim.run(16)
        assert np.isfinite(sim.state("v")).all()
    finally:
        sim.close()


def test_frame_geometry_and_pixels():
    """getUnderlyingID's pixel lists: every neuron in exactly one pixel, in neuron order, the
    far edge folded into the last pixel."""
    x = np.array([0.0, 1.0, 0.5, 0.26, 0.24, 1.0])
    y = np.array([0.0, 1.0, 0.5, 0.0, 0.99, 0.0])
    off, ids = FM.underlying_ids(x, y, 4, 2, 0.0, 1.0, 0.0, 1.0)
    assert off[-1] == 6 and len(off) == 9
    cells = {q: list(ids[off[q]:off[q + 1]]) for q in range(8) if off[q + 1] > off[q]}
    assert cells == {0: [0], 1: [3], 3: [5], 4: [4], 6: [2], 7: [1]}


@pytest.mark.gpu
@pytest.mark.parametrize("features", [False, True])
def test_frames_match_the_raster(native, features):
    """framePhyV1output + frameVisV1output + frameVisLGNoutput: the outputFrame of a driver run
    equals pixelizeOutput's sums recomputed on the host from the run's own rawData spike words
    and LGN_fr rates, pixel lists from getUnderlyingID.  With a V1 feature file (readFeature
    forced on by nOri, iOri and boostOri), the visual-field V1 frames split the neurons by the
    sign of their ocular dominance (src/patch.cu:3157-3170)."""
    import os
    wl = synth.make_workload("frames", seed=12, nblock=2, n_lgn=512, m=20, width=64, height=64,
                             nt=96, far_partners=50, adex_inh=True, nFrame=60)
    d = tempfile.mkdtemp() + "/"
    fn = synth.write_reference_files(wl, d, seed=2, nt=96, v1_visual=True)
    extra = []
    od = None
    if features:
        c0 = cfg.load(["-c", fn])
        rng = np.random.default_rng(5)
        feat = np.stack([rng.uniform(-1, 1, wl.spec.nV1), rng.uniform(0, 1, wl.spec.nV1)]).astype(np.float32)
        FM.write_v1_feature(cfg._prefixed(c0.resourceFolder, c0.fV1_feature) + cfg._suffix(c0.res_suffix), feat)
        od = feat[0]
        # boost (1, 0) leaves the drive unchanged; nOri with iOri forces readFeature on
        extra = ["--nOri", "6", "--iOri", "2", "--boostOri", "1.0", "--boostOri", "0.0"]
    c = cfg.load(["-c", fn, "--framePhyV1output", "true", "--frameVisV1output", "true",
                  "--frameVisLGNoutput", "true", "--dot", "1.0", "--phyWidth_scale", "0.25",
                  "--visWidth_scale", "0.25", "--saveLGN_fr", "true"] + extra)
    m = driver.run(c, chunk=40, log=lambda *_: None)
    P = cfg.resolve_paths(c)
    _, raw = FM.read_raw(P.raw)
    fr = FM.read_lgn_fr(P.lgn_fr)
    with open(os.path.join(c.outputFolder or os.path.dirname(P.raw), "outputFrame.bin"), "rb") as f:
        dt = np.fromfile(f, np.float32, 1)[0]
        ot, kinds = np.fromfile(f, np.uint32, 2)
        (pw, ph), (vw, vh), (lw, lh) = np.fromfile(f, np.uint32, 6).reshape(3, 2)
        frames = np.fromfile(f, np.float32)
    assert kinds == 7 and ot == 8 and dt == np.float32(c.dt) and (vw, vh) == (lw, lh)
    npix = pw * ph + 2 * vw * vh + 2 * lw * lh
    frames = frames.reshape(-1, npix)
    x0, xs, y0, ys = FM.read_v1_allpos_spans(P.v1_allpos)
    _, _, pos = FM.read_v1_allpos(P.v1_allpos)
    vx0, vxs, vy0, vys, vx, vy = FM.read_v1_allpos_visual(P.v1_allpos)
    lx0, lxs, ly0, lys = FM.read_lgn_vpos_spans(P.lgn_vpos)
    nI, nC, _, lx, ly, _ = FM.read_lgn_vpos(P.lgn_vpos)
    if od is None:
        vis = [FM.underlying_ids(vx, vy, int(vw), int(vh), vx0, vxs, vy0, vys),
               (np.zeros(vw * vh + 1, np.uint32), np.zeros(0, np.uint32))]
    else:
        ipsi = od < 0
        vis = [FM.underlying_ids(vx, vy, int(vw), int(vh), vx0, vxs, vy0, vys, pick=ipsi),
               FM.underlying_ids(vx, vy, int(vw), int(vh), vx0, vxs, vy0, vys, pick=~ipsi)]
        assert len(vis[0][1]) > 0 and len(vis[1][1]) > 0
    groups = [(FM.underlying_ids(pos[:, 0], pos[:, 1], int(pw), int(ph), x0, xs, y0, ys), True),
              (vis[0], True), (vis[1], True),
              (FM.underlying_ids(lx[:nI], ly[:nI], int(lw), int(lh), lx0, lxs, ly0, lys, dtype=np.float32), False),
              (FM.underlying_ids(lx[nI:], ly[nI:], int(lw), int(lh), lx0, lxs, ly0, lys, dtype=np.float32, n0=nI),
               False)]
    odt = np.float32(float(np.float32(np.float32(ot) * np.float32(c.dt))) / 1000.0)
    sI = raw[:, :m.spec.nV1]
    want, acc = [], np.zeros(npix, np.float32)
    for t in range(sI.shape[0]):
        if t % ot == 0:
            acc[:] = 0
        q0 = 0
        for (off, ids), spike in groups:
            src = sI[t] if spike else fr[t]
            for q in range(len(off) - 1):
                mq = int(off[q + 1] - off[q])
                if mq:
                    v = np.float32(0)
                    for j in ids[off[q]:off[q + 1]]:
                        if src[j] >= 0:
                            v = np.float32(v + (np.floor(src[j]) if spike else src[j]))
                    acc[q0 + q] = np.float32(acc[q0 + q] + np.float32(v / np.float32(np.float32(mq) * odt)))
            q0 += len(off) - 1
        if (t + 1) % ot == 0:
            want.append(acc.copy())
    np.testing.assert_array_equal(frames, np.array(want))
    for a, b in ((0, pw * ph), (pw * ph, pw * ph + vw * vh), (npix - 2 * lw * lh, npix)):
        assert frames[:, a:b].sum() > 0


@pytest.mark.gpu
def test_minimal_sample_file(written, native):
    """minimal = true writes only the sample file; its LGN rows and sample spike counts equal
    those of a full run of the same cfg (sample_t0 = 2 ms skips the first 15 steps' rows)."""
    import os
    import shutil
    wl, fn = written
    d = os.path.join(os.path.dirname(fn), "minimal") + "/"
    os.makedirs(d, exist_ok=True)
    lgn = cfg.resolve_paths(cfg.load(["-c", fn])).lgn
    shutil.copy(lgn, d + os.path.basename(lgn))
    full = cfg.load(["-c", fn, "--getLGN_sp", "true"])
    driver.run(full, chunk=40, log=lambda *_: None)
    P = cfg.resolve_paths(full)
    _, raw = FM.read_raw(P.raw)
    _, sp = FM.read_lgn_sp(P.lgn_sp)
    c = cfg.load(["-c", fn, "--outputFolder", d, "--minimal", "true", "--sampleSize", "300",
                  "--sample_t0", "2.0"])
    m = driver.run(c, chunk=40, log=lambda *_: None)
    assert not os.path.exists(d + "rawData.bin")
    with open(d + "sample_spikeCount.bin", "rb") as f:
        k = int(np.fromfile(f, np.uint32, 1)[0])
        t0, t1 = np.fromfile(f, np.float32, 2)
        nt, nLGN = (int(v) for v in np.fromfile(f, np.uint32, 2))
        rest = np.fromfile(f, np.uint8)
    assert k == 300 and t0 == np.float32(2.0) and nt == 96 and nLGN == sp.shape[1]
    steps = [s for s in range(nt) if s == nt - 1 or np.float32(np.float32(s + 1) * np.float32(c.dt)) >= t0]
    rows = rest[:len(steps) * nLGN * 4].view(np.float32).reshape(len(steps), nLGN)
    ids = rest[len(steps) * nLGN * 4:len(steps) * nLGN * 4 + 4 * k].view(np.uint32)
    counts = rest[len(steps) * nLGN * 4 + 4 * k:].view(np.uint32)
    assert len(steps) == nt - 15
    np.testing.assert_array_equal(rows, sp[steps])
    sI = raw[steps][:, ids]
    np.testing.assert_array_equal(counts, np.where(sI >= 1, np.floor(sI), 0).sum(axis=0).astype(np.uint32))
    assert (ids % m.spec.blockSize < m.spec.typeAcc[m.spec.nTypeE - 1]).all() and counts.sum() > 0


def test_orientation_boost_of_the_tonic_drive():
    """nOri > 0 with readFeature: the tonic drive scaled by the von Mises boost of each neuron's
    preferred orientation (V1_feature) around (iOri % nOri)/nOri + 1/2; boostOri = 1, 0 (the
    reference's minimal*.cfg) leaves it exactly as without nOri."""
    import math
    wl = synth.make_workload("ori", seed=6, nblock=1, n_lgn=256, m=20, width=64, height=64, nt=48, nFrame=40)
    d = tempfile.mkdtemp()
    fn = synth.write_reference_files(wl, d, seed=3, nt=48)
    c0 = cfg.load(["-c", fn])
    n = wl.spec.nV1
    rng = np.random.default_rng(0)
    feat = np.stack([rng.uniform(-1, 1, n), rng.uniform(0, 1, n)]).astype(np.float32)
    FM.write_v1_feature(cfg._prefixed(c0.resourceFolder, c0.fV1_feature) + cfg._suffix(c0.res_suffix), feat)
    base = driver.build(c0).net.tonicDep
    flat = driver.build(cfg.load(["-c", fn, "--nOri", "6", "--iOri", "2", "--boostOri", "1.0",
                                  "--boostOri", "0.0"])).net.tonicDep
    np.testing.assert_array_equal(flat, base)
    m = driver.build(cfg.load(["-c", fn, "--nOri", "6", "--iOri", "2", "--boostOri", "0.5", "--boostOri", "2.0"]))
    r = m.net.tonicDep.astype(np.float64) / base
    fOri = math.fmod(2 / 6 + 0.5, 1.0)
    dd = feat[1].astype(np.float64) - fOri
    dd = np.where(dd > 0.5, 1 - dd, np.where(dd < -0.5, 1 + dd, dd))
    A = 1 - math.exp(-4.0)
    want = 0.5 + 0.5 * (np.exp(2.0 * (np.cos(2 * math.pi * dd) - 1)) - 1 + A) / A
    np.testing.assert_allclose(r, want, rtol=2e-6, atol=2e-7)
    assert r.max() <= 1.0 + 1e-6 and r.min() >= 0.5 - 1e-6
    assert m.extra["feature"] is not None


def test_read_feature_rules():
    """readFeature as the reference resolves it (src/patch.cu:2842-2930): forced on by iOri or
    boostOri when nOri > 0 (so readFeature = false still gets the boost), and once on, the
    feature file is read and nOri > 0, iOri and boostOri are required (the reference asserts
    them)."""
    wl = synth.make_workload("ori", seed=6, nblock=1, n_lgn=256, m=20, width=64, height=64, nt=48, nFrame=40)
    d = tempfile.mkdtemp()
    fn = synth.write_reference_files(wl, d, seed=3, nt=48)
    c0 = cfg.load(["-c", fn])
    n = wl.spec.nV1
    rng = np.random.default_rng(1)
    feat = np.stack([rng.uniform(-1, 1, n), rng.uniform(0, 1, n)]).astype(np.float32)
    FM.write_v1_feature(cfg._prefixed(c0.resourceFolder, c0.fV1_feature) + cfg._suffix(c0.res_suffix), feat)
    ori = ["--nOri", "6", "--iOri", "2", "--boostOri", "0.5", "--boostOri", "2.0"]
    on = driver.build(cfg.load(["-c", fn, "--readFeature", "true"] + ori))
    forced = driver.build(cfg.load(["-c", fn, "--readFeature", "false"] + ori))
    np.testing.assert_array_equal(forced.net.tonicDep, on.net.tonicDep)
    np.testing.assert_array_equal(forced.extra["feature"], feat)
    assert driver.build(c0).extra["feature"] is None          # readFeature = false, no nOri
    for bad in (["--readFeature", "true"],                          # nOri = 0
                ["--nOri", "6", "--iOri", "2"],                      # no boostOri
                ["--nOri", "6", "--boostOri", "0.5", "--boostOri", "0.0"],   # no iOri
                ["--nOri", "6", "--iOri", "2", "--boostOri", "0.5", "--boostOri", "0.1",
                 "--boostOri", "0.2"]):                               # 3 values
        with pytest.raises(cfg.ConfigError):
            driver.build(cfg.load(["-c", fn] + bad))


LEARN_CFG = dict(tauLTP=[16.8], tauLTD=[33.7], tauTrip=[114.0], tauAvg=[1000.0, 800.0], targetFR=[2.0, 5.0],
                 A_LGN=[0.02, 0.015], r_LTD=[1.0], gmaxLGN=[0.6, 0.8], gminLGN=[0.0], applyHomeo=1,
                 FF_InfRatio=0.95, sampleInterval_LGN_V1=32, store_dsLGN=True, gmaxE=[1.0], gminE=[0.0], A_V1=[0.01])


def _learn_cfg(tmp, learning, **kw):
    wl = synth.make_workload("learnc", seed=3, nblock=1, n_lgn=256, m=10, width=32, height=32, nt=8,
                             adex_inh=True, nFrame=8)
    # the reference refuses more gmaxLGN values than FF types
    extra = dict(LEARN_CFG, learning=learning, gmaxLGN=[0.6, 0.8] if learning == 2 else [0.6])
    extra.update(kw)
    fn = synth.write_reference_files(wl, tmp, seed=3, nt=8, extra=extra)
    return cfg.load(["-c", fn])


def test_learning_modes_from_the_cfg(tmp_path):
    """The cfg rules of src/patch.cu:1092-1330 for learning 1-4: the mode's overrides of the
    type counts, the FF->I type from element [nLearnTypeFF_E] with tauAvg[1], targetFR[1] and
    sRatioLGN[1], the delivery's filtered-rate time constant tauAvg[0] while cortical E types
    exist, and the reference's refusals."""
    c = _learn_cfg(str(tmp_path / "a"), 2)
    m = driver.build(c)
    sr = m.extra["sRatioLGN"]
    L = driver._ff_learning(c, sr)
    assert (L.learning, L.nLearnTypeFF_E, L.nLearnTypeFF_I) == (2, 1, 1)
    assert L.A_LGN == 0.02 and L.A_LGN_I == 0.015 and L.gmaxLGN_I == 0.8 and L.gminLGN_I == 0.0
    assert L.tauAvg == 1000.0 and L.tauAvg_I == 800.0 and L.targetFR_I == 5.0 and L.sRatioLGN_I == float(sr[1])
    assert L.tauLTP_I == 16.8 and L.tauAvgCortical == 1000.0
    assert driver._learn_types(c) == (1, 1, 1)
    assert len(driver._ltd_ratio(L, 1, 1)) == 2
    c1 = _learn_cfg(str(tmp_path / "b"), 1)
    L1 = driver._ff_learning(c1, sr)
    assert L1.nLearnTypeFF_I == 0 and L1.tauAvgCortical == 1000.0
    c1e = _learn_cfg(str(tmp_path / "b2"), 1, nLearnTypeE=0)
    assert driver._ff_learning(c1e, sr).tauAvgCortical == 0.0
    c3 = _learn_cfg(str(tmp_path / "c"), 3)
    L3 = driver._ff_learning(c3, sr)
    assert L3.nLearnTypeFF_I == 0 and L3.tauAvgCortical == 0.0
    c4 = _learn_cfg(str(tmp_path / "d"), 4)
    assert driver._learn_types(c4) == (0, 0, 1)
    assert driver._ff_learning(c4, sr).tauAvgCortical == 1000.0
    # the reference's refusals
    for kw in (dict(tauAvg=[1.0, 2.0, 3.0]), dict(gmaxLGN=[0.6, 0.7, 0.8]), dict(tauLTD=[1.0, 2.0]),
               dict(A_LGN=[0.02]), dict(gmaxE=[])):
        with pytest.raises(cfg.ConfigError):
            driver._ff_learning(_learn_cfg(str(tmp_path / "e"), 2, **kw), sr)
    with pytest.raises(cfg.ConfigError):
        driver.build(_learn_cfg(str(tmp_path / "f"), 2, nLearnTypeFF_I=2))
    with pytest.raises(cfg.ConfigError):
        driver.build(_learn_cfg(str(tmp_path / "g"), 5))


@pytest.mark.gpu
@pytest.mark.parametrize("learning", [3, 2])
def test_learning_outputs_and_snapshot(native, learning):
    """learning 3 and 2 from a cfg: the sLGN file holds the header of src/patch.cu:4767-4776
    and the weights after every sampleInterval_LGN_V1 steps (equal to the weights of a
    Simulation run with the same FFLearning); the snapshot carries the weights and learning
    variables where the reference puts them (src/patch.cu:6844-6850); a run resumed from the
    snapshot cut to the reference's fields continues the weights and the records bit for bit."""
    import glob
    import os
    import shutil
    from visual_cortex_gb300 import _native as N
    from visual_cortex_gb300.model import Simulation
    wl = synth.make_workload("learn", seed=6, nblock=1, n_lgn=512, m=20, width=64, height=64, nt=96,
                             adex_inh=True, nFrame=40)
    d = tempfile.mkdtemp()
    nFI = 1 if learning == 2 else 0
    extra = dict(LEARN_CFG, learning=learning, gmaxLGN=[0.6, 0.8][:1 + nFI])
    fn = synth.write_reference_files(wl, d, seed=6, nt=96, extra=extra)
    outs = [os.path.join(d, x) + "/" for x in ("a", "b", "c")]
    lgn = cfg.resolve_paths(cfg.load(["-c", fn])).lgn
    for o in outs:
        os.makedirs(o, exist_ok=True)
        shutil.copy(lgn, o + os.path.basename(lgn))
    quiet = dict(chunk=16, log=lambda *_: None)
    ca = cfg.load(["-c", fn, "--outputFolder", outs[0], "--output_suffix", "s", "--nt", "64"])
    driver.run(ca, **quiet)
    h, W = FM.read_slgn(cfg.resolve_paths(ca).slgn)
    assert h["nt"] == 64 and h["interval"] == 32 and h["maxLGN"] == wl.net.maxLGN and W.shape[0] == 2
    assert abs(h["FF_InfRatio"] - 0.95) < 1e-7 and h["nLearnTypeFF_E"] == 1 and h["nLearnTypeFF_I"] == nFI
    np.testing.assert_array_equal(h["gmaxLGN"], np.float32([0.6, 0.8][:1 + nFI]))
    m = driver.build(ca)
    sim = Simulation(m.spec, m.net, m.lgn, m.stim, m.init, m.seeds)
    try:
        sim.set_ff_learning(driver._ff_learning(ca, m.extra["sRatioLGN"]))
        sim.run(32)
        np.testing.assert_array_equal(sim.state("sLGN").reshape(W[0].shape), W[0])
        sim.run(32)
        np.testing.assert_array_equal(sim.state("sLGN").reshape(W[1].shape), W[1])
        assert np.abs(W[1] - m.net.sLGN).max() > 1e-4
    finally:
        sim.close()
    snap_fn = glob.glob(outs[0] + "snapShot_*_s.bin")[0]
    snap, trailer = FM.read_reference_snapshot(snap_fn, m.spec.nI * m.spec.nblock, maxLGN=m.net.maxLGN,
                                               nE_total=m.spec.nE * m.spec.nblock, nFF_I=nFI)
    assert snap["learning"] == learning
    assert snap["learn"]["ff_pre"].size == (1 + nFI) * m.lgn.nLGN
    np.testing.assert_array_equal(snap["learn"]["sLGN"].reshape(W[1].shape), W[1])
    # resumed from the reference's fields only
    ref_only = outs[0] + "refsnap_s.bin"
    with open(snap_fn, "rb") as f:
        data = f.read()
    with open(ref_only, "wb") as f:
        f.write(data[:len(data) - len(trailer)])
    cb = cfg.load(["-c", fn, "--outputFolder", outs[1], "--output_suffix", "s", "--nt", "32",
                   "--fSnapshot", "!" + outs[0] + "refsnap", "--snapshot_suffix", "s", "--asInit", "false"])
    driver.run(cb, **quiet)
    cc = cfg.load(["-c", fn, "--outputFolder", outs[2], "--output_suffix", "s", "--nt", "96"])
    driver.run(cc, **quiet)
    _, rb = FM.read_raw(cfg.resolve_paths(cb).raw)
    _, rc = FM.read_raw(cfg.resolve_paths(cc).raw)
    assert rb.shape[0] == 32
    # the homeostasis totals restart from the connectome's weights, as in the reference, so the
    # records agree only while the totals have not moved the weights apart: compare the spikes
    # of the first resumed step and the weights' closeness at the end
    np.testing.assert_array_equal(rb[0, :m.spec.nV1], rc[64, :m.spec.nV1])
    _, Wb = FM.read_slgn(cfg.resolve_paths(cb).slgn)
    _, Wc = FM.read_slgn(cfg.resolve_paths(cc).slgn)
    assert np.abs(Wb[-1] - Wc[-1]).max() < 0.05 * Wc[-1].max()
