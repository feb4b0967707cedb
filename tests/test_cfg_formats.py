"""Config parsing (boost::program_options rules of src/patch.cu:172-611, src/util/po.h) and
the binary input/output layouts, on the CPU."""
import os
import tempfile

import numpy as np
import pytest

from visual_cortex_gb300 import cfg, formats as FM


def test_vector_keys_append_and_split():
    c = cfg.load([], "sRatioV1 = 0.3, 0.3\nsRatioV1 = 0.9;0.3 # comment, 7\n"
                     "nTypeHierarchy = 1 1\n")
    assert c.sRatioV1 == [0.3, 0.3, 0.9, 0.3]
    assert c.nTypeHierarchy == [1, 1]
    # a leading brace leaves an empty first item, which the reference's validator rejects
    with pytest.raises(cfg.ConfigError):
        cfg.load([], "synPerCon = {5.0, 7.5}\n")
    c = cfg.load([], "synPerCon = 5.0,7.5}\n")
    assert c.synPerCon == [5.0, 7.5]


def test_scalar_twice_and_unknown_keys_are_errors():
    with pytest.raises(cfg.ConfigError, match="more than once"):
        cfg.load([], "dt = 0.125\ndt = 0.25\n")
    with pytest.raises(cfg.ConfigError, match="unrecognised"):
        cfg.load([], "notAKey = 1\n")
    with pytest.raises(cfg.ConfigError):
        cfg.load([], "nt = 1.5\n")


def test_bools_defaults_and_command_line_precedence():
    c = cfg.load(["--nt", "100", "-s", "7", "--hWrite=no"],
                 "nt = 5\nminimal = True\nrawData = off\nseed = 3\n")
    assert c.nt == 100 and c.seed == 7 and c.hWrite is False
    assert c.minimal is True and c.rawData is False
    assert c.dt == 0.0625 and c.mau == 250.0 and c.noDelay == 1 and c.useNewLGN is True
    assert c.defaulted("dt") and not c.defaulted("nt")


def test_paths_and_suffixes():
    c = cfg.load([], "inputFolder = in/\nresourceFolder = res/\noutputFolder = out/\n"
                     "conV1_suffix = v1\nres_suffix = r\noutput_suffix = o\n"
                     "fV1_vec = !/abs/vec\nfStimulus = stim.bin\n")
    p = cfg.resolve_paths(c)
    assert p.v1_vec == "/abs/vec-v1.bin"
    assert p.conMat == "in/V1_conMat-v1.bin"
    assert p.lgn_v1_id == "in/LGN_V1_idList.bin"
    assert p.lgn_vpos == "res/LGN_vpos-r.bin"
    assert p.stimulus == "res/stim.bin"
    assert p.raw == "out/rawData-o.bin"
    assert p.lgn == "out/LGN"


def test_input_formats_round_trip():
    rng = np.random.default_rng(0)
    d = tempfile.mkdtemp()
    f = lambda n: os.path.join(d, n)
    FM.write_connectome_cfg(f("cc"), 2, 1, [768, 1024])
    assert [int(x) for x in FM.read_connectome_cfg(f("cc"))[2]] == [768, 1024]
    pos = rng.uniform(0, 1, (2 * 8, 2))
    FM.write_v1_allpos(f("pos"), 2, 8, pos)
    nb, bs, pos2 = FM.read_v1_allpos(f("pos"))
    assert (nb, bs) == (2, 8) and np.array_equal(pos, pos2)
    mat = rng.uniform(0, 1, (2, 1, 8, 8)).astype(np.float32)
    FM.write_mat(f("m"), 1, mat)
    assert np.array_equal(FM.read_mat(f("m"), 2, 8)[1], mat)
    FM.write_neighbor_block(f("nb"), [1, 1], [[0, 1], [1]])
    nNear, ids = FM.read_neighbor_block(f("nb"), 2, 1)
    assert list(nNear) == [1, 1] and ids[:, 0].tolist() == [0, 1]
    nVec = np.array([2, 0, 3], np.uint32)
    vid = np.array([1, 2, 0, 1, 2], np.uint32)
    s = rng.uniform(0, 1, 5).astype(np.float32)
    dl = rng.uniform(0, 1, 5).astype(np.float32)
    FM.write_v1_vec(f("vec"), nVec, vid, s, dl)
    out = FM.read_v1_vec(f("vec"), 3)
    for a, b in zip(out, (nVec, vid, s, dl)):
        assert np.array_equal(a, b)
    lists = [np.array([3, 4], np.uint32), np.zeros(0, np.uint32), np.array([7], np.uint32)]
    FM.write_list_of_lists(f("ids"), lists, np.uint32)
    assert all(np.array_equal(a, b) for a, b in zip(FM.read_list_of_lists(f("ids"), np.uint32), lists))
    fl = [x.astype(np.float32) * 0.5 for x in lists]
    FM.write_list_of_lists(f("s"), fl, np.float32, with_max=True)
    got, mx = FM.read_list_of_lists(f("s"), np.float32, with_max=True)
    assert mx == 2 and all(np.array_equal(a, b) for a, b in zip(got, fl))
    frames = rng.uniform(0, 1, (3, 3, 4, 5)).astype(np.float32)
    FM.write_stimulus(f("st"), frames, (0.5, 0.5, 0.5), (0.2, 2.0))
    st = FM.read_stimulus(f("st"))
    assert np.array_equal(st.frames, frames) and st.range == pytest.approx(2.0) and st.neye == 1


def test_output_headers_byte_layout():
    d = tempfile.mkdtemp()
    w = FM.RawDataWriter(os.path.join(d, "raw"), 0.125, 2, 4, 1, 1, True, 2, 2, 1)
    rec = np.arange(2 * w.rec, dtype=np.float32).reshape(2, w.rec)
    w.write(rec)
    w.close()
    b = open(os.path.join(d, "raw"), "rb").read()
    assert np.frombuffer(b[:4], np.float32)[0] == np.float32(0.125)
    assert np.frombuffer(b[4:36], np.uint32).tolist() == [2, 4, 1, 1, 1, 2, 2, 1]
    # sInfo, dep, w, v, gFF[2], hFF[2], gE[2], gI, hE[2], hI = 14 rows of nV1, plus mI gap
    assert w.rec == 14 * 4 + 1
    h, data = FM.read_raw(os.path.join(d, "raw"))
    assert h["nt"] == 2 and np.array_equal(data, rec)
    s = FM.LgnSpWriter(os.path.join(d, "sp"), 0.125, 1, 3)
    s.write(np.ones((1, 3)))
    s.close()
    dt, sp = FM.read_lgn_sp(os.path.join(d, "sp"))
    assert dt == 0.125 and sp.shape == (1, 3)


def test_reference_snapshot_layout_round_trip():
    """write_reference_snapshot puts the fields in the reference's order and sizes
    (src/patch.cu:6793-6912: 11 indices, iModel, learning, 7 sizes, the LGN block
    2 nLGN floats + nLGN generators, rGenCond, rNoisy, tBack, the spike-word ring, then dep, w,
    v, gFF, hFF, gE, gI, hE, hI, gap); read_reference_snapshot reads them back and returns what
    follows them."""
    import tempfile
    from visual_cortex_gb300 import formats as FM
    rng = np.random.default_rng(0)
    n, nl, depth, ngFF, ngE, ngI, nI = 64, 16, 3, 2, 2, 1, 16
    idx = {k: int(rng.integers(0, 1000)) for k in FM.SNAPSHOT_INDICES}
    f = lambda k: rng.standard_normal(k).astype(np.float32)
    lgn = dict(ltr=f(nl), lnl=f(nl), rng=rng.integers(0, 256, 48 * nl).astype(np.uint8))
    v1 = dict(rng_cond=rng.integers(0, 256, 48 * n).astype(np.uint8),
              rng_noisy=rng.integers(0, 256, 48 * n).astype(np.uint8), tBack=f(n))
    ring = f(depth * n).reshape(depth, n)
    state = dict(dep=f(n), w=f(n), v=f(n), gFF=f(ngFF * n), hFF=f(ngFF * n), gE=f(ngE * n), gI=f(ngI * n),
                 hE=f(ngE * n), hI=f(ngI * n), gap=f(nI))
    sizes = dict(nV1=n, nLGN=nl, ngFF=ngFF, ngE=ngE, ngI=ngI, nType=2, trainDepth=depth)
    with tempfile.TemporaryDirectory() as d:
        fn = d + "/snap.bin"
        FM.write_reference_snapshot(fn, idx, 1, 0, sizes, lgn, v1, ring, state, b"TRAILER")
        size = (11 + 2 + 7) * 4 + (2 * nl * 4 + nl * 48) + 2 * n * 48 + n * 4 + depth * n * 4 + \
            (n * 3 + 2 * (ngFF + ngE + ngI) * n + nI) * 4 + len(b"TRAILER")
        import os
        assert os.path.getsize(fn) == size
        snap, trailer = FM.read_reference_snapshot(fn, nI)
    assert trailer == b"TRAILER" and snap["idx"] == idx and snap["sizes"] == sizes and snap["iModel"] == 1
    for k in state:
        np.testing.assert_array_equal(snap["state"][k], state[k])
    np.testing.assert_array_equal(snap["spike_train"], ring)
    np.testing.assert_array_equal(snap["lgn"]["rng"], lgn["rng"])
    np.testing.assert_array_equal(snap["v1"]["tBack"], v1["tBack"])
