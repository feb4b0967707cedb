"""The outer boundary against the reference's own artefacts (CPU).

* The rawData and LGN_sp files this build writes (the driver's writers in formats.py) are read
  back with the reference's own readers -- readSpike (src/readPatchOutput.py:291-354) and
  readLGN_sp (:195-229), imported from the reference checkout with its plotting dependency
  stubbed -- and yield the spike times the records hold, multi-spike steps included.
* Every config file the reference ships (src/*.cfg) goes through this build's option parser:
  it is accepted, or rejected for the reason the reference's own parser would reject it (an
  option its table does not declare -- boost's parse_config_file at src/patch.cu:394 allows
  no unregistered option -- or a value that does not convert to the declared type).

The reference checkout is taken from REFERENCE_SRC, else from the folder `reference/src`
beside this repository; without it these tests are skipped.
"""
import importlib.util
import os
import re
import sys
import tempfile
import types
from pathlib import Path

import numpy as np
import pytest

from visual_cortex_gb300 import cfg
from visual_cortex_gb300 import formats as FM

ROOT = Path(__file__).resolve().parents[1]


def _reference_src():
    cand = [os.environ.get("REFERENCE_SRC"), str(ROOT.parent / "reference" / "src")]
    for c in cand:
        if c and (Path(c) / "patch.cu").exists():
            return Path(c)
    return None


REF = _reference_src()
pytestmark = pytest.mark.skipif(REF is None, reason="the reference checkout is not available")


@pytest.fixture(scope="module")
def reader():
    """src/readPatchOutput.py as a module; matplotlib (not installed here, used only by its
    plotting functions) is stubbed, and numpy's error state is restored after the import."""
    stubs = {}
    for name in ("matplotlib", "matplotlib.pyplot", "matplotlib.colors"):
        if name not in sys.modules:
            stubs[name] = sys.modules[name] = types.ModuleType(name)
    sys.modules["matplotlib"].pyplot = sys.modules["matplotlib.pyplot"]
    sys.modules["matplotlib"].colors = sys.modules["matplotlib.colors"]
    old = np.geterr()
    try:
        spec = importlib.util.spec_from_file_location("ref_readPatchOutput", REF / "readPatchOutput.py")
        mod = importlib.util.module_from_spec(spec)
        spec.loader.exec_module(mod)
    finally:
        np.seterr(**old)
        for name in stubs:
            del sys.modules[name]
    return mod


def _records(rng, nt, nV1, iModel, ngFF, ngE, ngI, hWrite, vThres):
    """Spike words (nsp + tsp/dt, some steps with two or three spikes) or sub-threshold v,
    and the rest of a rawData record filled with plausible values."""
    rec = nV1 * (3 + (iModel == 1) + (ngFF + ngE + ngI) * (1 + hWrite))
    out = rng.uniform(0.0, 0.5, (nt, rec)).astype(np.float32)
    s = rng.uniform(-70.0, vThres - 1.0, (nt, nV1)).astype(np.float32)
    fire = rng.random((nt, nV1)) < 0.08
    nsp = np.where(rng.random((nt, nV1)) < 0.15, rng.integers(2, 4, (nt, nV1)), 1)
    s[fire] = (nsp[fire] + rng.uniform(0.02, 0.98, fire.sum())).astype(np.float32)
    out[:, :nV1] = s
    return out, s


def _expected_times(words, dt):
    """The spike times the reference's reader assigns (several spikes of a step spread
    around the mean time, src/readPatchOutput.py:316-331)."""
    n = words.shape[1]
    out = [[] for _ in range(n)]
    for it in range(words.shape[0]):
        for j in np.nonzero(words[it] >= 1)[0]:
            w = words[it, j]
            k = int(np.floor(w))
            tsp = w - k
            if k > 1:
                d = tsp / k if 1 - tsp > 0.5 else (1 - tsp) / k
                t0 = tsp - (k // 2) * d
                out[j].extend([(it + t0 + q * d) * dt for q in range(k)])
            else:
                out[j].append((it + tsp) * dt)
    return out


@pytest.mark.parametrize("iModel,hWrite", [(1, 1), (0, 0)])
def test_raw_data_read_by_reference_reader(reader, iModel, hWrite):
    rng = np.random.default_rng(3 + iModel)
    nt, nV1, dt, vThres = 40, 96, 0.125, -50.0
    ngFF, ngE, ngI = 2, 2, 1
    recs, words = _records(rng, nt, nV1, iModel, ngFF, ngE, ngI, hWrite, vThres)
    with tempfile.TemporaryDirectory() as d:
        fn = os.path.join(d, "rawData.bin")
        w = FM.RawDataWriter(fn, dt, nt, nV1, iModel, 0, hWrite, ngFF, ngE, ngI)
        w.write(recs)
        w.close()
        sp = reader.readSpike(fn, os.path.join(d, "sp.npz"), "f4", 4, np.array([vThres]))
    want = _expected_times(words, np.float32(dt))
    assert sum(len(x) for x in want) > 200
    for j in range(nV1):
        np.testing.assert_allclose(sp[j], np.asarray(want[j], np.float32), rtol=0, atol=1e-5)


def test_lgn_sp_read_by_reference_reader(reader):
    rng = np.random.default_rng(9)
    nt, nLGN, dt = 50, 80, 0.125
    words = np.zeros((nt, nLGN), np.float32)
    fire = rng.random((nt, nLGN)) < 0.1
    nsp = np.where(rng.random((nt, nLGN)) < 0.2, rng.integers(2, 4, (nt, nLGN)), 1)
    words[fire] = (nsp[fire] + rng.uniform(0.02, 0.98, fire.sum())).astype(np.float32)
    with tempfile.TemporaryDirectory() as d:
        fn = os.path.join(d, "LGN_sp.bin")
        w = FM.LgnSpWriter(fn, dt, nt, nLGN)
        w.write(words)
        w.close()
        sp = reader.readLGN_sp(fn)
    # readLGN_sp spreads several spikes around the mean time with nsp/2 (not nsp//2)
    for j in range(nLGN):
        want = []
        for it in np.nonzero(words[:, j] >= 1)[0]:
            k = int(np.floor(words[it, j]))
            tsp = words[it, j] - k
            if k > 1:
                dd = tsp / k if 1 - tsp > 0.5 else (1 - tsp) / k
                t0 = tsp - (k / 2) * dd
                want.extend([(it + t0 + q * dd) * np.float32(dt) for q in range(k)])
            else:
                want.append((it + tsp) * np.float32(dt))
        np.testing.assert_allclose(sp[j], np.asarray(want, np.float32), rtol=0, atol=1e-5)


def _declared_options(patch_src: str) -> dict:
    """Option name -> declared value type in the reference's option table."""
    return {m.group(1): m.group(2) for m in
            re.finditer(r'\(\s*"([A-Za-z_0-9]+)"\s*,\s*po::value<\s*([^>]+?)\s*>', patch_src)}


def test_reference_config_files_parse():
    declared = _declared_options((REF / "patch.cu").read_text(errors="replace"))
    files = sorted(REF.glob("*.cfg"))
    assert len(files) >= 50
    accepted = 0
    for fn in files:
        try:
            cfg.load(["-c", str(fn)])
            accepted += 1
        except cfg.ConfigError as e:
            msg = str(e)
            m = re.search(r"unrecognised option '([^']+)'", msg)
            if m:
                assert m.group(1) not in declared, (fn.name, msg)
                continue
            m = re.search(r"invalid value '([^']*)' for option '([^']+)'", msg)
            assert m, (fn.name, msg)
            kind = declared.get(m.group(2), "")
            assert re.search(r"int|Size|Float|float|PosInt|bool|unsigned|vector", kind), (fn.name, msg, kind)
    assert accepted >= 38, accepted
