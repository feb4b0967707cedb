"""The patchV1 option table and its parsing rules (the drop-in's outer boundary).

The reference reads its keys with boost::program_options (src/patch.cu:172-405); this module
accepts the same keys, defaults and value syntax:

* a config file holds ``key = value`` lines; ``#`` starts a comment; surrounding white space
  is dropped; an unknown key is an error;
* a vector-valued key may appear several times and every occurrence appends; its values are
  split on ``;``, ``,``, ``{``, ``}`` or white space (src/util/po.h:25), an empty item is an
  error;
* a scalar key given twice in one source is an error ("multiple occurrences");
* the command line is stored first, so a key given there wins over the config file as a whole;
* booleans accept true/false, yes/no, on/off, 1/0 in any case;
* file names get their folder prefix unless they start with ``!`` (src/patch.cu:407-550),
  and the suffix rules of src/patch.cu:561-580 (``-<suffix>.bin``).
"""
from __future__ import annotations

import re
from dataclasses import dataclass, field

F, U, I, B, S = "float", "size", "int", "bool", "string"
VF, VU = "vfloat", "vsize"

# (key, kind, default); None = no default (the key is absent unless given)
OPTIONS = [
    ("seed", "ulong", None), ("cfg_file", S, "patchV1.cfg"), ("print", B, False),
    ("dt", F, 0.0625), ("nChunk", U, 10), ("matConcurrency", U, 10), ("speedOfThought", F, 1.0),
    ("nt", U, 8000), ("fbROI", VF, None), ("boostOri", VF, None), ("iOri", VU, None),
    ("nOri", U, 0), ("nFBperColumn", VU, None), ("fbSamplingRate", VF, None),
    ("fbEI_ratio", VF, None), ("fbFR", VF, None), ("snapshotInterval", U, 10000),
    ("nsig", F, 3.0), ("gauss_wv", F, 1.0), ("nSpatialSample1D", U, 32),
    ("mSpatialSample1D", U, 32), ("phyWidth_scale", F, 1.0), ("visWidth_scale", F, 1.0),
    ("tau", F, 250.0), ("mau", F, 250.0), ("Itau", F, 300.0), ("sRatioLGN", VF, None),
    ("sRatioV1", VF, None), ("synPerConFF", VF, None), ("synPerCon", VF, None),
    ("gapRatio", VF, None), ("convolRatio", F, 1.0), ("frRatioLGN", F, 1.0),
    ("spontPercent", F, 0.1), ("nKernelSample", U, 500), ("mKernelSample", U, 500),
    ("frameRate", U, 120), ("riseTimeFF", VF, None), ("riseTimeE", VF, None),
    ("riseTimeI", VF, None), ("decayTimeFF", VF, None), ("decayTimeE", VF, None),
    ("decayTimeI", VF, None), ("decayTimeHomeoFF", F, 250.0), ("FF_InfRatio", F, 1.0),
    ("applyHomeo", I, 0), ("symmetricHomeo", B, True), ("v0", VF, None), ("w0", VF, None),
    ("gFF0", VF, None), ("gE0", VF, None), ("gI0", VF, None), ("pFF", VF, None),
    ("pE", VF, None), ("pI", VF, None), ("learning", I, 1), ("rebound", I, 0),
    ("iModel", I, 0), ("noDelay", I, 1), ("noFarDelay", I, 1), ("InhGap", B, False),
    ("A_LGN", VF, None), ("r_LTD", VF, None), ("A_V1", VF, None), ("A_Q", VF, None),
    ("symQ", B, True), ("nLearnTypeFF_I", U, 1), ("nLearnTypeFF_E", U, 1),
    ("nLearnTypeE", U, 1), ("tauQ", VF, None), ("tauLTP", VF, None), ("tauLTD", VF, None),
    ("tauTrip", VF, None), ("tauAvg", VF, None), ("targetFR", VF, None),
    ("gmaxLGN", VF, None), ("gmaxE", VF, None), ("gmaxQ", VF, None), ("gminLGN", VF, None),
    ("gminE", VF, None), ("gminQ", VF, None), ("vR", VF, None), ("vThres", VF, None),
    ("gL", VF, None), ("C", VF, None), ("tRef", VF, None), ("vT", VF, None),
    ("deltaT", VF, None), ("tau_w", VF, None), ("a", VF, None), ("b", VF, None),
    ("nTypeHierarchy", VU, None), ("spE0", VF, None), ("spI0", VF, None),
    ("SCsplit", U, 0), ("noisyDep", VF, None), ("tonicDep", VF, None), ("CmoreDep", B, True),
    ("noiseOnTonic", B, True), ("tau_noise", F, 0.0), ("minTonicRatio", VF, None),
    ("synFailFF", VF, None), ("synFail", VF, None), ("manual", B, False),
    ("preList", VU, None), ("postList", VU, None), ("sList", VF, None),
    ("readFeature", B, True), ("hWrite", B, True), ("saveLGN_fr", B, True),
    ("rawData", B, True), ("learnData_FF", I, 1), ("learnData_V1", B, False),
    ("framePhyV1output", B, False), ("frameVisV1output", B, False),
    ("frameVisLGNoutput", B, False), ("dot", F, 16.0), ("saveLGN_gallery", B, True),
    ("saveOutputB4V1", B, True), ("ignoreRetinogeniculateDelay", B, True),
    ("flat_retina", B, False), ("uniform_LGN", B, False), ("virtual_LGN", B, False),
    ("LGN_switch", B, False), ("switchType", I, 0), ("nOther", U, 0),
    ("reverseInput", B, False), ("getLGN_sp", B, False), ("delPrevSnapshot", B, True),
    ("asInit", B, True), ("minimal", B, False), ("sampleSize", U, 1000),
    ("sample_t0", F, 0.0), ("use_v0", B, False), ("store_dsLGN", B, False),
    ("useNewLGN", B, True),
    # files
    ("inputFolder", S, ""), ("resourceFolder", S, ""), ("res_suffix", S, ""),
    ("conV1_suffix", S, ""), ("conLGN_suffix", S, ""), ("snapshot_suffix", S, None),
    ("fConnectome_cfg", S, "connectome_cfg"), ("fSnapshot", S, ""),
    ("fLGN_switch", S, "LGN_switch"), ("fStimulus", S, "stimulus.bin"),
    ("fLGN_vpos", S, "LGN_vpos"), ("fLGN_V1_ID", S, "LGN_V1_idList"),
    ("fLGN_V1_s", S, "LGN_V1_sList"), ("fLGN_surfaceID", S, "LGN_surfaceID"),
    ("fV1_allpos", S, "V1_allpos"), ("fV1_feature", S, "V1_feature"),
    ("fV1_conMat", S, "V1_conMat"), ("fV1_delayMat", S, "V1_delayMat"),
    ("fV1_gapMat", S, "V1_gapMat"), ("fConStats", S, "conStats"), ("fV1_vec", S, "V1_vec"),
    ("fV1_gapVec", S, "V1_gapVec"), ("fNeighborBlock", S, "neighborBlock"),
    ("fV1_RF", S, "V1_RF"), ("outputFolder", S, ""), ("output_suffix", S, ""),
    ("fPatchV1_cfg", S, "patchV1_cfg"), ("fLGN", S, "LGN"), ("fLGN_fr", S, "LGN_fr"),
    ("fRawData", S, "rawData"), ("fLearnData_FF", S, "learnData_FF"), ("f_sLGN", S, "sLGN"),
    ("f_dsLGN", S, "dsLGN"), ("sampleInterval_LGN_V1", U, 100), ("fLGN_sp", S, "LGN_sp"),
    ("fOutputFrame", S, "outputFrame"), ("fOutputB4V1", S, "outputB4V1"),
    ("fLGN_gallery", S, "LGN_gallery"), ("fSample", S, "sample_spikeCount"),
]
KIND = {k: kind for k, kind, _ in OPTIONS}
DEFAULT = {k: d for k, _, d in OPTIONS}
SHORT = {"s": "seed", "c": "cfg_file", "p": "print", "n": "nChunk", "h": "help"}

_SPLIT = re.compile(r"\s?(;|,|\{|\}|\s)\s?")


class ConfigError(ValueError):
    pass


def _split_vector(text: str) -> list[str]:
    """Items of one vector occurrence, as the token iterator of src/util/po.h:25-33 yields
    them: the pieces between separators, a trailing empty piece dropped."""
    parts = _SPLIT.split(text)[::2]  # re.split also returns the captured separators
    if parts and parts[-1] == "":
        parts.pop()
    return parts


def _to_bool(key: str, s: str) -> bool:
    t = s.strip().lower()
    if t in ("", "on", "yes", "1", "true"):
        return True
    if t in ("off", "no", "0", "false"):
        return False
    raise ConfigError(f"invalid bool value '{s}' for option '{key}'")


def _to_uint(key: str, s: str, bits: int = 32) -> int:
    if not re.fullmatch(r"\s*\+?\d+\s*", s):
        raise ConfigError(f"invalid value '{s}' for option '{key}'")
    v = int(s)
    if v >= 1 << bits:
        raise ConfigError(f"value '{s}' out of range for option '{key}'")
    return v


def _to_int(key: str, s: str) -> int:
    if not re.fullmatch(r"\s*[+-]?\d+\s*", s):
        raise ConfigError(f"invalid value '{s}' for option '{key}'")
    return int(s)


def _to_float(key: str, s: str) -> float:
    try:
        if s.strip() != s or s == "":
            raise ValueError
        return float(s)
    except ValueError:
        raise ConfigError(f"invalid value '{s}' for option '{key}'") from None


def _convert(key: str, occurrences: list[str]):
    kind = KIND[key]
    if kind in (VF, VU):
        out = []
        for occ in occurrences:
            for item in _split_vector(occ):
                out.append(_to_float(key, item) if kind == VF else _to_uint(key, item))
        return out
    if len(occurrences) > 1:
        raise ConfigError(f"option '{key}' cannot be specified more than once")
    s = occurrences[0]
    if kind == B:
        return _to_bool(key, s)
    if kind == U:
        return _to_uint(key, s)
    if kind == "ulong":
        return _to_uint(key, s, 64)
    if kind == I:
        return _to_int(key, s)
    if kind == F:
        return _to_float(key, s)
    return s


def parse_config_text(text: str) -> dict[str, list[str]]:
    """Raw occurrences per key of a config file (boost parse_config_file)."""
    raw: dict[str, list[str]] = {}
    prefix = ""
    for lineno, line in enumerate(text.splitlines(), 1):
        s = line.split("#", 1)[0].strip()
        if not s:
            continue
        if s.startswith("[") and s.endswith("]"):
            prefix = s[1:-1].strip() + "."
            continue
        if "=" not in s:
            raise ConfigError(f"line {lineno}: syntax error in '{line.strip()}'")
        k, v = s.split("=", 1)
        k = prefix + k.strip()
        if k not in KIND:
            raise ConfigError(f"unrecognised option '{k}'")
        raw.setdefault(k, []).append(v.strip())
    return raw


def parse_command_line(argv: list[str]) -> dict[str, list[str]]:
    raw: dict[str, list[str]] = {}
    i = 0
    while i < len(argv):
        a = argv[i]
        if a.startswith("--"):
            k, eq, v = a[2:].partition("=")
        elif a.startswith("-") and len(a) >= 2:
            k, v, eq = SHORT.get(a[1], a[1]), a[2:], "=" if len(a) > 2 else ""
        else:
            raise ConfigError(f"unexpected argument '{a}'")
        if k == "help":
            raw["help"] = [""]
            i += 1
            continue
        if k not in KIND:
            raise ConfigError(f"unrecognised option '{a}'")
        if not eq:
            if KIND[k] == B and (i + 1 >= len(argv) or argv[i + 1].startswith("-")):
                v = ""
            else:
                i += 1
                if i >= len(argv):
                    raise ConfigError(f"option '{k}' needs a value")
                v = argv[i]
        raw.setdefault(k, []).append(v)
        i += 1
    return raw


@dataclass
class Config:
    values: dict
    given: set = field(default_factory=set)   # keys not defaulted

    def __getattr__(self, k):
        try:
            return self.values[k]
        except KeyError:
            raise AttributeError(k) from None

    def defaulted(self, k) -> bool:
        return k not in self.given


def load(argv: list[str] | None = None, cfg_text: str | None = None) -> Config:
    """Command line first, then the config file (``-c``), then defaults, as po::store does."""
    cmd = parse_command_line(list(argv or []))
    values, given = {}, set()
    for k, occ in cmd.items():
        if k == "help":
            continue
        values[k] = _convert(k, occ)
        given.add(k)
    if cfg_text is None:
        fn = values.get("cfg_file", DEFAULT["cfg_file"])
        try:
            with open(fn) as f:
                cfg_text = f.read()
        except OSError:
            raise ConfigError(f"cannot find specified config file {fn}") from None
    for k, occ in parse_config_text(cfg_text).items():
        if k in given:
            continue          # an option stored from the command line is final
        values[k] = _convert(k, occ)
        given.add(k)
    for k, d in DEFAULT.items():
        if k not in values and d is not None:
            values[k] = d
    return Config(values, given)


def _prefixed(folder: str, name: str) -> str:
    return name[1:] if name.startswith("!") else folder + name


def _suffix(s: str) -> str:
    return ("-" + s if s else "") + ".bin"


@dataclass
class Paths:
    stimulus: str
    lgn_vpos: str
    v1_allpos: str
    connectome_cfg: str
    conMat: str
    delayMat: str
    conStats: str
    v1_vec: str
    neighborBlock: str
    lgn_v1_id: str
    lgn_v1_s: str
    lgn: str
    patchV1_cfg: str
    lgn_fr: str
    raw: str
    lgn_sp: str
    slgn: str
    dslgn: str


def resolve_paths(c: Config) -> Paths:
    """File names with folders and suffixes (src/patch.cu:407-580 and the open calls)."""
    res, inp, out = c.resourceFolder, c.inputFolder, c.outputFolder
    rs, v1s, lgs, outs = (_suffix(c.res_suffix), _suffix(c.conV1_suffix),
                          _suffix(c.conLGN_suffix), _suffix(c.output_suffix))
    return Paths(
        stimulus=_prefixed(res, c.fStimulus),
        lgn_vpos=_prefixed(res, c.fLGN_vpos) + rs,
        v1_allpos=_prefixed(res, c.fV1_allpos) + rs,
        connectome_cfg=_prefixed(inp, c.fConnectome_cfg) + v1s,
        conMat=_prefixed(inp, c.fV1_conMat) + v1s,
        delayMat=_prefixed(inp, c.fV1_delayMat) + v1s,
        conStats=_prefixed(inp, c.fConStats) + v1s,
        v1_vec=_prefixed(inp, c.fV1_vec) + v1s,
        neighborBlock=_prefixed(inp, c.fNeighborBlock) + v1s,
        lgn_v1_id=_prefixed(inp, c.fLGN_V1_ID) + lgs,
        lgn_v1_s=_prefixed(inp, c.fLGN_V1_s) + lgs,
        lgn=_prefixed(out, c.fLGN),           # read without a suffix when useNewLGN = false
        patchV1_cfg=_prefixed(out, c.fPatchV1_cfg) + outs,
        lgn_fr=_prefixed(out, c.fLGN_fr) + outs,
        raw=_prefixed(out, c.fRawData) + outs,
        lgn_sp=_prefixed(out, c.fLGN_sp) + outs,
        slgn=_prefixed(out, c.f_sLGN) + outs,
        dslgn=_prefixed(out, c.f_dsLGN) + outs,
    )


def format_value(v) -> str:
    if isinstance(v, bool):
        return "true" if v else "false"
    if isinstance(v, (list, tuple)):
        return ", ".join(repr(float(x)) if isinstance(x, float) else str(x) for x in v)
    return str(v)


def write_cfg(values: dict) -> str:
    """Config-file text for a dict of keys (vectors on one line)."""
    return "".join(f"{k} = {format_value(v)}\n" for k, v in values.items())


__all__ = ["OPTIONS", "Config", "ConfigError", "load", "parse_config_text",
           "parse_command_line", "resolve_paths", "Paths", "write_cfg"]
