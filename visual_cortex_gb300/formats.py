"""Binary files of the patchV1 path: little-endian, ``Size`` = uint32, ``Float`` = float32.

Inputs (read by the driver, written by the synthetic generator):
  connectome_cfg   src/patch.cu:636-645     nType, nTypeI, typeAccCount[nType]
  V1_allpos        src/patch.cu:2754-2776   nblock, blockSize, posDim, f64 x0, xspan, y0,
                                            yspan, f64 pos[2][nV1]
  V1_conMat        src/patch.cu:3442-3680   nearNeighborBlock, f32 [nblock][nnb][pre][post]
  V1_delayMat      src/patch.cu:3450-3460   same layout (distances in mm)
  neighborBlock    src/patch.cu:3481-3497   nNearNeighborBlock[nblock], nNeighborBlock[nblock],
                                            then per block its neighbour ids
  conStats         src/patch.cu:4119-4133   nType, nV1, f32 ffRatio[nV1] (rest unread)
  V1_vec           src/patch.cu:3313-3352   i32 connectLongRange, nVec[nV1] (a second nVec if
                                            connectLongRange == 1), then per post with
                                            nVec > 0: ids, f32 strengths, f32 distances
  LGN_V1_idList    src/util/util.h:162-186  nList, then per list: n, u32 ids[n]
  LGN_V1_sList     src/patch.h:30-77        nList, maxList, then per list: n, f32 s[n]
  stimulus         src/patch.cu:1393-1471   i32 inputType, nFrame, height, width, f32 init_L,
                                            init_M, init_S, f32 domain[2], u32 neye, then per
                                            frame L, M, S planes [height][width]
  LGN_vpos         src/patch.cu:1523-1700   nLGN_I, nLGN_C, f32 max_ecc, f32 x0, xspan, y0,
                                            yspan, f32 x[nLGN], y[nLGN], u32 LGNtype[nLGN]
  LGN              src/patch.cu:2505-2530   nLGN, u32 LGNtype[nLGN], f32 polar, ecc, rw, rh,
                                            orient, k, ratio, tauR, tauD, nR, nD, delay
                                            [2][nLGN], f32 spont, c50, sharpness [nLGN],
                                            u32 coneType[2][nLGN], f32 covariant[nLGN]
Outputs:
  rawData          src/patch.cu:4704-4713 header, one record per step (6140-6163, 6258,
                   6916-6925): sInfo, dep, [w], v, gFF, [hFF], gE, gI, [hE, hI], gap[mI]
  LGN_sp           src/patch.cu:4835-4837 {dt, nt, nLGN}, then sInfo[nLGN] per step (6423)
  LGN_fr           src/patch.cu:4682-4683 {nt, nLGN}, then fr[nLGN] per step (6346)
  patchV1_cfg      src/patch.cu:6954-7030
"""
from __future__ import annotations

import io
from dataclasses import dataclass

import numpy as np

f32, u32, i32, f64 = np.float32, np.uint32, np.int32, np.float64


def _w(f, arr, dtype):
    f.write(np.ascontiguousarray(arr, dtype=dtype).tobytes())


def _r(f, dtype, n=1):
    n = int(n)
    b = f.read(np.dtype(dtype).itemsize * n)
    if len(b) != np.dtype(dtype).itemsize * n:
        raise EOFError(f"file ends early ({len(b)} of {np.dtype(dtype).itemsize * n} bytes)")
    return np.frombuffer(b, dtype=dtype).copy()


def _r1(f, dtype):
    return _r(f, dtype, 1)[0].item()


# ------------------------------------------------------------------ inputs

def write_connectome_cfg(fn, nType, nTypeI, typeAcc):
    with open(fn, "wb") as f:
        _w(f, [nType, nTypeI], u32)
        _w(f, typeAcc, u32)


def read_connectome_cfg(fn):
    with open(fn, "rb") as f:
        nType = _r1(f, u32)
        nTypeI = _r1(f, u32)
        acc = _r(f, u32, nType)
    return nType, nTypeI, acc


def write_v1_allpos(fn, nblock, blockSize, pos, vpos=None):
    """pos: [nV1][2] in mm; vpos: optional visual-field positions [nV1][2] in degrees, written
    after the physical block."""
    pos = np.asarray(pos, dtype=f64)
    with open(fn, "wb") as f:
        _w(f, [nblock, blockSize, 2], u32)
        for p in ([pos] if vpos is None else [pos, np.asarray(vpos, dtype=f64)]):
            x0, y0 = p[:, 0].min(), p[:, 1].min()
            _w(f, [x0, p[:, 0].max() - x0, y0, p[:, 1].max() - y0], f64)
            _w(f, p[:, 0], f64)
            _w(f, p[:, 1], f64)


def read_v1_allpos(fn):
    with open(fn, "rb") as f:
        nblock, blockSize, posDim = (_r1(f, u32) for _ in range(3))
        if posDim > 2:
            raise ValueError("3-D positions are not implemented")
        _r(f, f64, 4)
        n = nblock * blockSize
        x = _r(f, f64, n)
        y = _r(f, f64, n)
    return nblock, blockSize, np.stack([x, y], 1)


def read_v1_allpos_spans(fn):
    """(x0, xspan, y0, yspan) of the physical V1 sheet from the V1_allpos header
    (src/patch.cu:2759-2767)."""
    with open(fn, "rb") as f:
        _r(f, u32, 3)
        x0, xspan, y0, yspan = (float(v) for v in _r(f, f64, 4))
    return x0, xspan, y0, yspan


def write_v1_feature(fn, values):
    """V1_feature: nFeature u32, then values [nFeature][nV1] f32 (feature 0: ocular dominance,
    < 0 ipsilateral; feature 1: preferred orientation in [0, 1))."""
    v = np.asarray(values, f32)
    with open(fn, "wb") as f:
        _w(f, [v.shape[0]], u32)
        _w(f, v, f32)


def read_v1_feature(fn, nV1):
    """src/patch.cu:2912-2925: [nFeature][nV1]."""
    with open(fn, "rb") as f:
        n = _r1(f, u32)
        return _r(f, f32, n * nV1).reshape(n, nV1)


def underlying_ids(x, y, width, height, x0, xspan, y0, yspan, dtype=f64, n0=0, pick=None):
    """getUnderlyingID (src/stats.cuh:26-60) for all cells given: pixel idx + idy*width of
    each position ((x - x0)/xspan*width in `dtype` -- double for V1, float for LGN --,
    truncated, the far edge folded into the last pixel); returns (offsets [width*height + 1],
    ids + n0 in cell order within each pixel)."""
    t = dtype
    x, y = np.asarray(x, t), np.asarray(y, t)
    index = np.arange(len(x))
    if pick is not None:      # only the picked cells, under their own indices
        index = np.nonzero(pick)[0]
        x, y = x[index], y[index]
    idx = ((x - t(x0)) / t(xspan) * t(width)).astype(np.int64)
    idy = ((y - t(y0)) / t(yspan) * t(height)).astype(np.int64)
    idx[idx == width] -= 1
    idy[idy == height] -= 1
    if (idx < 0).any() or (idx >= width).any() or (idy < 0).any() or (idy >= height).any():
        raise ValueError("a position lies outside the frame's span")
    pid = idx + idy * width
    order = np.argsort(pid, kind="stable")
    off = np.zeros(width * height + 1, np.int64)
    np.add.at(off, pid + 1, 1)
    return np.cumsum(off).astype(u32), (index[order] + n0).astype(u32)


def read_v1_allpos_visual(fn):
    """The visual-field block of V1_allpos that follows the physical positions when
    visual-field V1 frames are asked for (src/patch.cu:2774-2781): (vx0, vxspan, vy0, vyspan,
    vx, vy)."""
    with open(fn, "rb") as f:
        nblock, blockSize, _ = (_r1(f, u32) for _ in range(3))
        n = nblock * blockSize
        _r(f, f64, 4 + 2 * n)
        sp = [float(v) for v in _r(f, f64, 4)]
        if len(sp) < 4:
            raise ValueError(f"{fn}: no visual positions after the physical ones")
        vx = _r(f, f64, n)
        vy = _r(f, f64, n)
    return sp[0], sp[1], sp[2], sp[3], vx, vy


def read_lgn_vpos_spans(fn):
    """(x0, xspan, y0, yspan) of the LGN visual positions (src/patch.cu:1688-1701)."""
    with open(fn, "rb") as f:
        _r(f, u32, 2)
        _r(f, f32, 1)
        return tuple(float(v) for v in _r(f, f32, 4))


class OutputFrameWriter:
    """outputFrame: {dt f32, ot u32, iFrameOutput u32 (bits: 1 physical V1, 2 visual-field V1,
    4 visual-field LGN), then width, height u32 of each kind present} then the frames
    (src/patch.cu:4843-4871, 6778-6786)."""

    def __init__(self, fn, dt, ot, kinds, sizes):
        self.f = open(fn, "wb")
        _w(self.f, [dt], f32)
        _w(self.f, [ot, kinds], u32)
        for w, h in sizes:
            _w(self.f, [w, h], u32)

    def write(self, frames):
        self.f.write(np.ascontiguousarray(frames, f32).tobytes())

    def close(self):
        self.f.close()


def write_mat(fn, nnb, mat):
    """conMat / delayMat: mat [nblock][nnb][bs][bs]."""
    with open(fn, "wb") as f:
        _w(f, [nnb], u32)
        _w(f, mat, f32)


def read_mat(fn, nblock, blockSize):
    with open(fn, "rb") as f:
        nnb = _r1(f, u32)
        m = _r(f, f32, nblock * nnb * blockSize * blockSize)
    return nnb, m.reshape(nblock, nnb, blockSize, blockSize)


def write_neighbor_block(fn, nNear, neighbors):
    """nNear[nblock]; neighbors: per block the list of all neighbour ids (near ones first)."""
    with open(fn, "wb") as f:
        _w(f, nNear, u32)
        _w(f, [len(x) for x in neighbors], u32)
        for x in neighbors:
            _w(f, x, u32)


def read_neighbor_block(fn, nblock, nnb):
    with open(fn, "rb") as f:
        nNear = _r(f, u32, nblock)
        nAll = _r(f, u32, nblock)
        if nNear.max(initial=0) > nnb:
            raise ValueError("conMat nearNeighborBlock not compatible with nNearNeighborBlock")
        ids = np.zeros((nblock, nnb), u32)
        for b in range(nblock):
            if nAll[b] > 0:
                t = _r(f, u32, nAll[b])
                if t.max() >= nblock:
                    raise ValueError("conMat neighbor blockID exceeds nblock")
                ids[b, :nNear[b]] = t[:nNear[b]]
    return nNear, ids


def write_con_stats(fn, nType, ffRatio):
    with open(fn, "wb") as f:
        _w(f, [nType, len(ffRatio)], u32)
        _w(f, ffRatio, f32)


def read_con_stats(fn, nType, nV1):
    with open(fn, "rb") as f:
        t = _r1(f, u32)
        n = _r1(f, u32)
        if t != nType or n != nV1:
            raise ValueError(f"conStats holds nType={t}, nV1={n}; expected {nType}, {nV1}")
        return _r(f, f32, nV1)


def write_v1_vec(fn, nVec, vecID, conVec, delayVec):
    nVec = np.asarray(nVec, u32)
    with open(fn, "wb") as f:
        _w(f, [0], i32)
        _w(f, nVec, u32)
        off = 0
        for n in nVec:
            if n > 0:
                _w(f, vecID[off:off + n], u32)
                _w(f, conVec[off:off + n], f32)
                _w(f, delayVec[off:off + n], f32)
            off += int(n)


def read_v1_vec(fn, nV1):
    """nVec, vecID, conVec (unscaled), delayVec, flattened in post order."""
    with open(fn, "rb") as f:
        longRange = _r1(f, i32)
        nVec = _r(f, u32, nV1)
        if longRange == 1:
            _r(f, u32, nV1)
        ids, s, d = [], [], []
        for n in nVec:
            if n > 0:
                ids.append(_r(f, u32, n))
                s.append(_r(f, f32, n))
                d.append(_r(f, f32, n))
    cat = lambda xs, t: np.concatenate(xs).astype(t) if xs else np.zeros(0, t)
    return nVec, cat(ids, u32), cat(s, f32), cat(d, f32)


def write_list_of_lists(fn, lists, dtype, with_max=False):
    with open(fn, "wb") as f:
        _w(f, [len(lists)], u32)
        if with_max:
            _w(f, [max((len(x) for x in lists), default=0)], u32)
        for x in lists:
            _w(f, [len(x)], u32)
            _w(f, x, dtype)


def read_list_of_lists(fn, dtype, with_max=False):
    with open(fn, "rb") as f:
        n = _r1(f, u32)
        mx = _r1(f, u32) if with_max else None
        out = [_r(f, dtype, _r1(f, u32)) for _ in range(n)]
    return (out, mx) if with_max else out


def write_stimulus(fn, frames, init_LMS, domain=(0.0, 1.0), neye=1):
    """frames: [nFrame][3][h][w] f32 (L, M, S planes)."""
    frames = np.asarray(frames, f32)
    nFrame, _, h, w = frames.shape
    with open(fn, "wb") as f:
        _w(f, [-1], i32)
        _w(f, [nFrame, h, w], u32)
        _w(f, init_LMS, f32)
        _w(f, domain, f32)
        _w(f, [neye], u32)
        _w(f, frames, f32)


@dataclass
class StimulusFile:
    inputType: int
    frames: np.ndarray
    init_LMS: tuple
    buffer: float
    range: float
    neye: int


def read_stimulus(fn):
    with open(fn, "rb") as f:
        inputType = _r1(f, i32)
        nFrame, h, w = (_r1(f, u32) for _ in range(3))
        if inputType != -1:
            raise ValueError(f"inputType {inputType} does not match with normal external stimulus")
        init = tuple(float(x) for x in _r(f, f32, 3))
        dom = _r(f, f32, 2)
        neye = _r1(f, u32)
        frames = _r(f, f32, nFrame * 3 * h * w).reshape(nFrame, 3, h, w)
    return StimulusFile(inputType, frames, init, float(dom[0]), float(dom[1]), neye)


def write_lgn_vpos(fn, nLGN_I, nLGN_C, max_ecc, x, y, LGNtype):
    with open(fn, "wb") as f:
        _w(f, [nLGN_I, nLGN_C], u32)
        _w(f, [max_ecc], f32)
        _w(f, [x.min(), x.max() - x.min(), y.min(), y.max() - y.min()], f32)
        _w(f, x, f32)
        _w(f, y, f32)
        _w(f, LGNtype, u32)


def read_lgn_vpos(fn):
    with open(fn, "rb") as f:
        nI = _r1(f, u32)
        nC = _r1(f, u32)
        max_ecc = float(_r1(f, f32))
        _r(f, f32, 4)
        n = nI + nC
        x = _r(f, f32, n)
        y = _r(f, f32, n)
        t = _r(f, u32, n)
    return nI, nC, max_ecc, x, y, t


LGN_FIELDS2 = ("polar", "ecc", "rw", "rh", "orient", "k", "ratio", "tauR", "tauD", "nR", "nD",
               "delay")
LGN_FIELDS1 = ("spont", "c50", "sharpness")


def write_lgn_params(fn, LGNtype, p: dict):
    n = len(LGNtype)
    with open(fn, "wb") as f:
        _w(f, [n], u32)
        _w(f, LGNtype, u32)
        for k in LGN_FIELDS2:
            _w(f, p[k], f32)
        for k in LGN_FIELDS1:
            _w(f, p[k], f32)
        _w(f, p["coneType"], u32)
        _w(f, p.get("covariant", np.zeros(n, f32)), f32)


def read_lgn_params(fn, nLGN):
    with open(fn, "rb") as f:
        _r1(f, u32)
        out = {"LGNtype": _r(f, u32, nLGN)}
        for k in LGN_FIELDS2:
            out[k] = _r(f, f32, 2 * nLGN)
        for k in LGN_FIELDS1:
            out[k] = _r(f, f32, nLGN)
        out["coneType"] = _r(f, u32, 2 * nLGN)
        out["covariant"] = _r(f, f32, nLGN)
    return out


# ------------------------------------------------------------------ outputs

class RawDataWriter:
    """rawData: header, then one record per step in the order the step loop writes them."""

    def __init__(self, fn, dt, nt, nV1, iModel, mI, hWrite, ngFF, ngE, ngI):
        self.f = open(fn, "wb")
        _w(self.f, [dt], f32)
        _w(self.f, [nt, nV1], u32)
        _w(self.f, [iModel], i32)
        _w(self.f, [mI, int(bool(hWrite)), ngFF, ngE, ngI], u32)
        self.rec = nV1 * (3 + (iModel == 1) + (ngFF + ngE + ngI) * (1 + int(bool(hWrite)))) + mI

    def write(self, records: np.ndarray):
        records = np.ascontiguousarray(records, f32)
        assert records.size % self.rec == 0
        self.f.write(records.tobytes())

    def close(self):
        self.f.close()


def read_raw_header(f):
    dt = float(_r1(f, f32))
    nt, nV1 = (_r1(f, u32) for _ in range(2))
    iModel = _r1(f, i32)
    mI, hWrite, ngFF, ngE, ngI = (_r1(f, u32) for _ in range(5))
    return dict(dt=dt, nt=nt, nV1=nV1, iModel=iModel, mI=mI, hWrite=hWrite, ngFF=ngFF, ngE=ngE,
                ngI=ngI)


def read_raw(fn):
    """Header dict and the records [nt][floats per record], as src/readPatchOutput.py:291-354
    walks them."""
    with open(fn, "rb") as f:
        h = read_raw_header(f)
        rec = h["nV1"] * (3 + (h["iModel"] == 1) + (h["ngFF"] + h["ngE"] + h["ngI"]) *
                          (1 + h["hWrite"])) + h["mI"]
        data = np.frombuffer(f.read(), dtype=f32)
    assert data.size == h["nt"] * rec, (data.size, h["nt"], rec)
    return h, data.reshape(h["nt"], rec)


class LgnSpWriter:
    def __init__(self, fn, dt, nt, nLGN):
        self.f = open(fn, "wb")
        _w(self.f, [dt], f32)
        _w(self.f, [nt, nLGN], u32)

    def write(self, rows):
        self.f.write(np.ascontiguousarray(rows, f32).tobytes())

    def close(self):
        self.f.close()


class LgnFrWriter(LgnSpWriter):
    def __init__(self, fn, nt, nLGN):
        self.f = open(fn, "wb")
        _w(self.f, [nt, nLGN], u32)


class SLgnWriter:
    """f_sLGN (learnData_FF = 1): header {nt, sampleInterval_LGN_V1 (u32), dt (f32), nV1,
    max_LGNperV1 (u32), sRatioLGN[0..1] (f32), nLearnTypeFF_E, nLearnTypeFF_I (u32), gmaxLGN
    [nLearnTypeFF] (f32), FF_InfRatio (f32)} (src/patch.cu:4767-4776), then the LGN->V1 weights
    [max_LGNperV1][nV1] after every sampleInterval_LGN_V1 steps (src/patch.cu:6196-6200,
    6937-6938)."""

    def __init__(self, fn, nt, interval, dt, nV1, maxLGN, sRatioLGN2, nFF_E, nFF_I, gmaxLGN, FF_InfRatio):
        self.f = open(fn, "wb")
        _w(self.f, [nt, interval], u32)
        _w(self.f, [dt], f32)
        _w(self.f, [nV1, maxLGN], u32)
        _w(self.f, list(sRatioLGN2)[:2], f32)
        _w(self.f, [nFF_E, nFF_I], u32)
        _w(self.f, list(gmaxLGN)[:nFF_E + nFF_I], f32)
        _w(self.f, [FF_InfRatio], f32)

    def write(self, sLGN):
        self.f.write(np.ascontiguousarray(sLGN, f32).tobytes())

    def close(self):
        self.f.close()


class DsLgnWriter:
    """f_dsLGN (store_dsLGN with learnData_FF = 1): header {nt, sampleInterval_LGN_V1 (u32), dt
    (f32), nV1, max_LGNperV1 (u32), sRatioLGN[0..1] (f32), nLearnTypeFF_E, nLearnTypeFF_I
    (u32), A_LGN[nLearnTypeFF] (f32), the LTD ratio A_ratio * tauLTP of each type (f32),
    targetFR[0..1] (f32), learnData_FF (i32)} (src/patch.cu:4795-4810), then at each sample the
    filtered rates vAvgE [nblock*nE][2] when targetFR[0] > 0 and vAvgI [nblock*nI] when
    targetFR[1] > 0 (src/patch.cu:6201-6208)."""

    def __init__(self, fn, nt, interval, dt, nV1, maxLGN, sRatioLGN2, nFF_E, nFF_I, A_LGN, ltd_ratio, targetFR2,
                 learnData_FF):
        self.f = open(fn, "wb")
        _w(self.f, [nt, interval], u32)
        _w(self.f, [dt], f32)
        _w(self.f, [nV1, maxLGN], u32)
        _w(self.f, list(sRatioLGN2)[:2], f32)
        _w(self.f, [nFF_E, nFF_I], u32)
        _w(self.f, list(A_LGN)[:nFF_E + nFF_I], f32)
        _w(self.f, list(ltd_ratio), f32)
        _w(self.f, list(targetFR2)[:2], f32)
        _w(self.f, [learnData_FF], i32)
        self.targetFR = list(targetFR2)[:2]

    def write(self, avgE, avgI):
        if self.targetFR[0] > 0:
            self.f.write(np.ascontiguousarray(avgE, f32).tobytes())
        if self.targetFR[1] > 0:
            self.f.write(np.ascontiguousarray(avgI, f32).tobytes())

    def close(self):
        self.f.close()


def read_slgn(fn):
    """Header dict and the sampled weights [samples][max_LGNperV1][nV1] of an sLGN file."""
    with open(fn, "rb") as f:
        nt, interval = (_r1(f, u32) for _ in range(2))
        dt = float(_r1(f, f32))
        nV1, maxLGN = (_r1(f, u32) for _ in range(2))
        sr = _r(f, f32, 2)
        nE, nI = (_r1(f, u32) for _ in range(2))
        gmax = _r(f, f32, nE + nI)
        inf = float(_r1(f, f32))
        d = np.frombuffer(f.read(), f32)
    return (dict(nt=nt, interval=interval, dt=dt, nV1=nV1, maxLGN=maxLGN, sRatioLGN=sr, nLearnTypeFF_E=nE,
                 nLearnTypeFF_I=nI, gmaxLGN=gmax, FF_InfRatio=inf), d.reshape(-1, maxLGN, nV1))


def read_lgn_sp(fn):
    with open(fn, "rb") as f:
        dt = float(_r1(f, f32))
        nt, n = (_r1(f, u32) for _ in range(2))
        d = _r(f, f32, nt * n).reshape(nt, n)
    return dt, d


def read_lgn_fr(fn):
    with open(fn, "rb") as f:
        nt, n = (_r1(f, u32) for _ in range(2))
        d = _r(f, f32, nt * n).reshape(nt, n)
    return d


def _pad(v, n):
    v = list(v or [])
    return (v + [0.0] * n)[:n]


def patchv1_cfg_bytes(c, *, vL, vE, vI, nType, nTypeE, nTypeI, typeAcc, stimulus_filename, nLGN,
                      nV1, normViewDistance, L_x0, L_y0, R_x0, R_y0, ngFF, ngE, ngI,
                      seed) -> bytes:
    """patchV1_cfg as src/patch.cu:6954-7030 writes it; ``c`` is the parsed option set with
    the per-type vectors already expanded to nType as the reference does."""
    b = io.BytesIO()
    _w(b, [4], u32)
    _w(b, [vL, vE, vI], f32)
    _w(b, [nType, nTypeE, nTypeI], u32)
    for k in ("vR", "vThres", "gL", "vT"):
        _w(b, _pad(c[k], nType), f32)
    _w(b, _pad(c["nTypeHierarchy"], 2), u32)
    _w(b, typeAcc, u32)
    _w(b, _pad(c["sRatioLGN"], nType), f32)
    _w(b, _pad(c["sRatioV1"], nType * nType), f32)
    _w(b, [c["frRatioLGN"], c["convolRatio"]], f32)
    _w(b, [c["frameRate"]], u32)
    name = stimulus_filename.encode()
    _w(b, [len(name)], u32)
    b.write(name)
    _w(b, [nLGN, nV1, c["nt"]], u32)
    _w(b, [c["dt"], normViewDistance, L_x0, L_y0, R_x0, R_y0], f32)
    _w(b, _pad(c["tonicDep"], nType), f32)
    _w(b, _pad(c["noisyDep"], nType), f32)
    _w(b, [int(c["virtual_LGN"])], i32)
    _w(b, [seed], np.uint64)
    _w(b, [c["iModel"], c["learning"]], i32)
    _w(b, [ngFF, ngE, ngI], u32)
    for k, n in (("riseTimeFF", ngFF), ("decayTimeFF", ngFF), ("riseTimeE", ngE),
                 ("decayTimeE", ngE), ("riseTimeI", ngI), ("decayTimeI", ngI),
                 ("pFF", ngFF * nType), ("pE", ngE * nType), ("pI", ngI * nType),
                 ("C", nType), ("tRef", nType), ("a", nType), ("b", nType), ("tau_w", nType),
                 ("deltaT", nType)):
        _w(b, _pad(c[k], n), f32)
    nh = _pad(c["nTypeHierarchy"], 2)
    _w(b, _pad(c["spE0"], int(nh[0]) * 2), f32)
    _w(b, _pad(c["spI0"], int(nh[1]) * 2), f32)
    for k in ("v0", "w0", "gFF0", "gE0", "gI0"):
        _w(b, _pad(c[k], nType * 2), f32)
    _w(b, _pad(c["synFail"], nType * nType), f32)
    _w(b, _pad(c["synFailFF"], nType), f32)
    return b.getvalue()


# ------------------------------------------------------------------ snapshots (reference layout)

SNAPSHOT_INDICES = ("step", "frameCycle", "iFrameHead", "oldFrameHead", "currentFrame", "iFramePhaseHead",
                    "iFramePhaseTail", "mFramePhaseHead", "mFramePhaseTail", "iStatus", "currentTimeSlot")


def write_reference_snapshot(fn, idx: dict, iModel: int, learning: int, sizes: dict, lgn: dict, v1: dict,
                             spike_train, state: dict, trailer: bytes | None = None, learn: dict | None = None):
    """A snapshot in the reference's layout (src/patch.cu:6793-6912): 11 u32 indices (steps
    done, frame bookkeeping, iStatus, the next spike-word slot), iModel and learning (i32),
    nV1 nLGN ngFF ngE ngI nType trainDepth (u32); the LGN block (leftTimeRate, lastNegLogRand,
    the generators, 48 bytes each); rGenCond, rNoisy (48 bytes per neuron), tBack; the
    spike-word ring [trainDepth][nV1]; the state block dep, (w,) v, gFF, hFF, gE, gI, hE, hI,
    gap.  `trailer` (this build's own checkpoint) is appended after it: the reference's reader
    stops before it."""
    with open(fn, "wb") as f:
        _w(f, [idx[k] for k in SNAPSHOT_INDICES], u32)
        _w(f, [iModel, learning], i32)
        _w(f, [sizes[k] for k in ("nV1", "nLGN", "ngFF", "ngE", "ngI", "nType", "trainDepth")], u32)
        _w(f, lgn["ltr"], f32)
        _w(f, lgn["lnl"], f32)
        f.write(np.ascontiguousarray(lgn["rng"], np.uint8).tobytes())
        if learning:
            # the LGN->V1 weights, the post learning variables and the presynaptic traces
            # (src/patch.cu:6844-6850)
            _w(f, np.ravel(learn["sLGN"]), f32)
            _w(f, np.ravel(learn["ff_post"]), f32)
            _w(f, np.ravel(learn["ff_pre"]), f32)
        f.write(np.ascontiguousarray(v1["rng_cond"], np.uint8).tobytes())
        f.write(np.ascontiguousarray(v1["rng_noisy"], np.uint8).tobytes())
        _w(f, v1["tBack"], f32)
        _w(f, np.ravel(spike_train), f32)
        keys = ["dep"] + (["w"] if iModel == 1 else []) + ["v", "gFF", "hFF", "gE", "gI", "hE", "hI", "gap"]
        for k in keys:
            _w(f, np.ravel(state[k]), f32)
        if trailer is not None:
            f.write(trailer)


def read_reference_snapshot(fn, nI_total: int, maxLGN: int = 0, nE_total: int = 0, nFF_E: int = 1,
                            nFF_I: int = 0):
    """Reads a snapshot written by the reference (or by write_reference_snapshot); returns the
    fields and the bytes that follow them (this build's checkpoint, if it wrote the file).  A
    snapshot of a learning run also holds the LGN->V1 weights [maxLGN][nV1], the post learning
    variables (learnVar's FF block, src/patch.cu:4367-4369: 2 nE_total nFF_E + 2 nI_total nFF_I
    post traces, then vAvgE [nE_total][2] and vAvgI [nI_total]) and the presynaptic traces
    [nFF_E + nFF_I][nLGN]."""
    data = open(fn, "rb").read()
    off = 0

    def take(dtype, count):
        nonlocal off
        a = np.frombuffer(data, dtype, count, off)
        off += a.nbytes
        return a.copy()

    idx = dict(zip(SNAPSHOT_INDICES, (int(x) for x in take(u32, 11))))
    iModel, learning = (int(x) for x in take(i32, 2))
    sizes = dict(zip(("nV1", "nLGN", "ngFF", "ngE", "ngI", "nType", "trainDepth"), (int(x) for x in take(u32, 7))))
    n, nl = sizes["nV1"], sizes["nLGN"]
    lgn = dict(ltr=take(f32, nl), lnl=take(f32, nl), rng=take(np.uint8, 48 * nl))
    learn = None
    if learning:
        if not maxLGN:
            raise ValueError(f"{fn}: a snapshot of a learning run needs max_LGNperV1 to be read")
        post = 2 * nE_total * nFF_E + 2 * nI_total * nFF_I + 2 * nE_total + nI_total
        learn = dict(sLGN=take(f32, maxLGN * n), ff_post=take(f32, post), ff_pre=take(f32, (nFF_E + nFF_I) * nl))
    v1 = dict(rng_cond=take(np.uint8, 48 * n), rng_noisy=take(np.uint8, 48 * n), tBack=take(f32, n))
    spike_train = take(f32, sizes["trainDepth"] * n).reshape(sizes["trainDepth"], n)
    state = dict(dep=take(f32, n))
    if iModel == 1:
        state["w"] = take(f32, n)
    state["v"] = take(f32, n)
    for k, c in (("gFF", sizes["ngFF"]), ("hFF", sizes["ngFF"]), ("gE", sizes["ngE"]), ("gI", sizes["ngI"]),
                 ("hE", sizes["ngE"]), ("hI", sizes["ngI"])):
        state[k] = take(f32, c * n)
    state["gap"] = take(f32, nI_total)
    return dict(idx=idx, iModel=iModel, learning=learning, sizes=sizes, lgn=lgn, v1=v1,
                spike_train=spike_train, state=state, learn=learn), data[off:]
