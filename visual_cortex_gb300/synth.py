"""Seeded synthetic workloads in the reference's input layouts.

No dataset or connectome ships with the reference, so every workload is generated here from
a seed: a V1 sheet of blocks, Gaussian distance-dependent recurrent connectivity (a dense
conMat tile per block, a sparse far list with distance delays), ON/OFF magno LGN cells with
DoG receptive fields, simple-cell-like LGN->V1 wiring, and a drifting-grating stimulus.
The same objects are written to the reference's file formats by formats.py.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

from .model import InitState, LgnSpec, Seeds, Stimulus, V1Network, V1Spec, host_init_state
from .schedule import make_schedule
from .retina import retina_geometry

f32 = np.float32
u32 = np.uint32
DEG = math.pi / 180.0


@dataclass
class Workload:
    name: str
    spec: V1Spec
    net: V1Network
    lgn: LgnSpec
    stim: Stimulus
    init: InitState
    seeds: Seeds
    nt: int
    pos: np.ndarray          # V1 positions [nV1][2] (mm)
    rf_center: np.ndarray    # V1 RF centers [nV1][2] (deg)
    rf_orient: np.ndarray    # V1 preferred orientation [nV1] (rad)


def make_spec(nblock: int, blockSize: int = 1024, nE: int = 768, dt: float = 0.125,
              adex_inh: bool = False, vL: float = -65.0, noisyDep=(0.0, 0.0),
              synFail=(0.0, 0.0, 0.0, 0.0), synFailFF=(0.0, 0.0), noFarDelay: int = 0) -> V1Spec:
    """Neuron and synapse recipe of the benchmark configurations.

    Conductance-based LIF (gL 0.05/ms, C 1, threshold -50 mV, reset -60 mV, refractory
    2/1 ms) written as the reference's AdEx with a = b = 0 and vT = vThres; AMPA 1/5 ms,
    NMDA 2/80 ms (feed-forward and cortical excitation) and GABA 1/7 ms.  With adex_inh the
    inhibitory type is AdEx (a 0.02, b 0.4, tau_w 150 ms in the normalised units C = 1)."""
    a_i, b_i = (0.02, 0.4) if adex_inh else (0.0, 0.0)
    return V1Spec(
        nblock=nblock, blockSize=blockSize, typeAcc=[nE, blockSize], nTypeE=1,
        ngFF=2, ngE=2, ngI=1, dt=dt,
        riseFF=[1.0, 2.0], decayFF=[5.0, 80.0], riseE=[1.0, 2.0], decayE=[5.0, 80.0],
        riseI=[1.0], decayI=[7.0],
        vR=[-60.0, -60.0], vThres=[-50.0, -50.0], gL=[0.05, 0.05], C=[1.0, 1.0],
        tRef=[2.0, 1.0], vT=[-50.0, -50.0], deltaT=[1.0, 1.0], tau_w=[150.0, 150.0],
        a=[0.0, a_i], b=[0.0, b_i],
        pFF=[0.8, 0.2, 0.8, 0.2], pE=[0.8, 0.2, 0.8, 0.2], pI=[1.0, 1.0],
        synFail=list(synFail), synPerCon=[10.0, 10.0, 10.0, 10.0],
        synFailFF=list(synFailFF), synPerConFF=[10.0, 10.0], noisyDep=list(noisyDep),
        tau_noise=0.0, noiseOnTonic=True, iModel=1, noDelay=1, noFarDelay=noFarDelay,
        speedOfThought=1.0, hWrite=True, vE=0.0, vI=-75.0, vL=vL)


def grating_frames(nFrame: int, width: int, height: int, extent_deg: float, cpd: float,
                   tf_hz: float, contrast: float, orient: float, frame_rate: int,
                   mean: float = 0.5) -> np.ndarray:
    """Drifting sinusoidal grating, identical L, M, S planes, [nFrame][3][h][w] float32."""
    xs = (np.arange(width) + 0.5) / width * extent_deg - extent_deg / 2
    ys = (np.arange(height) + 0.5) / height * extent_deg - extent_deg / 2
    X, Y = np.meshgrid(xs, ys)
    proj = X * math.cos(orient) + Y * math.sin(orient)
    out = np.empty((nFrame, 3, height, width), f32)
    for f in range(nFrame):
        t = f / frame_rate
        img = mean * (1 + contrast * np.sin(2 * math.pi * (cpd * proj - tf_hz * t)))
        out[f, :] = img.astype(f32)
    return out


def make_lgn(n_lgn: int, rng: np.random.Generator, patch_deg: float, dt: float,
             frame_rate: int = 120, mSample1D: int = 16, mau: float = 250.0,
             mKernelSample: int = 250, sigma_c: float = 0.03, sigma_s: float = 0.09,
             stim_range_deg: float | None = None, buffer_deg: float = 0.2,
             jitter: float = 0.0, tjitter: float = 0.0, n_parvo: int = 0,
             tau: float | None = None, nKernelSample: int | None = None,
             nSample1D: int = 8, flat_retina: bool = True, contra: bool = False) -> tuple[LgnSpec, float]:
    """ON/OFF magno cells with centers uniform in a patch_deg square around the fixation;
    with n_parvo > 0 also parvocellular L/M-opponent cells (LGN ids 0..n_parvo-1, before the
    magno cells as the reference orders them), centre and surround at slightly different
    positions and orientations, each with its own temporal kernel, sampled over `tau` ms with
    nKernelSample taps.

    flat_retina = False: the cells sit in the right hemifield of a curved retina whose
    sample points are projected to the stimulus plane (the left eye's half of a binocular
    texture).

    Returns the spec and the full stimulus extent (deg) the texture spans."""
    nOn = n_lgn // 2
    xy = rng.uniform(-patch_deg / 2, patch_deg / 2, size=(n_lgn, 2))
    if not flat_retina:
        xy[:, 0] = np.abs(xy[:, 0]) + 0.1 * patch_deg
    polar = np.arctan2(xy[:, 1], xy[:, 0])
    ecc = np.hypot(xy[:, 0], xy[:, 1]) * DEG
    max_ecc = float(np.max(np.hypot(xy[:, 0], xy[:, 1])))
    if stim_range_deg is None:
        stim_range_deg = max(max_ecc, patch_deg / 2) * 1.05
    geo = retina_geometry(max_ecc, stim_range_deg, buffer_deg, flat_retina)
    extent, normViewDistance = geo["extent"], geo["normViewDistance"]
    sc = sigma_c * (1 + jitter * rng.uniform(-1, 1, n_lgn))
    ss = sigma_s * (1 + jitter * rng.uniform(-1, 1, n_lgn))
    two = lambda c, s: np.concatenate([c, s]).astype(f32)
    types = np.where(np.arange(n_lgn) < nOn, 4, 5)
    k_center = np.where(types == 4, 60.0, -60.0)
    sched = make_schedule(dt, frame_rate, mau if tau is None else tau, mau, mKernelSample if nKernelSample is None
                          else nKernelSample, mKernelSample)
    if n_parvo > 0:
        if contra and flat_retina:
            raise ValueError("a second eye needs the curved retina")
        return _with_parvo(n_lgn, n_parvo, rng, patch_deg, sched, mSample1D, nSample1D, sigma_c, sigma_s,
                           stim_range_deg, buffer_deg, jitter, flat_retina, contra)
    spec = LgnSpec(
        nParvo_I=0, nMagno_I=n_lgn, nParvo_C=0, nMagno_C=0, mSample1D=mSample1D, sched=sched,
        polar=two(polar, polar), ecc=two(ecc, ecc), rw=two(sc * DEG, ss * DEG),
        rh=two(sc * DEG, ss * DEG), orient=two(np.zeros(n_lgn), np.zeros(n_lgn)),
        k=two(k_center, -k_center), ratio=two(np.full(n_lgn, 1.0), np.full(n_lgn, 1.0)),
        tauR=two(1.5 * (1 + tjitter * rng.uniform(-1, 1, n_lgn)), np.full(n_lgn, 1.5)),
        tauD=two(4.5 * (1 + tjitter * rng.uniform(-1, 1, n_lgn)), np.full(n_lgn, 4.5)),
        nR=two(np.full(n_lgn, 19.0), np.full(n_lgn, 19.0)),
        nD=two(np.full(n_lgn, 9.5), np.full(n_lgn, 9.5)),
        delay=two(np.full(n_lgn, 14.0), np.full(n_lgn, 14.0)),
        spont=np.full(n_lgn, 0.1, f32), c50=np.full(n_lgn, 0.25, f32),
        sharpness=np.full(n_lgn, 3.0, f32),
        coneType=np.full(2 * n_lgn, 3, u32),
        normViewDistance=normViewDistance, L_x0=geo["L_x0"], L_y0=geo["L_y0"], R_x0=geo["R_x0"],
        R_y0=geo["R_y0"], nsig=3.0, convolRatio=1.0, frRatio=1.0, flat_retina=flat_retina)
    spec.types = types
    spec.xy = xy
    return spec, extent


def _with_parvo(n_magno, n_parvo, rng, patch_deg, sched, mSample1D, nSample1D, sigma_c, sigma_s,
                stim_range_deg, buffer_deg, jitter, flat_retina=True, contra=False):
    """LGN of n_parvo parvo cells (ids first) and n_magno ON/OFF magno cells, one eye; with
    contra (curved retina only) half of each kind in the second eye."""
    n = n_parvo + n_magno
    xy = rng.uniform(-patch_deg / 2, patch_deg / 2, size=(n, 2))
    if not flat_retina:
        xy[:, 0] = np.abs(xy[:, 0]) + 0.1 * patch_deg
    # surround centres of the parvo cells sit a little off their centres
    sxy = xy.copy()
    sxy[:n_parvo] += rng.normal(0.0, 0.01, size=(n_parvo, 2))
    polar = np.arctan2(xy[:, 1], xy[:, 0])
    ecc = np.hypot(xy[:, 0], xy[:, 1]) * DEG
    spolar = np.arctan2(sxy[:, 1], sxy[:, 0])
    secc = np.hypot(sxy[:, 0], sxy[:, 1]) * DEG
    max_ecc = float(max(np.max(np.hypot(xy[:, 0], xy[:, 1])), np.max(np.hypot(sxy[:, 0], sxy[:, 1]))))
    if stim_range_deg is None:
        stim_range_deg = max(max_ecc, patch_deg / 2) * 1.05
    geo = retina_geometry(max_ecc, stim_range_deg, buffer_deg, flat_retina)
    extent, normViewDistance = geo["extent"], geo["normViewDistance"]
    types = np.empty(n, np.int64)
    types[:n_parvo] = np.arange(n_parvo) % 4          # LonMoff, LoffMon, MonLoff, MoffLon
    types[n_parvo:] = np.where(np.arange(n_magno) < n_magno // 2, 4, 5)
    sc = sigma_c * (1 + jitter * rng.uniform(-1, 1, n))
    ss = sigma_s * (1 + jitter * rng.uniform(-1, 1, n))
    on_center = (types == 0) | (types == 2) | (types == 4)
    kc = np.where(on_center, 60.0, -60.0)
    ks = -kc
    ks[:n_parvo] *= 0.8
    orient_c = np.zeros(n)
    orient_s = np.zeros(n)
    orient_c[:n_parvo] = rng.uniform(0, math.pi, n_parvo)
    orient_s[:n_parvo] = orient_c[:n_parvo] + rng.uniform(-0.3, 0.3, n_parvo)
    rw_c = sc * DEG
    rh_c = sc * DEG
    rh_c[:n_parvo] *= 1.2                               # elongated parvo components
    rw_s = ss * DEG
    rh_s = ss * DEG * np.where(np.arange(n) < n_parvo, 0.9, 1.0)
    cone_c = np.full(n, 3, np.int64)
    cone_s = np.full(n, 3, np.int64)
    cone_c[:n_parvo] = np.where(types[:n_parvo] < 2, 0, 1)
    cone_s[:n_parvo] = 1 - cone_c[:n_parvo]
    tauR_c = np.full(n, 1.5)
    tauD_c = np.full(n, 4.5)
    tauR_s = np.full(n, 1.5)
    tauD_s = np.full(n, 4.5)
    tauR_s[:n_parvo] = 1.9
    tauD_s[:n_parvo] = 5.5
    delay_c = np.full(n, 14.0)
    delay_s = np.full(n, 14.0)
    delay_s[:n_parvo] = 17.0
    two = lambda c, s_: np.concatenate([c, s_]).astype(f32)
    spec = LgnSpec(
        nParvo_I=n_parvo, nMagno_I=n_magno, nParvo_C=0, nMagno_C=0, mSample1D=mSample1D, sched=sched,
        polar=two(polar, spolar), ecc=two(ecc, secc), rw=two(rw_c, rw_s), rh=two(rh_c, rh_s),
        orient=two(orient_c, orient_s), k=two(kc, ks), ratio=two(np.full(n, 1.0), np.full(n, 1.0)),
        tauR=two(tauR_c, tauR_s), tauD=two(tauD_c, tauD_s), nR=two(np.full(n, 19.0), np.full(n, 19.0)),
        nD=two(np.full(n, 9.5), np.full(n, 9.5)), delay=two(delay_c, delay_s),
        spont=np.full(n, 0.1, f32), c50=np.where(types < 4, 0.3, 0.25).astype(f32),
        sharpness=np.where(types < 4, 2.5, 3.0).astype(f32),
        coneType=np.concatenate([cone_c, cone_s]).astype(u32),
        normViewDistance=normViewDistance, L_x0=geo["L_x0"], L_y0=geo["L_y0"], R_x0=geo["R_x0"],
        R_y0=geo["R_y0"], nsig=3.0, convolRatio=1.0, frRatio=1.0, flat_retina=flat_retina, nSample1D=nSample1D,
        covariant=np.where(types < 4, 0.53753461391295254, 1.0).astype(f32))
    spec.types = types
    spec.xy = xy
    if contra:
        _split_eyes(spec, n_parvo, n_magno)
    return spec, extent


def _split_eyes(spec: LgnSpec, n_parvo: int, n_magno: int):
    """Moves the second half of the parvo and of the magno cells to the second eye, in the
    reference's order parvo_I, magno_I, parvo_C, magno_C (src/patch.cu:1723-1750)."""
    n = n_parvo + n_magno
    pI, mI = n_parvo // 2, n_magno // 2
    parvo, magno = np.arange(n_parvo), n_parvo + np.arange(n_magno)
    perm = np.concatenate([parvo[:pI], magno[:mI], parvo[pI:], magno[mI:]])
    for name, val in list(vars(spec).items()):
        if isinstance(val, np.ndarray) and val.shape[:1] == (2 * n,):
            setattr(spec, name, np.concatenate([val[:n][perm], val[n:][perm]]))
        elif isinstance(val, np.ndarray) and val.shape[:1] == (n,):
            setattr(spec, name, val[perm])
    spec.nParvo_I, spec.nMagno_I = pI, mI
    spec.nParvo_C, spec.nMagno_C = n_parvo - pI, n_magno - mI


def near_distances(spec: V1Spec, pos: np.ndarray, nNearNB, nbId) -> np.ndarray:
    """delayMat [nblock][nnb][pre][post]: cortical distance (mm) from each neuron of neighbour
    block k (pre) to each neuron of block b (post), the layout of conMat."""
    bs, nb = spec.blockSize, spec.nblock
    out = np.zeros((nb, nbId.shape[1], bs, bs), f32)
    for b in range(nb):
        post = pos[b * bs:(b + 1) * bs]
        for k in range(int(nNearNB[b])):
            q = int(nbId[b, k])
            pre = pos[q * bs:(q + 1) * bs]
            out[b, k] = np.sqrt(((pre[:, None, :] - post[None, :, :]) ** 2).sum(-1)).astype(f32)
    return out


def block_positions(nblock: int, blockSize: int, side_mm: float, rng: np.random.Generator,
                    nbx: int | None = None):
    """Jittered-grid positions, blocks tiled on a sheet; returns pos [nV1][2] in mm."""
    g = int(math.ceil(math.sqrt(blockSize)))
    if nbx is None:
        nbx = int(math.ceil(math.sqrt(nblock)))
    pos = np.empty((nblock * blockSize, 2))
    for b in range(nblock):
        bx, by = b % nbx, b // nbx
        cells = rng.permutation(g * g)[:blockSize]
        gx, gy = cells % g, cells // g
        jit = rng.uniform(0, 1, size=(blockSize, 2))
        pos[b * blockSize:(b + 1) * blockSize, 0] = (bx + (gx + jit[:, 0]) / g) * side_mm
        pos[b * blockSize:(b + 1) * blockSize, 1] = (by + (gy + jit[:, 1]) / g) * side_mm
    return pos, nbx


def near_conmat(spec: V1Spec, pos: np.ndarray, rng: np.random.Generator, sigma: float,
                nE_partners: float, nI_partners: float, wE: float, wI: float,
                side_mm: float) -> np.ndarray:
    """Dense-probabilistic within-block tiles conMat[b][0][pre][post] (self block only)."""
    bs, nE = spec.blockSize, spec.nE
    nI = bs - nE
    area = side_mm * side_mm
    p0E = min(1.0, nE_partners / ((nE / area) * 2 * math.pi * sigma * sigma))
    p0I = min(1.0, nI_partners / ((nI / area) * 2 * math.pi * sigma * sigma))
    out = np.zeros((spec.nblock, 1, bs, bs), f32)
    for b in range(spec.nblock):
        P = pos[b * bs:(b + 1) * bs]
        d2 = ((P[:, None, :] - P[None, :, :]) ** 2).sum(-1)   # [pre][post]
        p = np.exp(-d2 / (2 * sigma * sigma))
        p[:nE] *= p0E
        p[nE:] *= p0I
        np.fill_diagonal(p, 0.0)
        conn = rng.uniform(size=p.shape) < p
        w = rng.lognormal(0.0, 0.5, size=p.shape)
        w[:nE] *= wE
        w[nE:] *= wI
        out[b, 0] = np.where(conn, w, 0.0).astype(f32)
    return out


def far_vectors(spec: V1Spec, pos: np.ndarray, rng: np.random.Generator, n_partners: int,
                sigma: float, wE: float, wI: float, side_mm: float, nbx: int):
    """~n_partners Gaussian-distance partners per neuron from other blocks (V1_vec lists)."""
    bs, nV1 = spec.blockSize, spec.nV1
    nby = int(math.ceil(spec.nblock / nbx))
    g = int(math.ceil(math.sqrt(bs)))
    # lookup from (block, grid cell) to neuron id, built from the jittered grid positions
    cell_of = np.full((spec.nblock, g * g), -1, np.int64)
    bx = np.minimum((pos[:, 0] / side_mm).astype(int), nbx - 1)
    by = np.minimum((pos[:, 1] / side_mm).astype(int), nby - 1)
    gx = np.minimum(((pos[:, 0] / side_mm - bx) * g).astype(int), g - 1)
    gy = np.minimum(((pos[:, 1] / side_mm - by) * g).astype(int), g - 1)
    blk = np.arange(nV1) // bs
    cell_of[blk, gy * g + gx] = np.arange(nV1)
    ncand = n_partners * 3
    nVec = np.zeros(nV1, u32)
    ids, ws, ds = [], [], []
    chunk = 4096
    for s in range(0, nV1, chunk):
        e = min(nV1, s + chunk)
        P = pos[s:e]
        loc = P[:, None, :] + rng.normal(0, sigma, size=(e - s, ncand, 2))
        cbx = np.floor(loc[..., 0] / side_mm).astype(int)
        cby = np.floor(loc[..., 1] / side_mm).astype(int)
        ok = (cbx >= 0) & (cbx < nbx) & (cby >= 0) & (cby < nby)
        cb = np.where(ok, cby * nbx + cbx, 0)
        ok &= cb < spec.nblock
        cgx = np.clip(((loc[..., 0] / side_mm - cbx) * g).astype(int), 0, g - 1)
        cgy = np.clip(((loc[..., 1] / side_mm - cby) * g).astype(int), 0, g - 1)
        cand = np.where(ok, cell_of[np.where(ok, cb, 0), cgy * g + cgx], -1)
        own = (np.arange(s, e) // bs)[:, None]
        cand = np.where((cand >= 0) & (cand // bs != own), cand, -1)
        for r in range(e - s):
            c = cand[r]
            c = c[c >= 0]
            _, first = np.unique(c, return_index=True)
            c = c[np.sort(first)][:n_partners]
            i = s + r
            nVec[i] = len(c)
            d = np.sqrt(((pos[c] - pos[i]) ** 2).sum(-1))
            w = rng.lognormal(0.0, 0.5, size=len(c)) * np.where((c % bs) < spec.nE, wE, wI)
            ids.append(c.astype(u32))
            ws.append(w.astype(f32))
            ds.append(d.astype(f32))
    return (nVec, np.concatenate(ids) if ids else np.zeros(0, u32),
            np.concatenate(ws) if ws else np.zeros(0, f32),
            np.concatenate(ds) if ds else np.zeros(0, f32))


def lgn_to_v1(spec: V1Spec, lgn: LgnSpec, rng: np.random.Generator, m: int, w: float,
              patch_deg: float, sub_offset_deg: float = 0.05):
    """Simple-cell wiring: half ON cells near c + d*u, half OFF near c - d*u."""
    nV1 = spec.nV1
    xy = lgn.xy
    on = np.nonzero(lgn.types == 4)[0]
    off = np.nonzero(lgn.types == 5)[0]
    parvo = np.nonzero(lgn.types < 4)[0]
    centers = rng.uniform(-patch_deg / 2 * 0.8, patch_deg / 2 * 0.8, size=(nV1, 2))
    orient = rng.uniform(0, math.pi, nV1)
    u = np.stack([np.cos(orient + math.pi / 2), np.sin(orient + math.pi / 2)], -1)
    from scipy.spatial import cKDTree
    mp = m // 4 if parvo.size else 0      # parvo inputs: the cells nearest the RF centre
    mm = m - mp
    mo = mm // 2
    _, kon = cKDTree(xy[on]).query(centers + sub_offset_deg * u, k=mo)
    _, koff = cKDTree(xy[off]).query(centers - sub_offset_deg * u, k=mm - mo)
    kon = np.asarray(kon).reshape(nV1, mo)
    koff = np.asarray(koff).reshape(nV1, mm - mo)
    parts = [on[kon], off[koff]]
    if mp:
        _, kp = cKDTree(xy[parvo]).query(centers, k=mp)
        parts.append(parvo[np.asarray(kp).reshape(nV1, mp)])
    ids = np.concatenate(parts, axis=1).T.astype(u32).copy()
    s = (w * rng.uniform(0.5, 1.5, size=(m, nV1))).astype(f32)
    return np.full(nV1, m, u32), ids, s, centers, orient


def make_workload(name: str = "C1", seed: int = 0, nblock: int = 1, n_lgn: int = 512,
                  m: int = 20, width: int = 64, height: int = 64, nt: int = 8000,
                  orient: float = 0.0, contrast: float = 0.5, far_partners: int = 0,
                  adex_inh: bool = False, patch_deg: float = 2.0, nFrame: int = 120,
                  wFF: float = 0.2, wE: float = 0.004, wI: float = 0.6, wFar: float = 0.002,
                  noisyDep=(0.0, 0.0), synFail=(0.0, 0.0, 0.0, 0.0), synFailFF=(0.0, 0.0),
                  mSample1D: int = 16, dt: float = 0.125, tjitter: float = 0.0,
                  noDelay: int = 1, n_parvo: int = 0, tau: float | None = None,
                  nKernelSample: int | None = None, blockSize: int = 1024, nE: int = 768,
                  m_min: int | None = None, flat_retina: bool = True, spE0=None, spI0=None,
                  SCsplit: int = 0, nChunk: int = 1, contra: bool = False, host_init=None) -> Workload:
    """Builds one synthetic patch; C1 = 1x1024 V1 / 512 LGN; C2 = 32 blocks / 16384 LGN.
    noDelay = 0: near synapses are delivered after their distance delay (delayMat from the
    neuron positions, mm, at speedOfThought 1 mm/ms).  spE0/spI0: initial spike rates in Hz
    ([type][2] flattened, as in the cfg), converted to per-step chances as
    src/patch.cu:810-837 does.  host_init: the function that draws the initial state (default
    model.host_init_state, the library's; the oracle's restatement gives the same arrays)."""
    rng = np.random.default_rng(seed)
    spec = make_spec(nblock, blockSize=blockSize, nE=nE, adex_inh=adex_inh, noisyDep=noisyDep,
                     synFail=synFail, synFailFF=synFailFF, dt=dt)
    lgn, extent = make_lgn(n_lgn, rng, patch_deg, dt, mSample1D=mSample1D, tjitter=tjitter,
                           n_parvo=n_parvo, tau=tau, nKernelSample=nKernelSample, flat_retina=flat_retina,
                           contra=contra)
    side = 0.5
    pos, nbx = block_positions(nblock, spec.blockSize, side, rng)
    conMat = near_conmat(spec, pos, rng, sigma=0.1, nE_partners=100, nI_partners=50,
                         wE=wE, wI=wI, side_mm=side)
    if far_partners > 0 and nblock > 1:
        nVec, vecID, conVec, delayVec = far_vectors(spec, pos, rng, far_partners, 0.3,
                                                    wE=wFar, wI=4 * wFar, side_mm=side, nbx=nbx)
    else:
        nVec = np.zeros(spec.nV1, u32)
        vecID, conVec, delayVec = np.zeros(0, u32), np.zeros(0, f32), np.zeros(0, f32)
    nLGNperV1, lgnId, sLGN, rfc, rfo = lgn_to_v1(spec, lgn, rng, m, wFF, patch_deg)
    if m_min is not None:   # ragged LGN lists: m_min..m synapses per neuron (rows past the count unused)
        nLGNperV1 = rng.integers(m_min, m + 1, size=spec.nV1).astype(u32)
    tonic = np.where(spec.type_of(np.arange(spec.nV1) % spec.blockSize) == 0,
                     rng.uniform(0.3, 0.6, spec.nV1), rng.uniform(0.4, 0.7, spec.nV1)).astype(f32)
    nbId = np.arange(nblock, dtype=u32)[:, None].copy()
    delayMat = near_distances(spec, pos, np.ones(nblock, u32), nbId) if not noDelay else None
    if not noDelay:
        spec.noDelay = 0
    net = V1Network(nLGNperV1=nLGNperV1, lgnId=lgnId, sLGN=sLGN,
                    nNearNB=np.ones(nblock, u32), nbId=nbId,
                    conMat=conMat, nVec=nVec, vecID=vecID, conVec=conVec, delayVec=delayVec,
                    tonicDep=tonic, delayMat=delayMat)
    frames = grating_frames(nFrame, width, height, extent, cpd=4.0, tf_hz=8.0,
                            contrast=contrast, orient=orient, frame_rate=120)
    stim = Stimulus(frames=frames, init_LMS=(0.5, 0.5, 0.5))
    # seed sequence of src/patch.cu: logRand_init(seed), per-neuron host engines, init, spInit
    s_lgn = seed
    s_init = seed + 1 + spec.nV1
    s_sp = s_init + 1
    gFF0 = np.tile([0.01, 0.2, 0.0, 0.2], spec.nType * spec.ngFF).astype(f32)
    gE0 = np.tile([0.005, 0.2, 0.0, 0.2], spec.nType * spec.ngE).astype(f32)
    gI0 = np.tile([0.01, 0.2, 0.0, 0.2], spec.nType * spec.ngI).astype(f32)
    w0 = np.tile([0.0, 0.0], spec.nType).astype(f32)
    init = (host_init or host_init_state)(spec, s_init, tonic, nLGNperV1, None, w0, gFF0, gE0, gI0)
    max_delay = float(delayVec.max()) if delayVec.size else 0.0
    trainDepth = int(math.ceil(max(max_delay, 0.0) / spec.speedOfThought / spec.dt)) + 1
    if delayMat is not None:   # the near spike-word ring (src/patch.cu:3808-3813)
        conn = conMat != 0
        maxd = float(delayMat[conn].max()) if conn.any() else 0.0
        trainDepth = max(trainDepth, int(math.ceil(f32(f32(maxd) / f32(spec.speedOfThought)) / f32(spec.dt))) + 1)
    sp0 = None
    if spE0 is not None or spI0 is not None:
        nTE, nTI = spec.nTypeE, spec.nType - spec.nTypeE
        rates = list(spE0 if spE0 is not None else [0.0] * 2 * nTE) + list(spI0 if spI0 is not None else [0.0] * 2 * nTI)
        sp0 = tuple(sp0_chances(rates, spec.dt))
    seeds = Seeds(lgn=s_lgn, cond=s_sp, trainDepth=max(trainDepth, 2), sp0=sp0, SCsplit=SCsplit, nChunk=nChunk)
    return Workload(name=name, spec=spec, net=net, lgn=lgn, stim=stim, init=init, seeds=seeds,
                    nt=nt, pos=pos, rf_center=rfc, rf_orient=rfo)


def sp0_chances(rates_hz, dt: float) -> list:
    """Per-step initial spike chances: each float rate times dt/1000 evaluated in double and
    stored as float (src/patch.cu:820, 834)."""
    d = float(f32(dt)) / 1000.0
    return [float(f32(float(f32(r)) * d)) for r in rates_hz]


def config1(seed: int = 0, **kw) -> Workload:
    """1 block of 1024 V1 neurons (768 E / 256 I), 512 LGN, 64x64 frames, 1 s at 0.125 ms."""
    return make_workload("C1: 1x1024 V1, 512 LGN, 64x64 grating", seed=seed, nblock=1,
                         n_lgn=512, m=20, width=64, height=64, nt=8000, **kw)


def config2(seed: int = 0, orient: float = 0.0, **kw) -> Workload:
    """32 blocks x 1024 = 32768 V1 (80% LIF E / 20% AdEx I), 16384 LGN, 128x128 frames,
    ~400 far partners per neuron, 2 s at 0.125 ms."""
    return make_workload("C2: 32x1024 V1, 16384 LGN, 128x128 grating, 400 far partners",
                         seed=seed, nblock=32, n_lgn=16384, m=20, width=128, height=128,
                         nt=16000, orient=orient, far_partners=400, adex_inh=True,
                         patch_deg=4.0, nFrame=240, **kw)


def write_reference_files(wl: Workload, folder: str, seed: int = 0, nt: int | None = None,
                          extra: dict | None = None, v1_visual: bool = False) -> str:
    """Writes a workload as the reference's input files plus a patchV1 cfg; returns the cfg
    path.  The within-block distances of the near tiles go to V1_delayMat, a per-neuron
    feed-forward ratio to conStats (the tonic drive is then derived from it by the reader,
    CmoreDep = true), and the LGN cells to LGN_vpos + LGN (useNewLGN = false).  v1_visual: the
    V1 RF centres follow the physical positions in V1_allpos (visual-field V1 frames)."""
    import os
    from . import formats as FM
    from .cfg import write_cfg
    os.makedirs(folder, exist_ok=True)
    spec, net, lgn = wl.spec, wl.net, wl.lgn
    d = folder.rstrip("/") + "/"
    bs, nb = spec.blockSize, spec.nblock
    FM.write_connectome_cfg(d + "connectome_cfg.bin", spec.nType, spec.nType - spec.nTypeE,
                            spec.typeAcc)
    FM.write_v1_allpos(d + "V1_allpos.bin", nb, bs, wl.pos, vpos=wl.rf_center if v1_visual else None)
    FM.write_mat(d + "V1_conMat.bin", net.nnb, net.conMat)
    delay = net.delayMat if net.delayMat is not None else near_distances(spec, wl.pos, net.nNearNB, net.nbId)
    FM.write_mat(d + "V1_delayMat.bin", net.nnb, delay)
    FM.write_neighbor_block(d + "neighborBlock.bin", net.nNearNB,
                            [net.nbId[b, :int(net.nNearNB[b])] for b in range(nb)])
    rng = np.random.default_rng(seed + 12345)
    FM.write_con_stats(d + "conStats.bin", spec.nType, rng.uniform(0.2, 0.9, spec.nV1).astype(f32))
    FM.write_v1_vec(d + "V1_vec.bin", net.nVec, net.vecID, net.conVec, net.delayVec)
    ids = [net.lgnId[:int(net.nLGNperV1[i]), i] for i in range(spec.nV1)]
    ss = [net.sLGN[:int(net.nLGNperV1[i]), i] for i in range(spec.nV1)]
    FM.write_list_of_lists(d + "LGN_V1_idList.bin", ids, u32)
    FM.write_list_of_lists(d + "LGN_V1_sList.bin", ss, f32, with_max=True)
    buffer_deg = 0.2
    max_ecc = float(np.max(np.hypot(lgn.xy[:, 0], lgn.xy[:, 1])))
    patch = float(np.max(np.abs(lgn.xy))) * 2
    stim_range = max(max_ecc, patch / 2) * 1.05
    FM.write_stimulus(d + "stimulus.bin", wl.stim.frames, wl.stim.init_LMS,
                      domain=(buffer_deg, stim_range), neye=1 if lgn.flat_retina else 2)
    FM.write_lgn_vpos(d + "LGN_vpos.bin", lgn.nParvo_I + lgn.nMagno_I, lgn.nParvo_C + lgn.nMagno_C, max_ecc,
                      lgn.xy[:, 0].astype(f32), lgn.xy[:, 1].astype(f32), lgn.types)
    lp = {k: getattr(lgn, k) for k in FM.LGN_FIELDS2 + FM.LGN_FIELDS1 + ("coneType",)}
    if lgn.covariant is not None:
        lp["covariant"] = lgn.covariant
    FM.write_lgn_params(d + "LGN", lgn.types, lp)
    s = lgn.sched
    keys = dict(
        inputFolder=d, resourceFolder=d, outputFolder=d, seed=seed, dt=spec.dt,
        nt=wl.nt if nt is None else nt, frameRate=s.frameRate, tau=s.nRetrace * spec.dt,
        mau=s.mRetrace * spec.dt, nKernelSample=s.nKernelSample, mKernelSample=s.mKernelSample,
        mSpatialSample1D=lgn.mSample1D, nSpatialSample1D=lgn.nSample1D or 32, nsig=lgn.nsig,
        convolRatio=lgn.convolRatio,
        frRatioLGN=lgn.frRatio, flat_retina=bool(lgn.flat_retina), useNewLGN=False, learning=0,
        nTypeHierarchy=[spec.nTypeE, spec.nType - spec.nTypeE], sRatioLGN=[1.0],
        sRatioV1=[1.0], synPerCon=spec.synPerCon, synPerConFF=spec.synPerConFF,
        riseTimeFF=spec.riseFF, decayTimeFF=spec.decayFF, riseTimeE=spec.riseE,
        decayTimeE=spec.decayE, riseTimeI=spec.riseI, decayTimeI=spec.decayI,
        pFF=spec.pFF, pE=spec.pE, pI=spec.pI,
        gFF0=[0.01, 0.2, 0.0, 0.2] * (spec.nType * spec.ngFF),
        gE0=[0.005, 0.2, 0.0, 0.2] * (spec.nType * spec.ngE),
        gI0=[0.01, 0.2, 0.0, 0.2] * (spec.nType * spec.ngI),
        w0=[0.0, 0.0] * spec.nType, v0=[-60.0, 1.0] * spec.nType,
        iModel=spec.iModel, noDelay=spec.noDelay, noFarDelay=spec.noFarDelay,
        speedOfThought=spec.speedOfThought, tonicDep=[0.6, 0.7], minTonicRatio=[0.5, 0.5],
        CmoreDep=True, noisyDep=spec.noisyDep, tau_noise=spec.tau_noise,
        noiseOnTonic=spec.noiseOnTonic, synFail=spec.synFail, synFailFF=spec.synFailFF,
        vR=spec.vR, vThres=spec.vThres, gL=spec.gL, C=spec.C, tRef=spec.tRef, vT=spec.vT,
        deltaT=spec.deltaT, tau_w=spec.tau_w, a=spec.a, b=spec.b, hWrite=spec.hWrite,
        spE0=[0.0, 0.0], spI0=[0.0, 0.0], getLGN_sp=True, saveLGN_fr=True, rawData=True,
        readFeature=False)
    keys.update(extra or {})
    fn = d + "patchV1.cfg"
    with open(fn, "w") as f:
        f.write("# synthetic patch written by visual_cortex_gb300.synth\n" + write_cfg(keys))
    return fn


@dataclass
class Trial:
    wl: Workload          # the trial's full workload (network shared with the other trials)
    steps: int
    orient: float
    contrast: float


def batch_trials(n_trials: int = 64, seed: int = 0, nblock: int = 8, n_lgn: int = 4096,
                 width: int = 128, height: int = 128, nFrame: int = 120, n_ori: int = 12,
                 dur_ms=(250.0, 2000.0), contrast=(0.1, 1.0), far_partners: int = 400,
                 patch_deg: float = 2.0, base: Workload | None = None) -> list[Trial]:
    """Batched sweep: n_trials instances of one nblock x 1024 patch (the recipe of the 32-block
    patch), orientation (i mod n_ori) * pi / n_ori, contrast and duration uniform in the given
    ranges, each trial with its own seeds for the LGN generators, the V1 generators and the
    initial state."""
    rng = np.random.default_rng(seed + 777)
    if base is None:
        base = make_workload("batch base", seed=seed, nblock=nblock, n_lgn=n_lgn, m=20,
                             width=width, height=height, nt=0, far_partners=far_partners,
                             adex_inh=True, patch_deg=patch_deg, nFrame=nFrame)
    spec, net, lgn = base.spec, base.net, base.lgn
    extent = 2 * (max(float(np.max(np.hypot(lgn.xy[:, 0], lgn.xy[:, 1]))),
                      float(np.max(np.abs(lgn.xy)))) * 1.05 + 0.2)
    out = []
    for q in range(n_trials):
        ori = (q % n_ori) * math.pi / n_ori
        c = float(rng.uniform(*contrast))
        steps = int(round(float(rng.uniform(*dur_ms)) / spec.dt))
        frames = grating_frames(base.stim.frames.shape[0], base.stim.frames.shape[3],
                                base.stim.frames.shape[2], extent, cpd=4.0, tf_hz=8.0,
                                contrast=c, orient=ori, frame_rate=120)
        s = seed + 1000 * (q + 1)
        s_init = s + 1 + spec.nV1
        gFF0 = np.tile([0.01, 0.2, 0.0, 0.2], spec.nType * spec.ngFF).astype(f32)
        gE0 = np.tile([0.005, 0.2, 0.0, 0.2], spec.nType * spec.ngE).astype(f32)
        gI0 = np.tile([0.01, 0.2, 0.0, 0.2], spec.nType * spec.ngI).astype(f32)
        w0 = np.zeros(2 * spec.nType, f32)
        init = host_init_state(spec, s_init, net.tonicDep, net.nLGNperV1, None, w0, gFF0, gE0, gI0)
        wl = Workload(name=f"trial {q}", spec=spec, net=net, lgn=lgn,
                      stim=Stimulus(frames=frames, init_LMS=(0.5, 0.5, 0.5)), init=init,
                      seeds=Seeds(lgn=s, cond=s_init + 1, trainDepth=base.seeds.trainDepth),
                      nt=steps, pos=base.pos, rf_center=base.rf_center, rf_orient=base.rf_orient)
        out.append(Trial(wl=wl, steps=steps, orient=ori, contrast=c))
    return out
