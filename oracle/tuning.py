"""Firing-rate and orientation-tuning statistics of a V1 raster -- TEST INFRASTRUCTURE.

Restated from the reference's analysis scripts so that long runs of the library and of the
oracle can be compared on the quantities the reference reports:

* F1/F0 (src/plotV1_response.py:887-958): a neuron's spike times folded by the stimulus
  period tTF into TFbins bins, the histogram divided by (stacks * bin width) as a rate; F0 is
  its mean, F1 twice the modulus of its first Fourier component (get_FreqComp), F1/F0 their
  ratio (0 where F0 = 0).
* gOSI (src/getTuningCurve.py:1709-1719): |sum_k r_k exp(2 pi i k / nOri)| / sum_k r_k over
  the nOri orientations.
* OSI of the aligned tuning curve (src/getTuningCurve.py:1087-1126, 1721-1731).
* the von Mises fit b + a exp(s (cos 2(theta - theta0) - 1)) with its gOSI integral
  (src/getTuningCurve.py:301-421), scipy's curve_fit as the reference uses it.
"""
from __future__ import annotations

import numpy as np


def spike_times(sInfo: np.ndarray, dt: float, step0: int = 0):
    """Per neuron, the spike times (ms) of a spike-word raster [steps][nV1] (sInfo >= 1:
    nsp + tsp/dt, every spike of the step at its mean time)."""
    steps, n = sInfo.shape
    out = [[] for _ in range(n)]
    t, i = np.nonzero(sInfo >= 1)
    w = sInfo[t, i].astype(np.float64)
    nsp = np.floor(w)
    ts = (t + step0 + (w - nsp)) * dt
    for tt, ii, k in zip(ts, i, nsp.astype(int)):
        out[ii].extend([tt] * k)
    return out


def rates(sInfo: np.ndarray, dt: float) -> np.ndarray:
    """Spikes per second of each neuron over the raster."""
    w = np.where(sInfo >= 1, np.floor(sInfo), 0.0)
    return w.sum(axis=0) / (sInfo.shape[0] * dt * 1e-3)


def _freq_comp(data: np.ndarray, ifreq: int):
    nd = data.shape[-1]
    f = np.sum(data * np.exp(-2j * np.pi * ifreq * np.arange(nd) / nd), axis=-1) / nd
    return np.abs(f) * 2, np.angle(f, deg=True)


def f1f0(sp_times, duration_ms: float, tTF: float, TFbins: int):
    """F0, F1 and F1/F0 per neuron (rates in Hz), the reference's folding with stacks =
    duration / tTF periods."""
    n = len(sp_times)
    dtTF = tTF / TFbins
    edges = np.arange(TFbins + 1) * dtTF
    stacks = duration_ms / tTF
    F0 = np.zeros(n)
    F1 = np.zeros(n)
    for i, ts in enumerate(sp_times):
        if len(ts) == 0:
            continue
        tsp = np.mod(np.asarray(ts), tTF)
        nsp = np.histogram(tsp, bins=edges)[0] / (stacks * dtTF / 1000)
        F0[i] = nsp.mean()
        F1[i] = _freq_comp(nsp, 1)[0]
    ratio = np.zeros(n)
    pos = F0 > 0
    ratio[pos] = F1[pos] / F0[pos]
    return F0, F1, ratio


def gosi(fr: np.ndarray) -> np.ndarray:
    """Global OSI of tuning curves fr [nOri][nV1]."""
    nOri = fr.shape[0]
    theta = np.exp(1j * np.arange(nOri) / nOri * 2 * np.pi)
    out = np.zeros(fr.shape[1])
    pick = fr.max(axis=0) > 0
    out[pick] = np.abs((fr.T * theta).sum(axis=1)[pick]) / fr.T.sum(axis=1)[pick]
    return out


def aligned_osi(fr: np.ndarray):
    """(preferred orientation index, OSI) from tuning curves fr [nOri][nV1]: each curve rolled
    so its maximum sits at the middle position, the wrap-around point appended, OSI = (max -
    min) / (max + min) of the aligned curve."""
    nOri, n = fr.shape
    pref = np.argmax(fr, axis=0)
    mid = nOri // 2 if nOri % 2 == 0 else (nOri - 1) // 2
    idx = (np.arange(nOri)[None, :] + pref[:, None] - mid) % nOri
    idx = np.concatenate([idx, idx[:, :1]], axis=1)
    aligned = np.take_along_axis(fr.T, idx, axis=1)
    tmin, tmax = aligned[:, 0], aligned[:, mid]
    osi = np.zeros(n)
    pick = tmax > 0
    osi[pick] = (tmax[pick] - tmin[pick]) / (tmin[pick] + tmax[pick])
    return pref, osi


def von_mises_gosi(fr: np.ndarray, pref: np.ndarray):
    """The von Mises fit of each tuning curve and its gOSI (fit_gOSI of the reference)."""
    from scipy import integrate, optimize, special
    nOri, n = fr.shape
    theta = (np.arange(nOri) + 1) / nOri * np.pi

    def vm(th, a, b, s, th0):
        return b + a * np.exp(s * (np.cos(2 * (th - th0)) - 1))

    def vm0(th, a, s, th0):
        return a * np.exp(s * (np.cos(2 * (th - th0)) - 1))

    out = np.zeros(n)
    for i in range(n):
        q = fr[:, i]
        mx, mn = q.max(), q.min()
        if not mx > mn:
            continue
        iq, mn2 = 1, mn
        while mn2 == mn and iq < nOri:
            mn2 = np.partition(q, iq)[iq]
            iq += 1
        avg_min = (mn + mn2) / 2
        s0 = (np.log(mx - mn) - np.log(avg_min - mn)) / 2 if avg_min > mn else 1.0
        a0 = (mx - avg_min) / (1 - np.exp(-2 * s0))
        b0 = mx - a0
        if nOri % 2 == 0:
            th0 = pref[i] / nOri * np.pi
        else:
            nxt, prv = (pref[i] + 1) % nOri, (pref[i] + nOri - 1) % nOri
            th0 = (pref[i] + (prv if q[prv] > q[nxt] else nxt)) / 2 * np.pi
        try:
            if b0 < 0:
                b = 0.0
                (a, s, _), _ = optimize.curve_fit(vm0, theta, q, p0=[mx, s0, th0],
                                                  bounds=([0, 0, 0], [2 * mx, np.inf, np.pi]))
            else:
                (a, b, s, _), _ = optimize.curve_fit(vm, theta, q, p0=[a0, b0, s0, th0],
                                                     bounds=([0, 0, 0, 0], [2 * a0, mx, np.inf, np.pi]))
        except (RuntimeError, ValueError):
            a, b, s = max(a0, 0.0), max(b0, 0.0), 1.0
        integ = (integrate.quad(lambda x: np.exp(s * np.sqrt(1 - x * x)), 0, 1)[0]
                 - integrate.quad(lambda x: np.exp(-s * np.sqrt(1 - x * x)), 0, 1)[0])
        out[i] = integ / (b + 2 * a * special.i0(s)) * np.pi
    return out
