"""FP64 LGN rates of the BF16 tensor-core workload -- TEST INFRASTRUCTURE (the checker of the
BF16 and FP32 forms of visual_cortex_gb300/lgn_bf16.py, used by tests/ and bench.py's error
report), not part of the product.

The rates follow the same stages as the product's kernels, evaluated in float64 with numpy:
the DoG footprint of each cell over the frame's contrast (clipped to [-1, 1], as
src/discrete_input_convol.cu:1342-1585 clips it), the frame weights of the step's window, and
the logistic rate of LGN_nonlinear (src/discrete_input_convol.cu:1637-1821).
"""
from __future__ import annotations

import numpy as np

from visual_cortex_gb300.lgn_bf16 import PAD, TILE_K, TILE_N, LgnWorkload


def spatial64(wl: LgnWorkload, cells: np.ndarray) -> np.ndarray:
    """FP64 spatial stage of the given cells: [len(cells)][nFext] (column = frame + PAD)."""
    half = wl.side // 2
    nF = wl.frames.shape[0]
    contrast = np.clip(wl.frames.astype(np.float64) / wl.meanLum - 1.0, -1.0, 1.0)
    out = np.zeros((len(cells), wl.nFext))
    d = np.arange(wl.side) - half
    for r, c in enumerate(cells):
        ys = wl.cy[c] + d
        xs = wl.cx[c] + d
        patch = contrast[:, ys[:, None], xs[None, :]].reshape(nF, -1)   # [nF][side*side]
        s = patch @ wl.SW[c].astype(np.float64)
        cols = np.arange(PAD, wl.nFext)
        out[r, PAD:] = s[(cols - PAD) % nF]
    return out


def oracle_rates(wl: LgnWorkload, cells: np.ndarray, steps: np.ndarray) -> np.ndarray:
    """FP64 LGN rates [len(steps)][len(cells)] of the same workload (spatial stage, frame
    weights, logistic rate) for the error report of the BF16 and FP32 paths."""
    S = spatial64(wl, cells)                                   # [cells][nFext]
    out = np.empty((len(steps), len(cells)))
    for q, t in enumerate(steps):
        i, s = divmod(int(t), TILE_N)
        cols = wl.f0[i] + np.arange(TILE_K)
        ok = cols < wl.nFext
        conv = S[:, cols[ok]] @ wl.W[i, s][ok]                 # FP64 weights of the window
        cur = np.maximum(conv * np.abs(wl.k[cells]).astype(np.float64) * wl.convolRatio, 0.0)
        mx = wl.maxConvol[cells].astype(np.float64)
        X = 1.0 / (1.0 + np.exp(wl.sharp[cells] * (wl.c50[cells] - cur / mx)))
        out[q] = wl.frRatio * mx * (wl.la[cells] * X + wl.lb[cells])
    return out


def rate_errors(fr: np.ndarray, ref: np.ndarray) -> dict:
    rel = np.abs(fr.astype(np.float64) - ref) / np.abs(ref)
    return {"max_rel": float(rel.max()), "rms_rel": float(np.sqrt(np.mean(rel ** 2))),
            "mean_rate_hz": float(ref.mean())}
