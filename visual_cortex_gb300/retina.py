"""Texture-space geometry of the retina (src/patch.cu:1609-1636)."""
from __future__ import annotations

import math

import numpy as np

DEG = math.pi / 180.0


def retina_geometry(max_ecc: float, stim_range: float, buffer: float, flat: bool) -> dict:
    """Texture-space geometry of src/patch.cu:1609-1636 in single precision: the visual
    centres (L_x0, L_y0), (R_x0, R_y0) and the view distance in texture units.  Flat: one eye,
    the texture spans 2 (range + buffer) deg; curved: two eyes side by side, each range +
    2 buffer deg wide, the view distance such that tan(max_ecc) maps to max_ecc / (2 extent).
    `extent` is the horizontal span of the whole texture (deg)."""
    f = np.float32
    if flat:
        ext = f(2) * (f(stim_range) + f(buffer))
        norm = f(f(max_ecc) / ext)
        nvd = float(f(f(norm / f(max_ecc)) / f(DEG)))
        return dict(extent=float(ext), normViewDistance=nvd, L_x0=0.5, L_y0=0.5, R_x0=1.0, R_y0=1.0)
    ext = f(stim_range) + f(2) * f(buffer)
    norm = f(f(max_ecc) / (f(2) * ext))
    L_x0 = float(f(f(buffer) / (f(2) * ext)))
    nvd = float(f(norm / f(np.tan(f(f(max_ecc) * f(DEG))))))
    return dict(extent=float(f(2) * ext), normViewDistance=nvd, L_x0=L_x0, L_y0=0.5,
                R_x0=float(f(0.5) + f(L_x0)), R_y0=0.5)
