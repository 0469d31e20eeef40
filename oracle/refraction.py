"""CPU restatement of the reference's atmospheric-refraction ray trace
(AtmosphereModel_RefractionPath, src/AtmosphereModel/AtmosphereModel.c:4215-4291).

TEST INFRASTRUCTURE ONLY: the checker of atmwfs_refraction_path and
atmwfs_refraction_table; no product code path imports it.  Pure-Python FP64
loops (one ray is a few thousand 20 m steps per pass)."""
from __future__ import annotations

import math

import numpy as np


def _f32(v: float) -> float:
    """The float argument of the reference's model calls."""
    return float(np.float32(v))


def refraction_path(lam, zangle, site, N, K=None, path_lines=None):
    """Refraction [arcsec] and transmission of the last pass; N(alt, lam) and
    K(alt, lam) are the model (the reference calls its model with float
    altitude and wavelength).  path_lines (a list) receives the last pass's
    (h, x, y, alpha) rows."""
    Lstep, Re = 20.0, 6371000.0
    Z0 = zangle
    it, errV, flux = 0, 100000.0, 1.0
    alpha = Z0
    while it < 20 and errV > 0.00001:
        x0 = y0 = 0.0
        alpha = Z0
        n0 = 1.0 + N(_f32(site), _f32(lam))
        h1 = 0.0
        flux = 1.0
        rows = []
        while h1 < 99000.0:
            x1 = x0 + Lstep * math.sin(alpha)
            y1 = y0 + Lstep * math.cos(alpha)
            h1 = math.sqrt(x1 * x1 + (y1 + site + Re) * (y1 + site + Re)) - Re
            n1 = 1.0 + N(_f32(h1), _f32(lam))
            ae = math.atan2(x1, y1 + site + Re)
            flux *= math.exp(-Lstep * (K(_f32(h1), _f32(lam)) if K else 0.0))
            a0 = alpha - ae
            alpha = math.asin(n0 * math.sin(a0) / n1) + ae
            n0, x0, y0 = n1, x1, y1
            rows.append((h1, x0, y0, alpha))
        off = alpha - zangle
        Z0 -= off
        errV = abs(off / math.pi * 180.0 * 3600.0)
        it += 1
        if path_lines is not None:
            path_lines[:] = rows
    return (zangle - Z0) / math.pi * 180.0 * 3600.0, flux
