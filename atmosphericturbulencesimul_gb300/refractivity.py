"""Air refractivity for the chromatic phase scaling of the series.

The reference scales the reference-wavelength phase of each layer to the
science wavelength by Scoeff = (lambda_ref / lambda) * N(h, lambda) / N(h, lambda_ref)
(src/AtmosphericTurbulence/AtmosphericTurbulence.c:2661-2663), with N = n - 1
from its NRLMSISE-00 density table and a per-gas Lorentz-Lorenz sum
(AtmosphereModel.c:3212-3300).  For a fixed gas mixture N is proportional to
density, so the ratio depends on the dispersion only.  This module uses the
published standard-air dispersion of Ciddor (Appl. Opt. 35, 1566, 1996,
eq. 1 with the CO2 correction of eq. 2); a caller holding the reference's
own atmosphere model passes its Scoeff values through the C ABI instead.
"""
from __future__ import annotations

import numpy as np

# Ciddor (1996) eq. 1 constants, sigma in 1/um
_K0, _K1, _K2, _K3 = 238.0185, 5792105.0, 57.362, 167917.0


def n_minus_1_std_air(lam_m, co2_ppm: float = 450.0):
    """Refractivity (n - 1) of standard dry air (15 C, 101325 Pa) at vacuum wavelength lam [m]."""
    sigma2 = (1.0 / (np.asarray(lam_m, dtype=np.float64) * 1e6)) ** 2
    nas = 1e-8 * (_K1 / (_K0 - sigma2) + _K3 / (_K2 - sigma2))
    return nas * (1.0 + 0.534e-6 * (co2_ppm - 450.0))


def scoeff(lam_ref: float, lam: float, nlayers: int) -> np.ndarray:
    """Per-layer phase multiplier from lam_ref to lam (float32, like the reference's operands)."""
    lr = np.float32(lam_ref)
    n_l = np.float32(n_minus_1_std_air(lam))
    n_r = np.float32(n_minus_1_std_air(float(lr)))
    v = float(lr) / float(lam) * float(n_l) / float(n_r)
    return np.full(nlayers, v, dtype=np.float32)


def n_air(alt_m, lam_m, scale_height: float = 8000.0):
    """Refractive index of dry standard air at altitude alt [m]: the Ciddor
    refractivity scaled by an exponential density profile (the host driver's
    default model)."""
    return 1.0 + n_minus_1_std_air(lam_m) * np.exp(-np.asarray(alt_m, dtype=np.float64) / scale_height)


def hop_air_index(alt, cn2, fresnel_bin: float, lam: float, model=None, amplitude: int = 1, fresnel: int = 1,
                  zangle: float = 0.0) -> np.ndarray:
    """Air index of every propagation hop of a profile (the optional lambda / n
    hops of atmwfs_instance.hop_n), in the engine's hop order: n at the
    middle of the hop between the altitudes of its two super-layers.
    model(alt, lam) -> n defaults to n_air."""
    from .engine import layer_planes
    salt, sidx, planes, _ = layer_planes(alt, cn2, fresnel_bin, amplitude, fresnel, zangle)
    model = model or n_air
    mids = [0.5 * (salt[sidx[planes[h][0]]] + salt[sidx[planes[h + 1][0]]]) for h in range(len(planes) - 1)]
    return np.array([float(model(m, lam)) for m in mids], np.float64)
