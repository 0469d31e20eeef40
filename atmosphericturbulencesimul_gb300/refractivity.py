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
