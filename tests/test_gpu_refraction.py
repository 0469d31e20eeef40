"""Refraction ray traces on the GPU (atmwfs_refraction_table: one FP64 ray
per thread, table models) against the reference's results
(tests/golden/refract.npz) and the library's host trace on the same model.

Tolerances: 1e-4 arcsec against the reference (the table model, see
test_refraction.py); 1e-7 arcsec and 1e-12 in transmission against the host
trace (the same FP64 statements; the device's sin/asin/atan2/exp may differ
from the host's in the last place)."""
import numpy as np
import pytest

from test_refraction import DH, G

pytestmark = pytest.mark.gpu


def test_table_matches_reference(lib):
    from atmosphericturbulencesimul_gb300.mkwfs import refraction_table
    for k in range(3):
        lam, za, site, ref, tr = G[f"case{k}"]
        r, t = refraction_table([lam], [za], site, G[f"N{k}"][None], G[f"K{k}"][None], DH, where="gpu")
        assert abs(r[0, 0] - ref) < 1e-4, (k, r, ref)
        assert abs(t[0, 0] - tr) < 1e-12


def test_table_grid_matches_host_trace(lib):
    """Three wavelength tables x 24 zenith angles (0 to 80 degrees) with a
    made-up absorption; a sample of rays against the host trace."""
    from atmosphericturbulencesimul_gb300.mkwfs import refraction_path, refraction_table, table_model
    lams = [G[f"case{k}"][0] for k in range(3)]
    Ntab = np.stack([G[f"N{k}"] for k in range(3)])
    alt = np.arange(Ntab.shape[1]) * DH
    Ktab = np.stack([1e-6 * (1 + k) * np.exp(-alt / 8000.0) for k in range(3)])
    za = np.linspace(0.0, np.deg2rad(80.0), 24)
    r, t = refraction_table(lams, za, 0.0, Ntab, Ktab, DH, where="gpu")
    assert r.shape == (3, 24) and np.all(np.diff(r, axis=1) > 0)     # refraction grows with zenith angle
    assert r[0, 0] == 0.0 and np.all(t <= 1.0)
    for k, z in [(0, 5), (1, 17), (2, 23)]:
        N, K = table_model(Ntab[k], Ktab[k], DH)
        rh, th = refraction_path(lams[k], za[z], 0.0, N, K)
        assert abs(r[k, z] - rh) < 1e-7, (k, z, r[k, z], rh)
        assert abs(t[k, z] - th) < 1e-12
