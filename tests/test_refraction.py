"""Atmospheric refraction (AtmosphereModel_RefractionPath,
AtmosphereModel.c:4215-4291) on the CPU: the oracle's restatement
(oracle/refraction.py) and the library's host ray trace
(atmwfs_refraction_path) against the reference's own results
(tests/golden/refract.npz: the reference's ray trace with its atmosphere
model, and that model's N and absorption at the 10 m nodes of its density
tables, which a table model reads back with the reference's interpolation).

Tolerances: the table model equals the reference's model at the nodes and
interpolates N linearly between them where the reference interpolates the
gas densities (N is linear in them to 1e-8 relative), so refraction agrees
to 1e-4 arcsec; the library's trace and the oracle run the same FP64
statements on the same model and agree to 1e-9 arcsec."""
import numpy as np
import pytest

import golden_case as gcm
from oracle import refraction as orf

G = np.load(gcm.GOLDEN / "refract.npz")
DH = float(G["table"][0])


def _model(k):
    from atmosphericturbulencesimul_gb300.mkwfs import table_model
    return table_model(G[f"N{k}"], G[f"K{k}"], DH)


@pytest.mark.parametrize("k", range(3))
def test_oracle_matches_reference(lib, k):
    lam, za, site, ref, tr = G[f"case{k}"]
    N, K = _model(k)
    r, t = orf.refraction_path(lam, za, site, N, K)
    assert abs(r - ref) < 1e-4, (r, ref)
    assert abs(t - tr) < 1e-12


@pytest.mark.parametrize("k", range(3))
def test_library_host_trace_matches_reference_and_oracle(lib, k):
    from atmosphericturbulencesimul_gb300.mkwfs import refraction_path
    lam, za, site, ref, tr = G[f"case{k}"]
    N, K = _model(k)
    r, t = refraction_path(lam, za, site, N, K)
    assert abs(r - ref) < 1e-4, (r, ref)
    assert abs(t - tr) < 1e-12
    ro, _ = orf.refraction_path(lam, za, site, N, K)
    assert abs(r - ro) < 1e-9


def test_path_file_matches_reference(lib, tmp_path):
    """The last pass's path, refractpath.txt: same number of 20 m steps, the
    same altitudes and positions to the printed millimetre, angles to 1e-8."""
    from atmosphericturbulencesimul_gb300.mkwfs import refraction_path
    lam, za, site, ref, tr = G["case0"]
    N, K = _model(0)
    refraction_path(lam, za, site, N, K, path_file=tmp_path / "p.txt")
    got = np.loadtxt(tmp_path / "p.txt")
    want = np.array([l.split() for l in str(G["path0"]).splitlines()], float)
    assert got.shape == want.shape
    assert np.abs(got[:, :3] - want[:, :3]).max() <= 1.5e-3
    assert np.abs(got[:, 3] - want[:, 3]).max() < 1e-8


def test_absorption_and_errors(lib):
    """A made-up absorption profile: transmission exp(-sum 20 m K(h)) as in
    the oracle; a zenith angle at or past the horizon is refused."""
    from atmosphericturbulencesimul_gb300 import _lib
    from atmosphericturbulencesimul_gb300.mkwfs import refraction_path
    N, _ = _model(0)
    K = lambda alt, lam: 1e-6 * np.exp(-max(float(alt), 0.0) / 8000.0)
    r, t = refraction_path(0.7e-6, 0.3, 0.0, N, K)
    ro, to = orf.refraction_path(0.7e-6, 0.3, 0.0, N, K)
    assert abs(r - ro) < 1e-9 and abs(t - to) < 1e-12
    assert 0.9 < t < 1.0
    with pytest.raises(_lib.AtmwfsError):
        refraction_path(0.7e-6, np.pi / 2, 0.0, N)


def test_host_table_form_matches_reference(lib):
    """atmwfs_refraction_table_host: the table model traced on host threads."""
    from atmosphericturbulencesimul_gb300.mkwfs import refraction_table
    for k in range(3):
        lam, za, site, ref, tr = G[f"case{k}"]
        r, t = refraction_table([lam], [za, 0.2], site, G[f"N{k}"][None], G[f"K{k}"][None], DH, host_threads=2)
        assert abs(r[0, 0] - ref) < 1e-4 and abs(t[0, 0] - tr) < 1e-12
        assert 0 < r[0, 1] < r[0, 0]
