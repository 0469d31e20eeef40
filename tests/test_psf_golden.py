"""PSF consumers on the CPU: the oracle (oracle/psf_oracle.c) and the
library's host image measures against the reference's own outputs
(tests/golden/psf.npz, written by the checker build of the reference's
psf.c, image_filter.c and AtmosphericTurbulence.c; see
tests/golden/make_golden.py).

Tolerances: FP64 oracle vs the reference's float arithmetic -- Gaussian
filter 1e-6 relative, chromatic PSF 1e-6 relative, exposure PSFs 1e-5
relative (float FFT in the reference), centres 1e-6 px, FWHM / EE50 1e-5 px;
the library's host measures keep the reference's float types, so the
filtered image is bit-identical and the measures agree to 1e-6 px."""
import re

import numpy as np
import pytest

import golden_case as gcm

G = np.load(gcm.GOLDEN / "psf.npz")


def exposures(etime: float, dt: float, nframes: int, ntspan: int):
    """Frame groups of the reference's exposure loop (float etime_left)."""
    groups, cur, left = [], [], np.float32(etime)
    for t in range(ntspan):
        for f in range(nframes):
            cur.append((t, f))
            left = np.float32(left - np.float32(dt))
            if left < 0:
                groups.append(cur)
                cur, left = [], np.float32(etime)
    return groups, cur


@pytest.mark.parametrize("k", range(3))
def test_oracle_measures_match_reference(oracle64, k):
    im = G[f"meas_in{k}"]
    g = oracle64.gauss_filter(im)
    ref = G[f"meas_gauss{k}"]
    assert np.abs(g - ref).max() / np.abs(ref).max() < 1e-6
    xc, yc, fw, ee = oracle64.psf_measure(im)
    rx, ry, rf, re_ = G[f"meas_val{k}"]
    assert abs(xc - rx) < 1e-6 and abs(yc - ry) < 1e-6
    assert abs(fw - rf) < 1e-5 and abs(ee - re_) < 1e-5


@pytest.mark.parametrize("k", range(3))
def test_library_host_measures_match_reference(lib, k):
    from atmosphericturbulencesimul_gb300 import psf as P
    im = G[f"meas_in{k}"]
    assert np.array_equal(P.gauss_filter(im), G[f"meas_gauss{k}"])
    m = P.measure(im)
    rx, ry, rf, re_ = G[f"meas_val{k}"]
    assert abs(m["xcenter"] - rx) < 1e-6 and abs(m["ycenter"] - ry) < 1e-6
    assert abs(m["fwhm"] - rf) < 1e-6 and abs(m["ee50"] - re_) < 1e-6


def test_measure_quirks(lib):
    """The background of center_PSF is the pixel at index n/2 (the
    reference's float percentile does not sort), the FWHM interpolation
    term is not doubled, and the encircled-energy radius is offset by two
    rings; checked on a Gaussian whose values are known."""
    from atmosphericturbulencesimul_gb300 import psf as P
    n = 64
    y, x = np.mgrid[0:n, 0:n]
    img = np.exp(-((x - 32.0) ** 2 + (y - 32.0) ** 2) / (2 * 4.0 ** 2)).astype(np.float32)
    fw = P.fwhm(img, 32.0, 32.0)
    # rings of width 1: the half-maximum crossing lies between the ring means
    assert 2 * 4.0 * 1.1774 - 2.5 < fw < 2 * 4.0 * 1.1774 + 0.5
    # a bright pixel at index n*n/2 raises the background above the whole
    # Gaussian: no pixel passes, the centre is 0/0
    img2 = img.copy()
    img2.flat[n * n // 2] = 10.0
    xc, yc = P.center(img2)
    assert np.isnan(xc) and np.isnan(yc)


@pytest.mark.parametrize("k", range(2))
def test_oracle_chromatic_psf_matches_reference(oracle64, k):
    n, c1, c2, ns, apo = G[f"chromat_par{k}"]
    out = oracle64.chromat_psf(G[f"chromat_amp{k}"], G[f"chromat_pha{k}"], c1, c2, int(ns), apo)
    ref = G[f"chromat_out{k}"]
    assert np.abs(out - ref).max() / ref.max() < 1e-6


def test_oracle_exposures_match_reference(oracle64):
    etime, dt, W, nframes, ntspan = G["expo_par"]
    W, nframes, ntspan = int(W), int(nframes), int(ntspan)
    groups, rest = exposures(etime, dt, nframes, ntspan)
    pup, pha = G["expo_pupil"], G["expo_pha"]
    assert len(groups) == sum(1 for f in G.files if f.startswith("expo_psf"))
    for k, grp in enumerate(groups):
        psf = oracle64.psf_expo(pup, np.stack([pha[t][f] for t, f in grp]))
        ref = G[f"expo_psf{k}"]
        assert np.abs(psf - ref).max() / ref.max() < 1e-5, k
    last = oracle64.psf_expo(pup, np.stack([pha[t][f] for t, f in rest]))
    assert np.abs(last - G["expo_final"]).max() / G["expo_final"].max() < 1e-5
    # the log lines: exposure index, FWHM and 2 x EE50 (arcsec), centre
    lines = str(G["expo_log"]).splitlines()
    assert len(lines) == len(groups)
    for k, line in enumerate(lines):
        idx, fw, ee2, xc, yc = line.split()
        assert int(idx) == k
        oxc, oyc, ofw, oee = oracle64.psf_measure(G[f"expo_psf{k}"])
        assert abs(oxc - float(xc)) < 1e-5 and abs(oyc - float(yc)) < 1e-5
        assert re.fullmatch(r"-?\d+\.\d{6}", fw)


def test_exposure_grouping_follows_float_time():
    """etime 3 ms at 1 ms steps: float(0.003) - 3 * float(0.001) < 0, so every
    exposure holds three frames, and the groups run across time spans."""
    groups, rest = exposures(0.003, 0.001, 8, 2)
    assert [len(g) for g in groups] == [3] * 5 and len(rest) == 1
    assert groups[2] == [(0, 6), (0, 7), (1, 0)]
