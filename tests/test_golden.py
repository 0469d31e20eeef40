"""The oracle pinned to the reference's own outputs (tests/golden/, written by
the reference's code built from its sources with shims for FFTW, cfitsio
and the noise; see tests/golden/make_golden.py).

Tolerances (FP64 oracle vs the reference's FP32 arrays):
  * master-screen synthesis from the same noise: relative max error <= 1e-5;
  * Fresnel hop: relative max error <= 1e-5;
  * series cubes: wrapped phase error <= 1e-3 nm rms and <= 0.01 nm max,
    amplitude error <= 5e-6, no 2 pi jumps, OPD rms and amplitude variance
    within 1e-6 relative.
"""
import numpy as np
import pytest

import golden_case as gcm


@pytest.mark.parametrize("name", gcm.CASES)
def test_master_screens_match_reference(oracle64, oracle32, name):
    gc = gcm.load(name)
    for l in range(len(gc.alt)):
        u, g = oracle64.screen_noise(gc.seed, l, gc.M)
        s, _, _ = oracle32.master_screen(u, g, gc.outer[l] / gc.pupil, gc.inner[l] / gc.pupil)
        ref = gc.screens[l]
        assert np.abs(s - ref).max() / np.abs(ref).max() < 1e-5, l


def test_fresnel_matches_reference(oracle64):
    g = np.load(gcm.GOLDEN / "fresnel.npz")
    for k in range(2):
        n, dx, z, lam = g[f"par{k}"]
        got = oracle64.fresnel(g[f"in{k}"].astype(np.complex128), float(dx), float(z), float(lam))
        ref = g[f"out{k}"]
        assert np.abs(got - ref).max() / np.abs(ref).max() < 1e-5, k


@pytest.mark.parametrize("name", gcm.CASES)
def test_series_matches_reference(oracle64, oracle32, name):
    gc = gcm.load(name)
    got = gcm.run_oracle(gc, oracle64, oracle32)
    gcm.compare(got, gc, dict(wrapped_rms_nm=1e-3, wrapped_max_nm=1e-2, flip_frac=0.0, opd_rms_rel=1e-6,
                              amp_max_err=5e-6, amp_var_rel=1e-6))


def test_golden_cases_cover_the_quirks():
    """The fixtures exercise grouping, crop, zenith angle and source offsets."""
    b = gcm.load("mkwfs_b")
    assert b.Wout < b.W and b.zangle > 0 and b.src != (0.0, 0.0)
    assert np.diff(b.alt).min() < b.fbin          # two layers share a super-layer
    assert b.roffset[-1] > 0.01                   # about one pixel of refraction shift
    # the reference's Scoeff grows with altitude (less water vapour aloft)
    assert np.all(np.diff(b.scoeff) > 0)
