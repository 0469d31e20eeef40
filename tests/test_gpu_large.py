"""Large grids on the GPU: the 2-D DFT at 4096^2 and 8192^2 (rows in shared
memory, columns through a transpose), master screens of that size against
the FP64 oracle's synthesis from the same noise, and a series run on
4096^2 screens.

Tolerances (FP32 vs FP64): DFT relative max error <= 2e-5 at 4096 (numpy
reference), round trip and Parseval within 1e-5 at 8192; master screens
relative max error <= 1e-4 and structure-function constants within 1e-4
(the bar of the 256^2 screen test); series frames as the other parity
tests (0.05 nm rms wrapped OPD, 2e-3 amplitude)."""
import numpy as np
import pytest

from series_case import Case

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("sign", [-1, 1])
def test_fft2d_4096_matches_numpy(lib, sign):
    from atmosphericturbulencesimul_gb300 import fft2d
    n = 4096
    rng = np.random.default_rng(40)
    a = (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))).astype(np.complex64)
    got = fft2d(a, sign)
    ref = np.fft.fft2(a.astype(np.complex128)) if sign < 0 else np.fft.ifft2(a.astype(np.complex128)) * n * n
    err = np.abs(got - ref).max() / np.abs(ref).max()
    assert err < 2e-5, err


def test_fft2d_8192_round_trip_and_parseval(lib):
    from atmosphericturbulencesimul_gb300 import fft2d
    n = 8192
    rng = np.random.default_rng(81)
    a = (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))).astype(np.complex64)
    f = fft2d(a, -1)
    e_in = np.sum(np.abs(a.astype(np.complex128)) ** 2)
    assert abs(np.sum(np.abs(f.astype(np.complex128)) ** 2) / (n * n * e_in) - 1) < 1e-5
    # one known coefficient: F[0, 0] is the sum of the input
    s = a.astype(np.complex128).sum()
    assert abs(f[0, 0] - s) / np.sqrt(e_in) < 1e-5
    b = fft2d(f, 1) / np.float32(n * n)
    err = np.abs(b - a).max() / np.abs(a).max()
    assert err < 1e-5, err


@pytest.mark.parametrize("M", [4096, 8192])
def test_master_screen_large_matches_oracle(lib, oracle64, M):
    from atmosphericturbulencesimul_gb300 import master_screen
    g1, g2, gc = master_screen(11, M, 2000.0, 1.0, stream=3)
    u, g = oracle64.screen_noise(11, 3, M)
    o1, o2, oc = oracle64.master_screen(u, g, 2000.0, 1.0)
    del u, g
    assert np.abs(g1 - o1).max() / np.abs(o1).max() < 1e-4
    assert np.abs(g2 - o2).max() / np.abs(o2).max() < 1e-4
    assert np.allclose(gc, oc, rtol=1e-4)
    # the structure function over lags 1..64 follows the oracle's screen
    for s, o in ((g1, o1), (g2, o2)):
        for r in (1, 4, 16, 64):
            dg = np.mean((np.roll(s, -r, 1) - s).astype(np.float64) ** 2)
            do = np.mean((np.roll(o, -r, 1) - o) ** 2)
            assert abs(dg / do - 1) < 1e-3, (r, dg, do)


def test_series_on_4096_screens(lib, oracle64):
    from test_gpu_parity import _compare
    case = Case(alt=[0.0, 3000.0, 10000.0], cn2=[0.5, 0.3, 0.2], speed=[40.0, -60.0, 80.0],
                direction=[0.4, 1.9, 3.7], M=4096, W=256, Wout=256, fresnel_bin=100.0, dt=0.05)
    _compare(case, oracle64, 2)
