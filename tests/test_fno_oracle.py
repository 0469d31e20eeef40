"""The FP64 surrogate oracle (oracle/fno_oracle.py) pinned by finite
differences: its hand-derived gradient matches central differences of its
own loss along random directions, for every parameter tensor."""
import numpy as np
import pytest

from oracle import fno_oracle as fo

CFG = fo.Cfg(nin=3, width=4, modes=4, layers=2, proj=6, nout=2, grid=16)


@pytest.fixture(scope="module")
def case():
    rng = np.random.default_rng(0)
    p = fo.init_params(CFG, 1)
    x = rng.standard_normal((2, CFG.nin, CFG.grid, CFG.grid))
    t = rng.standard_normal((2, CFG.nout, CFG.grid, CFG.grid)) * 0.3
    return p, x, t


def test_gradient_matches_finite_differences(case):
    p, x, t = case
    loss, g = fo.loss_grad(p, x, t, CFG)
    rng = np.random.default_rng(3)
    for name, (o, n) in fo.layout(CFG).items():
        if name == "_total":
            continue
        v = np.zeros_like(p)
        v[o:o + n] = rng.standard_normal(n)
        eps = 1e-5
        lp, _ = fo.loss_grad(p + eps * v, x, t, CFG)
        lm, _ = fo.loss_grad(p - eps * v, x, t, CFG)
        fd = (lp - lm) / (2 * eps)
        an = float(g @ v)
        assert abs(fd - an) <= 1e-6 * max(1.0, abs(fd)), (name, fd, an)


def test_spectral_layer_is_a_real_fourier_filter():
    """With unit mode weights the spectral layer keeps exactly the retained
    Fourier components of a real field (with their Hermitian mirrors); the
    unpaired row ky = -m/2 at kx = 0 keeps half of its pair, as Re() does."""
    c = fo.Cfg(nin=1, width=1, modes=4, layers=1, proj=1, nout=1, grid=16)
    rng = np.random.default_rng(5)
    h = rng.standard_normal((1, 1, 16, 16))
    R = np.ones((4, 4, 1, 1), complex)
    s, _ = fo._spectral(h, R, fo._mats(c))
    H = np.fft.fft2(h[0, 0])            # axis 0: ky, axis 1: kx
    H2 = np.zeros_like(H)
    for ky in (0, 1, -2, -1):
        for kx in (1, 2, 3):
            H2[ky % 16, kx] = H[ky % 16, kx]
            H2[-ky % 16, -kx % 16] = H[-ky % 16, -kx % 16]
    for ky in (0, 1, -1):
        H2[ky % 16, 0] = H[ky % 16, 0]
    H2[2, 0] = 0.5 * H[2, 0]
    H2[14, 0] = 0.5 * H[14, 0]
    assert np.abs(s[0, 0] - np.real(np.fft.ifft2(H2))).max() < 1e-12
