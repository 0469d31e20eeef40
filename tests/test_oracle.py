"""The CPU oracle against independent references (numpy, analytic invariants,
published known-answer vectors) -- runs without a GPU."""
import numpy as np
import pytest

from oracle import oracle as orc


def test_philox_known_answers(oracle64):
    # Random123 philox4x32-10 known-answer vectors
    assert oracle64.philox4([0, 0, 0, 0], [0, 0]) == [0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8]
    assert oracle64.philox4([0xFFFFFFFF] * 4, [0xFFFFFFFF] * 2) == [0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD]
    assert oracle64.philox4([0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344], [0xA4093822, 0x299F31D0]) == [
        0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1]


def test_screen_noise_statistics(oracle64):
    u, g = oracle64.screen_noise(3, 0, 256)
    assert 0.0 <= u.min() and u.max() < 1.0
    assert abs(u.mean() - 0.5) < 0.01 and abs(g.mean()) < 0.02 and abs(g.std() - 1) < 0.02


@pytest.mark.parametrize("n", [8, 64, 256])
@pytest.mark.parametrize("bits", [64, 32])
def test_fft2d_matches_numpy(n, bits, oracle64, oracle32):
    o = oracle64 if bits == 64 else oracle32
    rng = np.random.default_rng(n)
    a = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    tol = 1e-12 if bits == 64 else 2e-6
    f = o.fft2d(a, -1)
    assert np.abs(f - np.fft.fft2(a)).max() / np.abs(f).max() < tol
    b = o.fft2d(a, +1)
    ref = np.fft.ifft2(a) * n * n
    assert np.abs(b - ref).max() / np.abs(ref).max() < tol


def test_fresnel_matches_numpy_restatement(oracle64):
    # Fresnel_propagate_wavefront written with numpy: fft2, fftshift, transfer, ifftshift, ifft2
    n, dx, z, lam = 128, 0.01, 3000.0, 1.6e-6
    rng = np.random.default_rng(2)
    a = np.exp(1j * rng.standard_normal((n, n)) * 2)
    coeff = np.pi * z * lam / (dx * n) ** 2
    ii = np.arange(n) - n // 2
    H = np.exp(-1j * coeff * (ii[None, :] ** 2 + ii[:, None] ** 2)) / n ** 2
    ref = np.fft.ifft2(np.fft.ifftshift(np.fft.fftshift(np.fft.fft2(a)) * H)) * n * n
    got = oracle64.fresnel(a, dx, z, lam)
    assert np.abs(got - ref).max() < 1e-10


def test_fresnel_invariants(oracle64):
    n = 64
    rng = np.random.default_rng(4)
    a = np.exp(1j * rng.standard_normal((n, n)))
    # z = 0 is the identity; energy is conserved (Parseval)
    assert np.abs(oracle64.fresnel(a, 0.01, 0.0, 0.5e-6) - a).max() < 1e-12
    b = oracle64.fresnel(a, 0.01, 5000.0, 0.5e-6)
    assert abs(np.sum(np.abs(b) ** 2) / np.sum(np.abs(a) ** 2) - 1) < 1e-12
    # a plane wave stays a plane wave
    p = np.ones((n, n), complex)
    assert np.abs(oracle64.fresnel(p, 0.01, 5000.0, 0.5e-6) - p).max() < 1e-12


def test_window_matches_direct_bicubic(oracle64):
    M, W = 64, 16
    rng = np.random.default_rng(5)
    S = rng.standard_normal((M, M))
    xpos, ypos = 61.3, 0.7
    got = oracle64.window(S, xpos, ypos, W)

    def keys(t):
        return np.array([0.5 * (-t ** 3 + 2 * t ** 2 - t), 0.5 * (3 * t ** 3 - 5 * t ** 2 + 2),
                         0.5 * (-3 * t ** 3 + 4 * t ** 2 + t), 0.5 * (t ** 3 - t ** 2)])

    ref = np.zeros((W, W))
    for jj in range(W):
        for ii in range(W):
            X, Y = (xpos + ii) % M, (ypos + jj) % M
            xi, yi = int(X), int(Y)
            wx, wy = keys(X - xi), keys(Y - yi)
            for b in range(4):
                for a in range(4):
                    ref[jj, ii] += wx[a] * wy[b] * S[(yi - 1 + b) % M, (xi - 1 + a) % M]
    assert np.abs(got - ref).max() < 1e-12
    # the Keys kernel reproduces the samples at integer positions
    assert np.allclose(oracle64.window(S, 3.0, 5.0, W), np.roll(np.roll(S, -5, 0), -3, 1)[:W, :W])


def test_superlayer_grouping(oracle64):
    alt = [0.0, 50.0, 5000.0, 12000.0]
    cn2 = np.array([0.4, 0.2, 0.3, 0.1])
    salt, sidx = oracle64.superlayers(alt, cn2, 100.0)
    assert len(salt) == 3 and list(sidx) == [0, 0, 1, 2]
    assert abs(salt[0] - (0.4 * 0 + 0.2 * 50) / 0.6) < 1e-12
    salt, sidx = oracle64.superlayers([5000.0], [1.0], 100.0)
    assert list(salt) == [5000.0] and list(sidx) == [0]
    # a bin wider than every gap collapses the profile to one super-layer
    salt, sidx = oracle64.superlayers([0.0, 500.0, 1000.0], np.array([1, 1, 1]) / 3, 1e6)
    assert len(salt) == 1 and list(sidx) == [0, 0, 0]


def test_position_wrap(oracle64):
    M = 256
    p, c = oracle64.position_step(255.9, 0, 300.0, np.float32(0.001), M)
    assert c == -1 and abs(p - (255.9 + 300 * float(np.float32(0.001)) - M)) < 1e-12
    p, c = oracle64.position_step(0.1, 0, -300.0, np.float32(0.001), M)
    assert c == 1 and p > 0
    # pos == M exactly is kept (strict comparison in the reference)
    p, c = oracle64.position_step(float(M) - 1.0, 0, 2.0, np.float32(0.5), M)
    assert p == float(M) and c == 0


def test_master_screen_structure_function(oracle64):
    M = 256
    u, g = oracle64.screen_noise(1, 0, M)
    o1, o2, cf = oracle64.master_screen(u, g, 2000.0, 0.5)
    for o in (o1, o2):
        # after normalisation D(r) ~ r^(5/3) over lags (1..2)^2 in the geometric mean
        v = []
        for lx in (1, 2):
            for ly in (1, 2):
                D = np.mean((o - np.roll(np.roll(o, -ly, 0), -lx, 1)) ** 2)
                v.append(np.log10(D) - 5 / 3 * np.log10(np.hypot(lx, ly)))
        assert abs(np.mean(v)) < 1e-9
    assert cf[0] > 0 and cf[1] > 0


def test_unwrap_reference_output_is_consistent(oracle64):
    # a smooth geometric phase with no propagation: the unwrapped science
    # phase equals the geometric phase sum
    W = 64
    y, x = np.mgrid[0:W, 0:W]
    phasum = 0.2 * x + 0.1 * y - 5.0
    field = np.exp(1j * phasum)
    pha, amp, bins, it = oracle64.output_sci(phasum, field, W)
    assert np.abs(pha - phasum).max() < 1e-9
    assert np.allclose(amp, 1)
    pr, ar = oracle64.output_ref(phasum, field, W)
    assert np.abs(pr - phasum).max() < 1e-9


def test_float_port_tracks_fp64(oracle64, oracle32):
    from series_case import Case, make_screens
    case = Case(alt=[0.0, 3000.0], cn2=[0.6, 0.4], speed=[10.0, 20.0], direction=[0.1, 1.0], M=128, W=64, Wout=64)
    screens = make_screens(case, oracle64)
    salt, sidx = oracle64.superlayers(case.alt, np.array([0.6, 0.4]), 100.0)
    x = np.array([6.4, 30.2])
    y = np.array([6.4, 90.9])
    a = oracle64.frame(screens, x, y, None, sidx, salt, 0.01, 0.0, 0.5e-6, 64)
    b = oracle32.frame(screens, x, y, None, sidx, salt, 0.01, 0.0, 0.5e-6, 64)
    assert np.abs(a[1] - b[1]).max() < 1e-4
