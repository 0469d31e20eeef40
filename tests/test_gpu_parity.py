"""GPU parity: the CUDA engine (through the C ABI) against the FP64 oracle and numpy.

Tolerances (floating point, FP32 engine vs FP64 oracle):
  * 2-D FFT: relative max error <= 2e-5 (FP32 Stockham, log2 N stages);
  * Fresnel hop: relative max error <= 2e-5;
  * series frames: wrapped phase error <= 0.05 nm rms, amplitude error <= 2e-3,
    and (the reference's bar) relative OPD rms and amplitude variance within 1e-4;
    the unwrapped phase may differ by a 2 pi jump on at most 0.2 % of the pixels.
"""
import numpy as np
import pytest

from series_case import Case, compare, make_screens, run_gpu

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("n", [64, 128, 256, 512, 1024, 2048])
@pytest.mark.parametrize("sign", [-1, 1])
def test_fft2d_matches_numpy(lib, n, sign):
    from atmosphericturbulencesimul_gb300 import fft2d
    rng = np.random.default_rng(n)
    a = (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))).astype(np.complex64)
    got = fft2d(a, sign)
    ref = np.fft.fft2(a.astype(np.complex128)) if sign < 0 else np.fft.ifft2(a.astype(np.complex128)) * n * n
    err = np.abs(got - ref).max() / np.abs(ref).max()
    assert err < 2e-5, err


@pytest.mark.parametrize("n,z,lam", [(128, 5000.0, 0.5e-6), (256, 8000.0, 2.2e-6), (1024, 500.0, 1.6e-6)])
def test_fresnel_matches_oracle(lib, oracle64, n, z, lam):
    from atmosphericturbulencesimul_gb300 import fresnel
    rng = np.random.default_rng(n)
    ph = rng.standard_normal((n, n)) * 3
    a = np.exp(1j * ph).astype(np.complex64)
    dx = float(np.float32(0.01))
    got = fresnel(a, dx, z, lam)
    ref = oracle64.fresnel(a.astype(np.complex128), dx, z, lam)
    err = np.abs(got - ref).max() / np.abs(ref).max()
    assert err < 2e-5, err
    # Parseval: the hop conserves energy
    assert abs(np.sum(np.abs(got) ** 2) / np.sum(np.abs(a) ** 2) - 1) < 1e-5


def _compare(case, o64, nsteps, wrapped_nm=0.05, flip=2e-3):
    return compare(case, o64, nsteps, wrapped_nm=wrapped_nm, flip=flip)


def test_series_three_planes(lib, oracle64):
    case = Case(alt=[0.0, 2000.0, 8000.0], cn2=[0.6, 0.25, 0.15], speed=[10.0, 20.0, 15.0],
                direction=[0.5236, 2.0, 4.0], M=256, W=128, Wout=128, fresnel_bin=100.0)
    _compare(case, oracle64, 4)


def test_series_crop_and_grouped_layers(lib, oracle64):
    # layers at 0 and 50 m share a super-layer; 64-pixel crop of a 128 grid
    case = Case(alt=[0.0, 50.0, 5000.0, 12000.0], cn2=[0.4, 0.2, 0.3, 0.1], speed=[8.0, 12.0, 25.0, 30.0],
                direction=[0.1, 1.0, 3.0, 5.5], M=256, W=128, Wout=64, fresnel_bin=100.0,
                sci=[(1.25e-6, 0.0, 0.0), (2.2e-6, 4.85e-5, -4.85e-5)])
    _compare(case, oracle64, 3)


@pytest.mark.parametrize("cfg", [0, 1, 2])
def test_series_every_tile_configuration(lib, oracle64, monkeypatch, cfg):
    """Each compiled tile configuration (separate or overlaid screen tile,
    1..32 rows per CTA) on grouped layers, a crop and two grid sizes."""
    monkeypatch.setenv("ATMWFS_TILE_CFG", str(cfg))
    case = Case(alt=[0.0, 50.0, 5000.0, 12000.0], cn2=[0.4, 0.2, 0.3, 0.1], speed=[8.0, 12.0, 25.0, 30.0],
                direction=[0.1, 1.0, 3.0, 5.5], M=512, W=256, Wout=200, fresnel_bin=100.0,
                sci=[(1.25e-6, 0.0, 0.0), (2.2e-6, 4.85e-5, -4.85e-5)])
    _compare(case, oracle64, 2)


def test_series_air_index_hops(lib, oracle64):
    """The optional lambda / n(air) hops: each hop's transfer function uses
    the air index at its middle (WFpropagate.c:91 uses the vacuum lambda);
    the oracle runs the same hops.  The frames must also differ from the
    vacuum-lambda frames by more than the parity bar."""
    kw = dict(alt=[0.0, 2000.0, 8000.0], cn2=[0.6, 0.25, 0.15], speed=[10.0, 20.0, 15.0], direction=[0.5236, 2.0, 4.0],
              M=256, W=128, Wout=128, fresnel_bin=100.0, sci=[(0.5e-6, 0.0, 0.0), (2.2e-6, 4.85e-5, 0.0)])
    case = Case(air_index=True, **kw)
    _compare(case, o64 := oracle64, 2)
    screens = make_screens(case, o64)
    _, fa, _, _ = run_gpu(case, screens, 1)
    _, fv, _, _ = run_gpu(Case(**kw), screens, 1)
    assert max(np.abs(a[1] - v[1]).max() for a, v in zip(fa, fv)) > 1e-4


def test_series_single_layer_no_hop(lib, oracle64):
    case = Case(alt=[5000.0], cn2=[1.0], speed=[10.0], direction=[0.5236], M=256, W=256, Wout=256)
    _compare(case, oracle64, 3)


def test_series_phase_only(lib, oracle64):
    case = Case(alt=[0.0, 3000.0], cn2=[0.5, 0.5], speed=[10.0, -20.0], direction=[0.3, 1.2], M=256, W=64,
                Wout=64, amplitude=0)
    _compare(case, oracle64, 3)


def test_series_bins_straddling_three_rows(lib, oracle64, monkeypatch):
    # 32-row tiles (tile configuration 0 of a 128 grid) with a 100-pixel crop:
    # the rows 32..63 tile covers output rows 18..49, i.e. science bins 0, 1, 2
    monkeypatch.setenv("ATMWFS_TILE_CFG", "0")
    case = Case(alt=[0.0, 6000.0], cn2=[0.7, 0.3], speed=[12.0, 25.0], direction=[0.2, 2.4], M=256, W=128,
                Wout=100, fresnel_bin=100.0)
    _compare(case, oracle64, 2)


def test_series_large_grid(lib, oracle64):
    case = Case(alt=[0.0, 4000.0, 16000.0], cn2=[0.5, 0.3, 0.2], speed=[10.0, 20.0, 30.0], direction=[0.5, 2.5, 4.5],
                M=1024, W=512, Wout=512, fresnel_bin=100.0)
    _compare(case, oracle64, 2)


def test_output_ring_holds_every_instance(lib, oracle64):
    """A device output ring of several slots with several instances of
    different crops returns the same frames as a single slot."""
    case = Case(alt=[0.0, 3000.0], cn2=[0.6, 0.4], speed=[10.0, 20.0], direction=[0.3, 2.0], M=256, W=128,
                Wout=100, sci=[(1.25e-6, 0.0, 0.0), (2.2e-6, 4.85e-5, 0.0)])
    screens = make_screens(case, oracle64)
    _, f1, _, _ = run_gpu(case, screens, 5, ring=1)
    _, f3, _, _ = run_gpu(case, screens, 5, ring=3)
    for a, b in zip(f1, f3):
        assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])


def test_master_screen_matches_oracle(lib, oracle64):
    from atmosphericturbulencesimul_gb300 import master_screen
    M = 256
    g1, g2, gc = master_screen(11, M, 2000.0, 1.0, stream=3)
    u, g = oracle64.screen_noise(11, 3, M)
    o1, o2, oc = oracle64.master_screen(u, g, 2000.0, 1.0)
    assert np.abs(g1 - o1).max() / np.abs(o1).max() < 1e-4
    assert np.abs(g2 - o2).max() / np.abs(o2).max() < 1e-4
    assert np.allclose(gc, oc, rtol=1e-4)


def test_normalize_matches_oracle(lib, oracle32):
    from oracle import oracle as orc
    from atmosphericturbulencesimul_gb300 import InstanceSpec, Series
    M = 256
    rng = np.random.default_rng(5)
    screens = [rng.standard_normal((M, M)).astype(np.float32) * 5 for _ in range(2)]
    s = Series([0.0, 1000.0], [0.7, 0.3], [5.0, 5.0], [0.0, 1.0], master_size=M,
               instances=[InstanceSpec(lam=0.5e-6, wf_raw_size=64)], pupil_scale=0.01, time_step=0.001)
    for l, sc in enumerate(screens):
        s.load_screen(l, sc)
    r0g = s.normalize(np.float32(0.5e-6), np.float32(0.6875))
    ref = [x.copy() for x in screens]
    r0o = orc.r0_renormalise(oracle32, ref, np.float32(0.5e-6), np.float32(0.6875), np.float32(0.01),
                             np.array([0.7, 0.3]), np.float32(0.0))
    assert np.allclose(r0g, r0o, rtol=1e-6)
    s.close()


def test_series_odd_crops(lib, oracle64):
    """Crops that break the 16-byte vectors (129 of 256, 257 of 512, 75 of 128):
    the phase sum, the epilogue and the science apply take their one-column
    paths; science bins of 21-22 pixels (nb = Wout / 20 rounded down)."""
    case = Case(alt=[0.0, 3000.0, 9000.0], cn2=[0.5, 0.3, 0.2], speed=[9.0, 17.0, 26.0], direction=[0.4, 2.1, 4.0],
                M=512, W=256, Wout=129, fresnel_bin=100.0,
                sci=[(1.25e-6, 0.0, 0.0), (2.2e-6, 4.85e-5, 0.0, 512, 257), (0.7e-6, 0.0, 4.85e-5, 128, 75)])
    _compare(case, oracle64, 2)


def test_zero_steps_then_steps(lib, oracle64):
    """A run of zero steps is a no-op that returns OK; the steps after it give
    the same frames as a context that never ran it."""
    case = Case(alt=[0.0, 4000.0], cn2=[0.6, 0.4], speed=[10.0, 20.0], direction=[0.3, 2.0], M=256, W=128, Wout=128)
    screens = make_screens(case, oracle64)
    from atmosphericturbulencesimul_gb300 import Series
    from series_case import instances

    def frames(zero_first):
        s = Series(case.alt, case.cn2, case.speed, case.direction, master_size=case.M, instances=instances(case),
                   pupil_scale=case.pupil, time_step=case.dt, fresnel_bin=case.fresnel_bin)
        for l, sc in enumerate(screens):
            s.load_screen(l, sc)
        if zero_first:
            z = s.run_frames(0)
            assert all(p.shape[0] == 0 and a.shape[0] == 0 for p, a in z)
        out = s.run_frames(2)
        s.close()
        return out

    for (p0, a0), (p1, a1) in zip(frames(False), frames(True)):
        assert np.array_equal(p0, p1) and np.array_equal(a0, a1)
