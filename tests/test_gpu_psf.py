"""PSF consumers on the GPU: exposure PSFs and the chromatic PSF through the
C ABI against the FP64 oracle and the reference's own outputs
(tests/golden/psf.npz), and the exposure command end to end.

Tolerances: FP32 transforms vs FP64 -- relative max error 2e-5 of the
image maximum (exposure and chromatic PSFs; the chromatic sum also carries
the float bilinear weights of the reference); the exposure log within
1e-3 arcsec (FWHM and EE50 are read from the filtered image, whose
ring-crossing interpolation amplifies the FP32 differences) and 1e-3 px
(centres)."""
import numpy as np
import pytest

import golden_case as gcm
from test_psf_golden import G, exposures

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("W,nf,per_frame_amp", [(32, 3, False), (64, 5, True), (256, 2, False), (1024, 1, False)])
def test_expo_accumulate_matches_oracle(lib, oracle64, W, nf, per_frame_amp):
    from atmosphericturbulencesimul_gb300 import psf as P
    rng = np.random.default_rng(W + nf)
    y, x = np.mgrid[0:W, 0:W] - (W / 2 - 0.5)
    pup = (np.hypot(x, y) < W / 2).astype(np.float32)
    pha = (rng.standard_normal((nf, W, W)) * 0.8).astype(np.float32)
    amp = (pup * rng.uniform(0.5, 1.0, (nf, W, W))).astype(np.float32) if per_frame_amp else pup
    got = P.expo_accumulate(pha, amp)
    ref = oracle64.psf_expo(amp, pha)
    assert np.abs(got - ref).max() / ref.max() < 2e-5
    # accumulation into an existing image keeps the earlier exposure
    twice = P.expo_accumulate(pha, amp, got)
    assert np.abs(twice - 2 * ref).max() / ref.max() < 4e-5


def test_expo_device_api_and_layout(lib):
    """Accumulator layout round trip and the device entry points on torch
    buffers: batches accumulated one after the other equal one call."""
    torch = pytest.importorskip("torch")
    from atmosphericturbulencesimul_gb300 import psf as P
    W = 128
    rng = np.random.default_rng(5)
    pha = torch.tensor(rng.standard_normal((7, W, W)) * 0.5, dtype=torch.float32, device="cuda")
    amp = torch.ones((W, W), dtype=torch.float32, device="cuda")
    acc1 = torch.zeros((2 * W, 2 * W), dtype=torch.float32, device="cuda")
    acc2 = torch.zeros_like(acc1)
    P.expo_accumulate_dev(pha, amp, acc1)
    P.expo_accumulate_dev(pha[:3], amp, acc2)
    P.expo_accumulate_dev(pha[3:], amp, acc2)
    img1, img2 = torch.empty_like(acc1), torch.empty_like(acc1)
    P.expo_image_dev(acc1, img1)
    P.expo_image_dev(acc2, img2)
    torch.cuda.synchronize()
    a, b = img1.cpu().numpy(), img2.cpu().numpy()
    assert np.abs(a - b).max() / a.max() < 1e-6
    host = P.expo_accumulate(pha.cpu().numpy(), amp.cpu().numpy())
    assert np.abs(a - host).max() / a.max() < 1e-6
    # a flat phase: the centred PSF peaks at (W, W) with the squared pupil sum
    flat = P.expo_accumulate(np.zeros((1, W, W), np.float32), np.ones((W, W), np.float32))
    assert np.unravel_index(np.argmax(flat), flat.shape) == (W, W)
    assert abs(flat[W, W] / float(W * W) ** 2 - 1) < 1e-6


def test_expo_psfs_match_reference(lib):
    from atmosphericturbulencesimul_gb300 import psf as P
    etime, dt, W, nframes, ntspan = G["expo_par"]
    groups, rest = exposures(etime, dt, int(nframes), int(ntspan))
    pup, pha = G["expo_pupil"], G["expo_pha"]
    for k, grp in enumerate(groups):
        got = P.expo_accumulate(np.stack([pha[t][f] for t, f in grp]), pup)
        ref = G[f"expo_psf{k}"]
        assert np.abs(got - ref).max() / ref.max() < 2e-5, k


@pytest.mark.parametrize("k", range(2))
def test_chromatic_psf_matches_reference(lib, oracle64, k):
    from atmosphericturbulencesimul_gb300 import psf as P
    n, c1, c2, ns, apo = G[f"chromat_par{k}"]
    got = P.chromat_psf(G[f"chromat_amp{k}"], G[f"chromat_pha{k}"], c1, c2, int(ns), apo)
    ref = G[f"chromat_out{k}"]
    assert np.abs(got - ref).max() / ref.max() < 2e-5
    o = oracle64.chromat_psf(G[f"chromat_amp{k}"], G[f"chromat_pha{k}"], c1, c2, int(ns), apo)
    assert np.abs(got - o).max() / o.max() < 2e-5


def test_chromatic_psf_large(lib, oracle64):
    """512^2 pupil, 9 steps with apodisation, against the oracle."""
    from atmosphericturbulencesimul_gb300 import psf as P
    n = 512
    y, x = np.mgrid[0:n, 0:n] - (n / 2 - 0.5)
    amp = (np.hypot(x, y) < n / 4).astype(np.float32)
    pha = (np.sin(x / 17.0) * np.cos(y / 23.0) * 2.0 * amp).astype(np.float32)
    got = P.chromat_psf(amp, pha, 0.7, 1.4, 9, 0.3)
    ref = oracle64.chromat_psf(amp, pha, 0.7, 1.4, 9, 0.3)
    assert np.abs(got - ref).max() / ref.max() < 2e-5


@pytest.mark.parametrize("amplitude_on", [0, 1])
def test_expoframes_matches_reference(lib, tmp_path, monkeypatch, amplitude_on):
    """The exposure command on the reference's inputs: PSF%04d.fits, the
    final PSF file and the log lines.  The amplitude cubes equal the pupil,
    so both amplitude sources give the reference's field."""
    import sys
    sys.path.insert(0, str(gcm.GOLDEN))
    import fits_io
    from atmosphericturbulencesimul_gb300 import psf as P
    from atmosphericturbulencesimul_gb300.mkwfs import fits_read
    monkeypatch.chdir(tmp_path)
    etime, dt, W, nframes, ntspan = G["expo_par"]
    W, nframes, ntspan = int(W), int(nframes), int(ntspan)
    (tmp_path / "WFS_files").mkdir()
    fits_io.write(tmp_path / "pupil.fits", G["expo_pupil"])
    for t in range(ntspan):
        fits_io.write(tmp_path / "WFS_files" / f"wf_{t:08d}.{1650000:09d}.pha.fits", G["expo_pha"][t])
        fits_io.write(tmp_path / "WFS_files" / f"wf_{t:08d}.{1650000:09d}.amp.fits",
                      np.repeat(G["expo_pupil"][None], nframes, 0))
    (tmp_path / "WFsim.conf").write_text(str(G["expo_conf"]))
    final = P.expoframes(float(etime), "expo.log", amplitude_on=amplitude_on)
    k = 0
    while f"expo_psf{k}" in G.files:
        got = fits_read(tmp_path / f"PSF{k:04d}.fits")
        ref = G[f"expo_psf{k}"]
        assert np.abs(got - ref).max() / ref.max() < 2e-5, k
        k += 1
    assert not (tmp_path / f"PSF{k:04d}.fits").exists()
    fin = fits_read(tmp_path / "PSF")
    assert np.abs(fin - G["expo_final"]).max() / G["expo_final"].max() < 2e-5
    got_lines = (tmp_path / "expo.log").read_text().splitlines()
    ref_lines = str(G["expo_log"]).splitlines()
    assert len(got_lines) == len(ref_lines)
    for a, b in zip(got_lines, ref_lines):
        va, vb = np.array(a.split(), float), np.array(b.split(), float)
        assert va[0] == vb[0]
        assert np.all(np.abs(va[1:3] - vb[1:3]) < 1e-3), (a, b)
        assert np.all(np.abs(va[3:] - vb[3:]) < 1e-3), (a, b)
    assert abs(final - float(G["expo_final_fwhm"])) < 1e-3
