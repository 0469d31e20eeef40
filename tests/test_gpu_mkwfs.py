"""The series command end to end on the GPU: atmwfs_mkwfs() reads the
reference's configuration and profile files and master screens, runs the
engine and writes the FITS cubes, which must match the cubes the reference
wrote on the same inputs (tests/golden/).  Also: master-screen synthesis,
extra master files, SKIP_EXISTING, WFOUTPUT 0 and the shared-memory stream.

Tolerances as in test_gpu_golden.py (FP32 engine vs the reference)."""
import ctypes as C
import ctypes.util
import os
import struct
from pathlib import Path

import numpy as np
import pytest

import golden_case as gcm
from test_gpu_golden import GPU_LIMITS

pytestmark = pytest.mark.gpu


def _stage(gc, d: Path, screens: bool = True):
    (d / "WF_files").mkdir(exist_ok=True)
    (d / "WFS_files").mkdir(exist_ok=True)
    (d / "WFsim.conf").write_text(gc.conf)
    (d / "turbul.prof").write_text(gc.prof)
    if screens:
        from atmosphericturbulencesimul_gb300.mkwfs import fits_write
        sfx = "f" if gc.precision == 0 else "d"
        for l, s in enumerate(gc.screens):
            fits_write(d / f"t{l:03d}_{gc.M}_{sfx}.fits", s.astype(np.float32 if gc.precision == 0 else np.float64))


def _read_cubes(gc, d: Path) -> dict:
    from atmosphericturbulencesimul_gb300.mkwfs import cube_name, fits_read
    out = {}
    for key, pre in (("ref", "WF_files/wf_"), ("sci", "WFS_files/wf_")):
        for q in ("pha", "amp") if gc.amplitude else ("pha",):
            out[f"{key}_{q}"] = np.concatenate([fits_read(d / cube_name(pre, t, gc.slam, q)) for t in range(gc.ntspan)])
    return out


@pytest.mark.parametrize("name", gcm.CASES)
def test_mkwfs_matches_reference_files(lib, tmp_path, monkeypatch, name):
    from atmosphericturbulencesimul_gb300.mkwfs import mkwfs
    gc = gcm.load(name)
    monkeypatch.chdir(tmp_path)
    _stage(gc, tmp_path)
    mkwfs(gc.slam_um, gc.precision, scoeff=gc.scoeff, roffset=gc.roffset)
    got = _read_cubes(gc, tmp_path)
    assert set(got) == set(gc.cubes)
    if gc.precision == 1:        # double files, as the reference's WFprecision 1
        assert b"BITPIX  =                  -64" in (tmp_path / "WFS_files" / os.listdir("WFS_files")[0]).read_bytes()[:400]
    gcm.compare(got, gc, GPU_LIMITS)


def test_mkwfs_with_refractivity_callback(lib, tmp_path, monkeypatch):
    """Scoeff and offsets from a refractivity model passed as a callback."""
    from atmosphericturbulencesimul_gb300.mkwfs import mkwfs
    gc = gcm.load("mkwfs")
    monkeypatch.chdir(tmp_path)
    _stage(gc, tmp_path)
    calls = []

    def N(alt, lam):
        calls.append((alt, lam))
        # the reference's Scoeff at these layers, expressed as a dispersion ratio
        return 2.7e-4 * (1.0 if abs(lam - gc.lam_ref) < 1e-12 else
                         float(np.interp(alt, gc.alt, gc.scoeff)) * gc.slam / gc.lam_ref)

    mkwfs(gc.slam_um, 0, refractivity=N)
    assert len(calls) == 2 * len(gc.alt)          # zenith: Scoeff only, no offset integration
    gcm.compare(_read_cubes(gc, tmp_path), gc, GPU_LIMITS)


def test_mkwfs_synthesises_missing_masters(lib, tmp_path, monkeypatch):
    from atmosphericturbulencesimul_gb300.mkwfs import fits_read, mkwfs
    gc = gcm.load("mkwfs")
    monkeypatch.chdir(tmp_path)
    _stage(gc, tmp_path, screens=False)
    mkwfs(gc.slam_um, 0, seed=gc.seed, scoeff=gc.scoeff)
    # the driver synthesised Philox-seeded screens; the reference synthesised
    # the same noise into the golden screens
    for l in range(len(gc.alt)):
        s = fits_read(tmp_path / f"t{l:03d}_{gc.M}_f.fits")
        assert np.abs(s - gc.screens[l]).max() / np.abs(gc.screens[l]).max() < 1e-4
    gcm.compare(_read_cubes(gc, tmp_path), gc, GPU_LIMITS)


def test_mkwfs_extra_master_enters_r0(lib, tmp_path, monkeypatch):
    """A master file beyond the layer count enters the mean r0 (:2246-2285):
    a fourth screen with twice the phase has a smaller r0, so the mean r0
    drops and every layer is scaled down."""
    from atmosphericturbulencesimul_gb300.mkwfs import fits_write, mkwfs
    gc = gcm.load("mkwfs")
    monkeypatch.chdir(tmp_path)
    _stage(gc, tmp_path)
    mkwfs(gc.slam_um, 0, scoeff=gc.scoeff)
    first = _read_cubes(gc, tmp_path)
    gcm.compare(first, gc, GPU_LIMITS)
    fits_write(tmp_path / f"t003_{gc.M}_f.fits", 2 * gc.screens[0])
    mkwfs(gc.slam_um, 0, scoeff=gc.scoeff)
    second = _read_cubes(gc, tmp_path)
    assert second["ref_pha"].std() < 0.95 * first["ref_pha"].std()


def test_mkwfs_skip_existing_and_wfoutput0(lib, tmp_path, monkeypatch):
    from atmosphericturbulencesimul_gb300.mkwfs import cube_name, mkwfs
    gc = gcm.load("mkwfs_c")          # two time spans
    monkeypatch.chdir(tmp_path)
    _stage(gc, tmp_path)
    (tmp_path / "WFsim.conf").write_text(gc.conf + "SKIP_EXISTING 1\nWFOUTPUT 0\n")
    first = tmp_path / cube_name("WFS_files/wf_", 0, gc.slam, "pha")
    first.write_bytes(b"placeholder")
    mkwfs(gc.slam_um, 0, scoeff=gc.scoeff)
    assert first.read_bytes() == b"placeholder"      # span 0 skipped
    second = tmp_path / cube_name("WFS_files/wf_", 1, gc.slam, "pha")
    assert second.stat().st_size > 2880
    # WFOUTPUT 0: the reference-wavelength files of the computed span exist, empty
    ref1 = tmp_path / cube_name("WF_files/wf_", 1, gc.slam, "pha")
    assert ref1.exists() and ref1.stat().st_size == 0
    assert not (tmp_path / cube_name("WF_files/wf_", 0, gc.slam, "pha")).exists()
    # positions restart with the run (the reference does not restore them):
    # span 1's frames equal the reference's span 0 frames
    from atmosphericturbulencesimul_gb300.mkwfs import fits_read
    got = fits_read(second)
    for f in range(gc.nframes):
        e = gcm.frame_errors(got[f], None, gc.cubes["sci_pha"][f], None, gc.slam)
        assert e["wrapped_rms_nm"] < GPU_LIMITS["wrapped_rms_nm"], (f, e)


MD = struct.Struct("@80sl3lli dd ll iii lll")


def test_mkwfs_science_stream(lib, tmp_path, monkeypatch):
    """SHM_SOUTPUT: the last science frame in /tmp/<prefix>pha.im.shm, in um (SHM_SOUTPUTM 2)."""
    from atmosphericturbulencesimul_gb300.mkwfs import mkwfs
    gc = gcm.load("mkwfs")
    monkeypatch.chdir(tmp_path)
    _stage(gc, tmp_path)
    prefix = f"atmwfs_s{os.getpid()}_"
    (tmp_path / "WFsim.conf").write_text(gc.conf + f"SHM_SOUTPUT 1\nSHM_SPREFIX {prefix}\nSHM_SOUTPUTM 2\n")
    libc = C.CDLL(ctypes.util.find_library("c") or "libc.so.6")
    libc.sem_unlink.argtypes = [C.c_char_p]
    try:
        mkwfs(gc.slam_um, 0, scoeff=gc.scoeff, roffset=gc.roffset)
        raw = Path(f"/tmp/{prefix}pha.im.shm").read_bytes()
        md = MD.unpack_from(raw)
        assert md[14] == gc.frames                                  # cnt0: one per frame
        n = gc.Wout * gc.Wout
        last = np.frombuffer(raw, np.float32, n, MD.size).reshape(gc.Wout, gc.Wout)
        want = gc.cubes["sci_pha"][-1] * (gc.slam / 2 / np.pi * 1e6)
        assert np.sqrt(np.mean((last - want) ** 2)) * 1e3 < GPU_LIMITS["wrapped_rms_nm"]  # um -> nm
        amp = np.frombuffer(Path(f"/tmp/{prefix}amp.im.shm").read_bytes(), np.float32, n, MD.size)
        assert np.abs(amp.reshape(gc.Wout, gc.Wout) - gc.cubes["sci_amp"][-1]).max() < GPU_LIMITS["amp_max_err"]
    finally:
        for q in ("pha", "amp"):
            p = Path(f"/tmp/{prefix}{q}.im.shm")
            if p.exists():
                p.unlink()
            for k in range(10):
                libc.sem_unlink(f"{prefix}{q}_sem{k:02d}".encode())
            libc.sem_unlink(f"{prefix}{q}_semlog".encode())


def test_mkwfs_realtime_surrogate_and_fallback(lib, tmp_path, monkeypatch):
    """SURROGATE_MODEL in real-time mode: frames come from the network
    (phase = geometric phase + arg(1 + D)); a model that does not fit the run
    (another grid) leaves the plain propagation in place, bit for bit."""
    from atmosphericturbulencesimul_gb300 import fno as F
    from atmosphericturbulencesimul_gb300.mkwfs import cube_name, fits_read, mkwfs
    gc = gcm.load("mkwfs")
    monkeypatch.chdir(tmp_path)
    _stage(gc, tmp_path)
    # real time with factor 0: every frame at t = 0, so runs are comparable
    rt = gc.conf + "REALTIME 1\nREALTIMEFACTOR 0\n"
    sci = lambda q: fits_read(tmp_path / cube_name("WFS_files/wf_", 0, gc.slam, q))
    (tmp_path / "WFsim.conf").write_text(rt)
    mkwfs(gc.slam_um, 0, scoeff=gc.scoeff, roffset=gc.roffset)
    plain_pha, plain_amp = sci("pha"), sci("amp")
    # geometric phase of the same windows: the phase-only run
    (tmp_path / "WFsim.conf").write_text(rt + "WAVEFRONT_AMPLITUDE 0\n")
    mkwfs(gc.slam_um, 0, scoeff=gc.scoeff, roffset=gc.roffset)
    geo = sci("pha")
    # a fitting model (3 layers + wavelength, 64 grid)
    F.Surrogate(F.FnoConfig(nin=4, width=8, modes=8, layers=1, proj=8, grid=64), seed=2).save(tmp_path / "m.bin")
    (tmp_path / "WFsim.conf").write_text(rt + "SURROGATE_MODEL m.bin\n")
    mkwfs(gc.slam_um, 0, scoeff=gc.scoeff, roffset=gc.roffset)
    pha, amp = sci("pha"), sci("amp")
    assert np.all(np.isfinite(pha)) and np.all(np.isfinite(amp))
    assert not np.array_equal(amp, plain_amp)
    assert np.median(np.abs(pha - geo)) < 0.5          # an untrained network keeps D small
    # a model for another grid: the plain path runs
    F.Surrogate(F.FnoConfig(nin=4, width=8, modes=8, layers=1, proj=8, grid=32), seed=2).save(tmp_path / "m32.bin")
    (tmp_path / "WFsim.conf").write_text(rt + "SURROGATE_MODEL m32.bin\n")
    mkwfs(gc.slam_um, 0, scoeff=gc.scoeff, roffset=gc.roffset)
    assert np.array_equal(sci("pha"), plain_pha) and np.array_equal(sci("amp"), plain_amp)
