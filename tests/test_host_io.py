"""Host side of the series command (no GPU): configuration reads against the
reference's own read_config_parameter outputs, the profile reader against
the layer table the reference printed, FITS cubes, and the shared-memory
stream layout of the reference's image files."""
import ctypes as C
import ctypes.util
import json
import os
import struct
import sys
from pathlib import Path

import numpy as np
import pytest

import golden_case as gcm

sys.path.insert(0, str(gcm.GOLDEN))
import fits_io  # noqa: E402


@pytest.fixture(scope="module")
def mk(lib):
    from atmosphericturbulencesimul_gb300 import mkwfs
    return mkwfs


def test_conf_reads_match_reference(mk, tmp_path):
    g = json.loads((gcm.GOLDEN / "conf.json").read_text())
    f = tmp_path / "t.conf"
    f.write_text(g["text"])
    for kw, exists, found, content in g["reads"]:
        assert mk.conf_exists(f, kw) == bool(exists), kw
        assert mk.conf_read(f, kw) == (bool(found), content), kw


@pytest.mark.parametrize("name", gcm.CASES)
def test_conf_load_of_golden_runs(mk, tmp_path, name):
    gc = gcm.load(name)
    f = tmp_path / "WFsim.conf"
    f.write_text(gc.conf)
    c = mk.load_conf(f)
    assert c["lambda"] == np.float32(gc.lam_ref)
    assert c["pupil_scale"] == np.float32(gc.pupil)       # mkwfs_c repeats it: last line wins
    assert c["wf_raw_size"] == gc.W and c["wfsize"] == gc.Wout and c["master_size"] == gc.M
    assert c["wavefront_amplitude"] == gc.amplitude
    assert c["fresnel_propagation"] == gc.amplitude        # forced to 0 without amplitude
    assert c["nb_tspan"] == gc.ntspan and c["skip_existing"] == 0
    assert c["zangle"] == np.float32(gc.zangle)
    assert c["prof_file"] == "turbul.prof" and c["wf_file_prefix"] == "./WF_files/wf_"
    nf = int(1.0 * float(c["time_span"]) / float(c["wftime_step"]) + 0.5)
    assert nf == gc.nframes


def test_conf_defaults_and_missing(mk, tmp_path):
    f = tmp_path / "WFsim.conf"
    f.write_text("WF_RAW_SIZE 256\nSKIP_EXISTING\n")
    c = mk.load_conf(f)
    assert c["wfoutput"] == 1 and c["shm_output"] == 0 and c["shm_soutput"] == 0   # guarded reads
    assert c["skip_existing"] == 1                       # enabled by the keyword alone
    assert c["wf_raw_size"] == 256 and c["realtime_factor"] == 0.0   # missing -> "-" -> 0
    assert c["prof_file"] == "-"
    from atmosphericturbulencesimul_gb300 import _lib
    with pytest.raises(_lib.AtmwfsError) as e:
        mk.load_conf(tmp_path / "absent.conf")
    assert e.value.status == 4


@pytest.mark.parametrize("name", gcm.CASES)
def test_profile_matches_reference_parse(mk, tmp_path, name):
    gc = gcm.load(name)
    f = tmp_path / "turbul.prof"
    f.write_text(gc.prof)
    got = mk.read_profile(f, 0.0)
    want = np.column_stack([gc.alt, gc.cn2, gc.speed, gc.direction, gc.outer, gc.inner,
                            np.load(gcm.GOLDEN / f"{name}.npz")["profile"][:, 6:]])
    assert np.array_equal(got, want)
    # the table the reference printed: normalised Cn2, six decimals
    ref = gc.logprof
    assert ref.shape == got.shape
    norm = got.copy()
    norm[:, 1] /= norm[:, 1].sum()
    assert np.allclose(norm, ref, atol=6e-7, rtol=0)


def test_profile_quirks_and_errors(mk, tmp_path):
    from atmosphericturbulencesimul_gb300 import _lib
    f = tmp_path / "p.prof"
    f.write_text("1000 1 2 3 4 5 6 7\n\n2000 1 2\n")
    got = mk.read_profile(f)
    assert got.shape == (3, 8)
    assert np.array_equal(got[1], got[0])                # blank line repeats the layer
    assert list(got[2]) == [2000, 1, 2, 3, 4, 5, 6, 7]   # short line keeps the previous values
    f.write_text("5 1 2 3 4 5 6 7\n")
    with pytest.raises(_lib.AtmwfsError):
        mk.read_profile(f, 100.0)                         # below the site: the reference leaves it unset
    f.write_text("5 1 2\n")
    with pytest.raises(_lib.AtmwfsError):
        mk.read_profile(f)                                # first layer line short: nothing to inherit


def test_fits_round_trip(mk, tmp_path):
    rng = np.random.default_rng(1)
    for dt in (np.float32, np.float64):
        for shape in ((7,), (5, 9), (3, 4, 6)):
            a = rng.standard_normal(shape).astype(dt)
            name = tmp_path / f"x{a.ndim}{a.dtype}.fits"
            mk.fits_write(name, a)
            assert np.array_equal(mk.fits_read(name), a.astype(np.float32))
            assert np.array_equal(fits_io.read(name), a)          # an independent reader
            assert name.stat().st_size % 2880 == 0
    # an independent writer, integer types with scaling
    b = (rng.standard_normal((6, 8)) * 100).astype(np.int16)
    fits_io.write(tmp_path / "i.fits", b)
    assert np.array_equal(mk.fits_read(tmp_path / "i.fits"), b.astype(np.float32))


def test_fits_overwrite_rule(mk, tmp_path):
    from atmosphericturbulencesimul_gb300 import _lib
    a = np.ones((4, 4), np.float32)
    name = tmp_path / "o.fits"
    mk.fits_write(name, a)
    with pytest.raises(_lib.AtmwfsError):
        mk.fits_write(name, a)                            # exists, no '!'
    mk.fits_write("!" + str(name), 2 * a)
    assert np.array_equal(mk.fits_read(name), 2 * a)


# IMAGE_METADATA of the reference's src/CLIcore.h, member by member, in
# native alignment: char name[80]; long naxis; long size[3]; long nelement;
# int atype; double creation_time, last_access; struct timespec wtime;
# int shared, write, status; long cnt0, cnt1, NBkw.
MD = struct.Struct("@80sl3lli dd ll iii lll")


def _libc():
    libc = C.CDLL(ctypes.util.find_library("c") or "libc.so.6", use_errno=True)
    libc.sem_open.restype = C.c_void_p
    libc.sem_open.argtypes = [C.c_char_p, C.c_int]
    libc.sem_post.argtypes = [C.c_void_p]
    libc.sem_close.argtypes = [C.c_void_p]
    libc.sem_unlink.argtypes = [C.c_char_p]
    return libc


def test_shm_stream_layout(mk):
    name = f"atmwfs_t{os.getpid()}"
    path = Path(f"/tmp/{name}.im.shm")
    libc = _libc()
    try:
        rng = np.random.default_rng(2)
        with mk.ShmImage(name, 12, 10, np.float32) as s:
            raw = path.read_bytes()
            assert len(raw) == MD.size + 12 * 10 * 4
            f = MD.unpack_from(raw)
            assert f[0].rstrip(b"\0").decode() == name
            naxis, sx, sy, sz, nel, atype = f[1:7]
            assert (naxis, sx, sy, nel, atype) == (2, 12, 10, 120, 3)
            shared, write, status, cnt0, cnt1, nbkw = f[11:17]
            assert shared == 1 and write == 0 and cnt0 == 0 and nbkw == 0
            for k in range(3):
                fr = rng.standard_normal((10, 12)).astype(np.float32)
                s.write(fr, bump=True)
            raw = path.read_bytes()
            assert MD.unpack_from(raw)[14] == 3                        # cnt0
            assert np.array_equal(np.frombuffer(raw, np.float32, 120, MD.size).reshape(10, 12), fr)
            s.write(fr * 0, bump=False)                                  # copy only
            assert MD.unpack_from(path.read_bytes())[14] == 3
            for k in range(10):
                assert libc.sem_open(f"{name}_sem{k:02d}".encode(), 0) not in (None, 0)
        # a semaphore wait: bounded, then released by a post
        from atmosphericturbulencesimul_gb300 import _lib
        with pytest.raises(_lib.AtmwfsError) as e:
            mk.shm_semwait(name, 0, 0.05)
        assert e.value.status == 5
        h = libc.sem_open(f"{name}_sem00".encode(), 0)
        libc.sem_post(h)
        mk.shm_semwait(name, 0, 1.0)
        libc.sem_close(h)
        with pytest.raises(_lib.AtmwfsError) as e:
            mk.shm_semwait(name + "_absent", 0, 0.05)
        assert e.value.status == 1
    finally:
        if path.exists():
            path.unlink()
        for k in range(10):
            libc.sem_unlink(f"{name}_sem{k:02d}".encode())
        libc.sem_unlink(f"{name}_semlog".encode())


def test_shm_double_stream(mk):
    name = f"atmwfs_d{os.getpid()}"
    path = Path(f"/tmp/{name}.im.shm")
    libc = _libc()
    try:
        with mk.ShmImage(name, 4, 4, np.float64) as s:
            s.write(np.arange(16.0).reshape(4, 4))
            raw = path.read_bytes()
            assert MD.unpack_from(raw)[6] == 4
            assert np.array_equal(np.frombuffer(raw, np.float64, 16, MD.size), np.arange(16.0))
    finally:
        if path.exists():
            path.unlink()
        for k in range(10):
            libc.sem_unlink(f"{name}_sem{k:02d}".encode())
        libc.sem_unlink(f"{name}_semlog".encode())


def test_mkwfs_rejects_bad_configuration_before_device_work(mk, tmp_path, monkeypatch):
    from atmosphericturbulencesimul_gb300 import _lib
    monkeypatch.chdir(tmp_path)
    gc = gcm.load("mkwfs")
    (tmp_path / "turbul.prof").write_text(gc.prof)
    # WF_RAW_SIZE / WFsize (integer division) must be 1, 2, 4 or 8 (:1855-1870): 64 / 20 = 3
    (tmp_path / "WFsim.conf").write_text(gc.conf + "WFsize 20\n")
    with pytest.raises(_lib.AtmwfsError) as e:
        mk.mkwfs(1.6)
    assert e.value.status == 1 and "contraction" in str(e.value)
    # a profile layer below the site altitude
    (tmp_path / "WFsim.conf").write_text(gc.conf + "SITE_ALT 100\n")
    with pytest.raises(_lib.AtmwfsError) as e:
        mk.mkwfs(1.6)
    assert e.value.status == 1 and "site altitude" in str(e.value)


def test_hv_profile_matches_reference(mk, tmp_path, monkeypatch):
    """mkHVturbprof: the profile file and conf_turb.txt the reference wrote
    (tests/golden/hv.json), to the printed digits."""
    monkeypatch.chdir(tmp_path)
    g = json.loads((gcm.GOLDEN / "hv.json").read_text())
    for case in g["cases"]:
        ws, r0, site, n = case["args"]
        see = mk.make_hv_profile("prof.txt", ws, r0, site, n)
        got = (tmp_path / "prof.txt").read_text().splitlines()
        want = case["profile"].splitlines()
        assert got[:2] == want[:2] and len(got) == len(want)
        for a, b in zip(got[2:], want[2:]):
            va, vb = np.array(a.split(), float), np.array(b.split(), float)
            assert np.allclose(va, vb, rtol=0, atol=2e-6), (a, b)
        assert abs(float((tmp_path / "conf_turb.txt").read_text()) - float(case["conf_turb"])) < 2e-6
        assert abs(see - float(case["conf_turb"])) < 1e-6
        # the profile reader accepts it
        prof = mk.read_profile(tmp_path / "prof.txt", site)
        assert prof.shape == (n, 8) and abs(prof[:, 1].sum() - 1.0) < 1e-5
