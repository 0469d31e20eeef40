#!/usr/bin/env python3
"""Generate the golden fixtures of tests/golden/ by running the reference's
own code (the checker build oracle/_ref/atmref, compiled from the reference
sources by oracle/ref/build_ref.py) on small seeded cases.

  fresnel.npz  Fresnel_propagate_wavefront (WFpropagate.c:68) on seeded
               complex_float fields.
  mkwfs.npz    make_AtmosphericTurbulence_wavefront_series (mkwfs <slambda> 0)
  mkwfs_b.npz  on the two profiles of MKWFS_CASES, with master screens
               synthesised by the reference from Philox noise injected into
               its rand()/GSL calls: the master screens it wrote (before its
               r0 renormalisation), the Scoeff of each layer and the start-row
               refraction offsets from its atmosphere model, and its
               lambda_ref and science phase/amplitude cubes.

  psf.npz      the PSF consumers: measure_wavefront_series_expoframes
               (AtmosphericTurbulence.c:6592), PSF_makeChromatPSF
               (psf.c:54) and the image measures of the exposure loop.
  refract.npz  AtmosphereModel_RefractionPath (AtmosphereModel.c:4215) with
               the reference's atmosphere model, and that model's N and
               absorption at the 10 m nodes of its density tables.

Run from the repository root where the reference is mounted:
    python tests/golden/make_golden.py          (every fixture)
    python tests/golden/make_golden.py psf      (psf.npz only)
    python tests/golden/make_golden.py refract  (refract.npz only)
"""
from __future__ import annotations

import json
import os
import re
import subprocess
import sys
import tempfile
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path[:0] = [str(ROOT), str(HERE)]

from oracle import oracle as orc  # noqa: E402
import fits_io as fitsio  # noqa: E402

ATMREF = ROOT / "oracle" / "_ref" / "atmref"

# altitude, relative Cn2, speed, direction, L0, l0, sigma wind, wind outer scale
MKWFS_CASES = {
    # three super-layers, full-frame output, zenith
    "mkwfs": dict(
        M=128, W=64, Wout=64, nframes=3, lam_ref_um=0.5, slam_um=1.6, seeing=0.6875, pupil=0.01, dt=0.001,
        bin=100.0, seed=2024, zangle=0.0, src=(0.0, 0.0),
        profile=[(0.0, 0.5, 10.0, 0.5236, 20.0, 0.01, 1.0, 10.0),
                 (3000.0, 0.3, 20.0, 2.0, 20.0, 0.01, 1.0, 10.0),
                 (10000.0, 0.2, 15.0, 4.0, 20.0, 0.01, 1.0, 10.0)]),
    # layers 0 and 50 m share a super-layer; 100-pixel crop of a 128 grid
    # (5 x 5 science bins); 0.5 rad zenith angle (refraction offsets, slant
    # hops, Cn2 / cos z); off-axis source
    "mkwfs_b": dict(
        M=256, W=128, Wout=100, nframes=3, lam_ref_um=0.5, slam_um=2.2, seeing=0.8, pupil=0.01, dt=0.002,
        bin=100.0, seed=77, zangle=0.5, src=(4.85e-5, -2.4e-5),
        profile=[(0.0, 0.4, 8.0, 0.1, 25.0, 0.01, 1.0, 10.0),
                 (50.0, 0.2, 12.0, 1.0, 25.0, 0.01, 1.0, 10.0),
                 (5000.0, 0.3, 25.0, 3.0, 25.0, 0.01, 1.0, 10.0),
                 (12000.0, 0.1, 30.0, 5.5, 25.0, 0.01, 1.0, 10.0)]),
    # phase only (WAVEFRONT_AMPLITUDE 0), a 64 crop of a 128 grid, two time
    # spans; the profile file has comments, a blank line after a layer (the
    # reference repeats that layer) and a short line (missing columns keep
    # the previous line's values); PUPIL_SCALE appears twice (last wins)
    "mkwfs_c": dict(
        M=128, W=128, Wout=64, nframes=2, ntspan=2, amplitude=0, lam_ref_um=0.5, slam_um=1.25, seeing=0.6875,
        pupil=0.01, dt=0.001, bin=100.0, seed=5, zangle=0.0, src=(0.0, 0.0),
        conf_prefix="PUPIL_SCALE 0.05\n",
        prof_text="# alt cn2 speed dir L0 l0 sigma Lwind\n0 0.5 10 0.5236 20 0.01 1 10\n\n"
                  "2500 0.3 20 2.0 20 0.01 1 10\n  # indented comment\n8000.0 0.2 15 4.0 25\n",
        profile=[(0.0, 0.5, 10.0, 0.5236, 20.0, 0.01, 1.0, 10.0),
                 (0.0, 0.5, 10.0, 0.5236, 20.0, 0.01, 1.0, 10.0),
                 (2500.0, 0.3, 20.0, 2.0, 20.0, 0.01, 1.0, 10.0),
                 (8000.0, 0.2, 15.0, 4.0, 25.0, 0.01, 1.0, 10.0)]),
    # double precision (mkwfs <lambda> 1): _d master screens and BITPIX -64 cubes
    "mkwfs_d": dict(
        M=128, W=64, Wout=32, nframes=2, lam_ref_um=0.5, slam_um=2.2, seeing=0.6875, pupil=0.01, dt=0.001,
        bin=100.0, seed=11, zangle=0.0, src=(0.0, 0.0), precision=1,
        profile=[(0.0, 0.6, 9.0, 1.0, 20.0, 0.01, 1.0, 10.0),
                 (6000.0, 0.4, 21.0, 2.5, 20.0, 0.01, 1.0, 10.0)]),
}


def conf_text(c: dict) -> str:
    kv = [
        ("TURBULENCE_REF_WAVEL", f"{c['lam_ref_um']:f}"), ("TURBULENCE_SEEING", f"{c['seeing']:f}"),
        ("TURBULENCE_PROF_FILE", "turbul.prof"), ("ZENITH_ANGLE", f"{c['zangle']!r}"), ("SOURCE_XPOS", f"{c['src'][0]!r}"),
        ("SOURCE_YPOS", f"{c['src'][1]!r}"), ("TIME_DAY_OF_YEAR", "150"), ("TIME_LOCAL_SOLAR_TIME", "0.0"),
        ("SITE_ALT", "0.0"), ("SITE_LATITUDE", "20.0"), ("SITE_LONGITUDE", "-155.5"), ("CO2_PPM", "400.0"),
        ("SITE_TP_AUTO", "1"), ("SITE_TEMP", "273.15"), ("SITE_PRESS", "1.0"), ("SITE_H2O_METHOD", "1"),
        ("SITE_RH", "30.0"), ("SITE_TPW", "10.0"), ("SITE_PW_SCALEH", "2000.0"), ("WFOUTPUT", "1"),
        ("WF_FILE_PREFIX", "./WF_files/wf_"), ("SHM_OUTPUT", "0"), ("MAKE_SWAVEFRONT", "1"),
        ("SLAMBDA", f"{c['slam_um']:f}"), ("SWF_WRITE2DISK", "1"), ("SWF_FILE_PREFIX", "./WFS_files/wf_"),
        ("SHM_SOUTPUT", "0"), ("SHM_SPREFIX", "outwf"), ("SHM_SOUTPUTM", "2"), ("WFsize", str(c["Wout"])),
        ("PUPIL_SCALE", f"{c['pupil']:f}"), ("REALTIME", "0"), ("REALTIMEFACTOR", "1.0"),
        ("WFTIME_STEP", f"{c['dt']:f}"), ("TIME_SPAN", f"{c['dt'] * c['nframes']:f}"), ("NB_TSPAN", str(c.get("ntspan", 1))),
        ("SIMTDELAY", "0"), ("WAITFORSEM", "0"), ("WAITSEMIMNAME", "wfsimwait"),
        ("WF_RAW_SIZE", str(c["W"])), ("MASTER_SIZE", str(c["M"])), ("WAVEFRONT_AMPLITUDE", str(c.get("amplitude", 1))),
        ("FRESNEL_PROPAGATION", "1"), ("FRESNEL_PROPAGATION_BIN", f"{c['bin']:f}"),
    ]
    return "\n".join(f"{k:25s} {v:>20s}  # generated" for k, v in kv) + "\n"


def run(cmd, cwd, env=None):
    r = subprocess.run(cmd, cwd=cwd, env=env, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(" ".join(map(str, cmd)) + "\n" + r.stdout[-2000:] + r.stderr[-2000:])
    return r.stdout


def make_fresnel() -> dict:
    out = {}
    cases = [(64, 0.01, 3000.0, 1.6e-6), (128, 0.01, 8000.0, 0.5e-6)]
    with tempfile.TemporaryDirectory() as td:
        for k, (n, dx, z, lam) in enumerate(cases):
            rng = np.random.default_rng(100 + k)
            a = np.exp(1j * rng.standard_normal((n, n)) * 2).astype(np.complex64)
            a.tofile(Path(td) / "in.c64")
            run([str(ATMREF), "fresnel", str(n), repr(dx), repr(z), repr(lam), "in.c64", "out.c64"], td)
            b = np.fromfile(Path(td) / "out.c64", np.complex64).reshape(n, n)
            out[f"in{k}"] = a
            out[f"out{k}"] = b
            out[f"par{k}"] = np.array([n, dx, z, lam])
    return out


LAYER_LOG = re.compile(r"Turbulence layer (\d+) : alt = (\S+) m\s+CN2 = (\S+)\s+V = (\S+) m/s\s+Angle = (\S+) rad"
                       r"\s+outerscale = (\S+) m\s+innerscale = (\S+) m\s+sigmaWind = (\S+) m/s\s+Lwind = (\S+) m")


def make_mkwfs(c: dict) -> dict:
    M, L = c["M"], len(c["profile"])
    prec = c.get("precision", 0)
    ntspan = c.get("ntspan", 1)
    amp = c.get("amplitude", 1)
    o64 = orc.Oracle(64)
    conf = c.get("conf_prefix", "") + conf_text(c)
    prof = c.get("prof_text") or ("# alt cn2 speed dir L0 l0 sigmawind Lwind\n" + "".join(
        " ".join(f"{v:g}" for v in row) + "\n" for row in c["profile"]))
    with tempfile.TemporaryDirectory() as td:
        td = Path(td)
        (td / "WF_files").mkdir()
        (td / "WFS_files").mkdir()
        (td / "WFsim.conf").write_text(conf)
        (td / "turbul.prof").write_text(prof)
        # the wind-scatter series is unused by the loop: pre-create it
        for l in range(L):
            fitsio.write(td / f"wspeed_{l:03d}.fits", np.zeros((3, 8), np.float32))
        noise = []
        for l in range(L):
            u, g = o64.screen_noise(c["seed"], l, M)
            noise += [u, g]
        np.concatenate([x.ravel() for x in noise]).astype(np.float32).tofile(td / "noise.f32")
        env = dict(os.environ, ATMREF_NOISE=str(td / "noise.f32"), ATMREF_NOISE_M=str(M))
        log = run([str(ATMREF), "mkwfs", f"{c['slam_um']}", str(prec)], td, env)
        logprof = np.array([[float(x) for x in m.groups()[1:]] for m in LAYER_LOG.finditer(log)])
        sfx = "f" if prec == 0 else "d"
        screens = [fitsio.read(td / f"t{l:03d}_{M}_{sfx}.fits") for l in range(L)]
        lam_pm = int(c["slam_um"] * 1e-6 * 1e12 + 0.5)
        cubes = {}
        for key, pre in (("ref", "WF_files/wf_"), ("sci", "WFS_files/wf_")):
            for q in ("pha", "amp") if amp else ("pha",):
                cubes[f"{key}_{q}"] = np.concatenate(
                    [fitsio.read(td / f"{pre}{t:08d}.{lam_pm:09d}.{q}.fits") for t in range(ntspan)])
        # Scoeff(h) = CONF_LAMBDA/SLAMBDA * N(h, SLAMBDA)/N(h, CONF_LAMBDA) from the
        # reference's atmosphere model, with its float operands (:2661-2663)
        lam_ref = np.float32(c["lam_ref_um"] * 1e-6)
        slam = c["slam_um"] * 1e-6
        args = []
        for row in c["profile"]:
            args += [repr(row[0]), repr(float(lam_ref)), repr(row[0]), repr(slam)]
        txt = run([str(ATMREF), "stdN", "WFsim.conf", repr(slam)] + args, td)
        vals = [float(line.split()[3]) for line in txt.splitlines() if line.startswith("STDN")]
        scoeff = []
        for l in range(L):
            n_ref, n_sci = np.float32(vals[2 * l]), np.float32(vals[2 * l + 1])
            scoeff.append(float(lam_ref) / slam * float(n_sci) / float(n_ref))
        # the start-row refraction offsets (RoffsetS - Roffset, metres)
        txt = run([str(ATMREF), "roffset", "WFsim.conf", repr(slam), repr(float(lam_ref)), repr(slam),
                   repr(c["zangle"])] + [repr(row[0]) for row in c["profile"]], td)
        roffset = [float(line.split()[2]) for line in txt.splitlines() if line.startswith("ROFF")]
    out = dict(screens=np.stack(screens), scoeff=np.array(scoeff), roffset=np.array(roffset), **cubes,
               profile=np.array(c["profile"]), logprof=logprof, conf=np.array(conf), prof=np.array(prof),
               params=np.array([M, c["W"], c["Wout"], c["nframes"], c["lam_ref_um"], c["slam_um"], c["seeing"],
                                c["pupil"], c["dt"], c["bin"], c["seed"], c["zangle"], c["src"][0], c["src"][1],
                                prec, ntspan, amp]))
    return out


# configuration-file reads: text with repeated keywords, a bare keyword
# line, tabs, blank lines, comments and keyword prefixes
CONF_TEXT = """# comment line
PUPIL_SCALE 0.02
WFsize\t\t64   # trailing comment

TURBULENCE_SEEING 0.8
TURBULENCE_SEEING
  MASTER_SIZE 1024
WFsizeX 9
PUPIL_SCALE 0.01 extra tokens
SLAMBDA 1.6
SLAMBDA
EMPTYVALUE
"""
CONF_KEYS = ["PUPIL_SCALE", "WFsize", "TURBULENCE_SEEING", "MASTER_SIZE", "WFsizeX", "SLAMBDA", "EMPTYVALUE",
             "MISSING", "#", "comment"]


def make_conf() -> dict:
    with tempfile.TemporaryDirectory() as td:
        (Path(td) / "t.conf").write_text(CONF_TEXT)
        txt = run([str(ATMREF), "conf", "t.conf"] + CONF_KEYS, td)
    rows = []
    for line in txt.splitlines():
        if line.startswith("CONF\t"):
            f = line.split("\t")
            rows.append([f[1], int(f[2]), int(f[3]), f[4] if len(f) > 4 else ""])
    return {"text": CONF_TEXT, "reads": rows}


# Hufnagel-Valley profiles: (wind speed, r0 at 550 nm, site altitude, layers)
HV_CASES = [(10.0, 0.15, 4200.0, 10), (25.0, 0.08, 0.0, 7), (5.0, 0.3, 2500.0, 20)]


def make_hv() -> dict:
    out = []
    with tempfile.TemporaryDirectory() as td:
        for ws, r0, site, n in HV_CASES:
            run([str(ATMREF), "hv", repr(ws), repr(r0), repr(site), str(n), "prof.txt"], td)
            out.append({"args": [ws, r0, site, n], "profile": (Path(td) / "prof.txt").read_text(),
                        "conf_turb": (Path(td) / "conf_turb.txt").read_text()})
    return {"cases": out}


def _pupil(n: int, rin: float = 0.0) -> np.ndarray:
    y, x = np.mgrid[0:n, 0:n] - (n / 2 - 0.5)
    r = np.hypot(x, y) / (n / 2)
    return ((r < 1.0) & (r >= rin)).astype(np.float32)


def _phase(n: int, seed: int, rms: float) -> np.ndarray:
    """A smooth seeded phase screen (k^-11/6 filtered noise), rad."""
    rng = np.random.default_rng(seed)
    k = np.hypot(*np.meshgrid(np.fft.fftfreq(n), np.fft.fftfreq(n)))
    k[0, 0] = 1.0
    f = (rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))) * k ** (-11 / 6)
    f[0, 0] = 0.0
    p = np.fft.ifft2(f).real
    return (p / p.std() * rms).astype(np.float32)


PSF_EXPO = dict(W=64, nframes=8, ntspan=2, etime=0.003, dt=0.001)


def make_psf() -> dict:
    """PSF consumers: the exposure measures on three images, the chromatic
    PSF on two pupils, and the exposure command on a two-span series whose
    amplitude cube equals the pupil in every frame (so that the reference's
    uninitialised amplitude_on selects the same field either way)."""
    out = {}
    with tempfile.TemporaryDirectory() as td:
        d = Path(td)
        # measures
        imgs = []
        pup = _pupil(64)
        f = np.zeros((128, 128), np.complex128)
        f[32:96, 32:96] = pup * np.exp(1j * _phase(64, 1, 1.0))
        imgs.append(np.abs(np.fft.fftshift(np.fft.fft2(f))) ** 2)
        y, x = np.mgrid[0:64, 0:64]
        imgs.append(np.exp(-((x - 37.3) ** 2 + (y - 28.6) ** 2) / (2 * 3.1 ** 2)) * 100.0 +
                    np.random.default_rng(3).uniform(0.0, 0.5, (64, 64)))
        f = np.zeros((128, 128), np.complex128)
        f[32:96, 32:96] = _pupil(64, 0.3) * np.exp(1j * _phase(64, 2, 2.5))
        imgs.append(np.abs(np.fft.fftshift(np.fft.fft2(f))) ** 2)
        for k, im in enumerate(imgs):
            im = im.astype(np.float32)
            n = im.shape[0]
            im.tofile(d / "in.f32")
            txt = run([str(ATMREF), "measure", str(n), "in.f32", "g.f32"], td)
            xc, yc, fw, ee = [float(v) for v in next(l for l in txt.splitlines() if l.startswith("MEAS")).split()[1:]]
            out[f"meas_in{k}"] = im
            out[f"meas_gauss{k}"] = np.fromfile(d / "g.f32", np.float32).reshape(n, n)
            out[f"meas_val{k}"] = np.array([xc, yc, fw, ee])
        # chromatic PSF
        for k, (n, c1, c2, ns, apo, rms) in enumerate([(64, 0.8, 1.25, 5, 0.2, 0.7), (128, 1.0, 1.6, 4, 0.0, 1.5)]):
            amp, pha = _pupil(n // 2 if n == 128 else n), None
            amp = np.pad(amp, (n - amp.shape[0]) // 2) if amp.shape[0] < n else amp
            pha = (_phase(n, 10 + k, rms) * (amp > 0)).astype(np.float32)
            amp.astype(np.float32).tofile(d / "amp.f32")
            pha.tofile(d / "pha.f32")
            run([str(ATMREF), "chromat", str(n), "amp.f32", "pha.f32", repr(c1), repr(c2), str(ns), repr(apo),
                 "cpsf.f32"], td)
            out[f"chromat_amp{k}"] = amp.astype(np.float32)
            out[f"chromat_pha{k}"] = pha
            out[f"chromat_par{k}"] = np.array([n, c1, c2, ns, apo])
            out[f"chromat_out{k}"] = np.fromfile(d / "cpsf.f32", np.float32).reshape(n, n)
        # exposure command
        c = PSF_EXPO
        W = c["W"]
        (d / "WFS_files").mkdir()
        pup = _pupil(W)
        fitsio.write(d / "pupil.fits", pup)
        cube_cfg = dict(MKWFS_CASES["mkwfs"], Wout=W, W=W, nframes=c["nframes"], ntspan=c["ntspan"], dt=c["dt"])
        (d / "WFsim.conf").write_text(conf_text(cube_cfg) + "PUPIL_AMPL_FILE pupil.fits\n")
        phs = []
        for t in range(c["ntspan"]):
            ph = np.stack([_phase(W, 100 * t + f, 1.2) * pup for f in range(c["nframes"])]).astype(np.float32)
            phs.append(ph)
            fitsio.write(d / "WFS_files" / f"wf_{t:08d}.{1650000:09d}.pha.fits", ph)
            fitsio.write(d / "WFS_files" / f"wf_{t:08d}.{1650000:09d}.amp.fits",
                         np.repeat(pup[None], c["nframes"], 0))
        txt = run([str(ATMREF), "expo", repr(c["etime"]), "expo.log"], td)
        m = re.search(r"FWHM = (\S+) arcseconds", txt.splitlines()[-1] if txt else "")
        out["expo_pupil"] = pup
        out["expo_pha"] = np.stack(phs)
        out["expo_conf"] = np.array(conf_text(cube_cfg) + "PUPIL_AMPL_FILE pupil.fits\n")
        out["expo_log"] = np.array((d / "expo.log").read_text())
        out["expo_final_fwhm"] = np.array(float(m.group(1)) if m else np.nan)
        k = 0
        while (d / f"PSF{k:04d}.fits").exists():
            out[f"expo_psf{k}"] = fitsio.read(d / f"PSF{k:04d}.fits").astype(np.float32)
            k += 1
        out["expo_final"] = fitsio.read(d / "PSF").astype(np.float32)
        out["expo_par"] = np.array([c["etime"], c["dt"], W, c["nframes"], c["ntspan"]])
    return out


# (lambda, zenith angle, site altitude): refraction ray traces
REFRACT_CASES = [(0.55e-6, 0.5, 0.0), (1.6e-6, 1.0, 4200.0), (0.4e-6, 1.2, 0.0)]
REFRACT_DH, REFRACT_N = 10.0, 10001


def make_refract() -> dict:
    """AtmosphereModel_RefractionPath with the reference's atmosphere model,
    and that model's N and absorption at the nodes of its 10 m density
    tables (what a caller's table model reproduces), plus the path file of
    the first case."""
    out = {}
    with tempfile.TemporaryDirectory() as td:
        d = Path(td)
        for k, (lam, za, site) in enumerate(REFRACT_CASES):
            conf = re.sub(r"^SITE_ALT\s+\S+", f"SITE_ALT {site:.1f}", conf_text(MKWFS_CASES["mkwfs"]), flags=re.M)
            (d / "WFsim.conf").write_text(conf)
            txt = run([str(ATMREF), "refract", "WFsim.conf", repr(lam), repr(lam), repr(za), "1" if k == 0 else "0"], td)
            r, tr, sa = [float(v) for v in next(l for l in txt.splitlines() if l.startswith("REFR")).split()[1:]]
            if k == 0:   # before the next model set-up renames the file
                out["path0"] = np.array((d / "refractpath.txt").read_text())
            run([str(ATMREF), "ntable", "WFsim.conf", repr(lam), repr(lam), repr(REFRACT_DH), str(REFRACT_N), "t.bin"], td)
            raw = (d / "t.bin").read_bytes()
            out[f"N{k}"] = np.frombuffer(raw[:4 * REFRACT_N], np.float32).copy()
            out[f"K{k}"] = np.frombuffer(raw[4 * REFRACT_N:], np.float64).copy()
            out[f"case{k}"] = np.array([lam, za, sa, r, tr])
    out["table"] = np.array([REFRACT_DH, REFRACT_N])
    return out


def main():
    if not ATMREF.exists():
        sys.path.insert(0, str(ROOT / "oracle" / "ref"))
        import build_ref
        build_ref.build()
    if sys.argv[1:] == ["psf"]:
        np.savez_compressed(HERE / "psf.npz", **make_psf())
        print("wrote psf.npz")
        return
    if sys.argv[1:] == ["refract"]:
        np.savez_compressed(HERE / "refract.npz", **make_refract())
        print("wrote refract.npz")
        return
    (HERE / "conf.json").write_text(json.dumps(make_conf(), indent=1) + "\n")
    (HERE / "hv.json").write_text(json.dumps(make_hv(), indent=1) + "\n")
    np.savez_compressed(HERE / "fresnel.npz", **make_fresnel())
    np.savez_compressed(HERE / "psf.npz", **make_psf())
    np.savez_compressed(HERE / "refract.npz", **make_refract())
    for name, case in MKWFS_CASES.items():
        np.savez_compressed(HERE / f"{name}.npz", **make_mkwfs(case))
    print("wrote", ", ".join(["conf.json", "hv.json", "fresnel.npz"] + [f"{n}.npz" for n in MKWFS_CASES]))


if __name__ == "__main__":
    main()
