#!/usr/bin/env python3
"""Calibrate the CPU baseline: time the reference's own frame loop (the
checker build oracle/_ref/atmref: the reference's C sources with the shim
FFT of this directory) beside the oracle's float port of the same loop, one
thread each, on the 7-layer profile of the batched benchmark.

For each grid W the reference runs `mkwfs` twice on the same 2048^2 master
screens (written here from the oracle's synthesis, so the reference loads
them instead of synthesising its own) with n1 and n2 frames; the difference
of the two wall times over n2 - n1 is the loop time of one step
(AtmosphericTurbulence.c:2561 onward), which computes a lambda-ref frame and
a science frame.  The port computes the same two frames per step.

Checker infrastructure: run where the reference is mounted, after
build_ref.py.  Prints one JSON line.
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
ROOT = HERE.parent.parent
sys.path[:0] = [str(ROOT), str(ROOT / "tests" / "golden")]

from oracle import oracle as orc  # noqa: E402
import fits_io  # noqa: E402
from make_golden import conf_text  # noqa: E402

ATMREF = HERE.parent / "_ref" / "atmref"


def profile():
    from bench import workload
    wl = workload("batched")
    rows = [(a, c, float(s), float(d), 20.0, 0.01, 1.0, 10.0)
            for a, c, s, d in zip(wl["alt"], wl["cn2"], wl["speed"], wl["direction"])]
    return wl, rows


def time_reference(W: int, screens, rows, n1: int = 1, n2: int = 4) -> float:
    """Seconds per step of the reference loop at grid W."""
    M = screens[0].shape[0]
    ts = []
    for nf in (n1, n2):
        c = dict(M=M, W=W, Wout=W, nframes=nf, lam_ref_um=0.5, slam_um=1.6, seeing=0.6875, pupil=0.01, dt=0.001,
                 bin=100.0, zangle=0.0, src=(0.0, 0.0))
        with tempfile.TemporaryDirectory() as td:
            td = Path(td)
            (td / "WF_files").mkdir()
            (td / "WFS_files").mkdir()
            (td / "WFsim.conf").write_text(conf_text(c))
            (td / "turbul.prof").write_text("# alt cn2 speed dir L0 l0 sigmawind Lwind\n" + "".join(
                " ".join(f"{v:g}" for v in r) + "\n" for r in rows))
            for l, s in enumerate(screens):
                fits_io.write(td / f"t{l:03d}_{M}_f.fits", s)
                fits_io.write(td / f"wspeed_{l:03d}.fits", np.zeros((3, 8), np.float32))
            env = dict(os.environ, OMP_NUM_THREADS="1")
            t0 = time.perf_counter()
            r = subprocess.run([str(ATMREF), "mkwfs", "1.6", "0"], cwd=td, env=env, capture_output=True, text=True)
            ts.append(time.perf_counter() - t0)
            if r.returncode != 0:
                raise RuntimeError(r.stdout[-2000:] + r.stderr[-2000:])
    return (ts[1] - ts[0]) / (n2 - n1)


def time_port(W: int, screens, wl, nsteps: int = 3) -> float:
    """Seconds per step of the oracle's float port (lambda-ref + science frame)."""
    o32 = orc.Oracle(32)
    o32.set_threads(1)
    L = len(wl["alt"])
    cn2 = np.asarray(wl["cn2"]) / np.sum(wl["cn2"])
    salt, sidx = o32.superlayers(wl["alt"], cn2, wl["fresnel_bin"])
    x, y, vx, vy = orc.init_positions(wl["M"], wl["alt"], wl["speed"], wl["direction"], wl["pupil"])
    xc, yc = [0] * L, [0] * L
    sc = np.full(L, float(np.float32(0.5e-6)) / 1.6e-6)
    t0 = time.perf_counter()
    for _ in range(nsteps):
        orc.step_positions(x, y, xc, yc, vx, vy, wl["dt"], wl["M"])
        ph, f = o32.frame(screens, x, y, None, sidx, salt, 0.01, 0.0, float(np.float32(0.5e-6)), W)
        o32.output_ref(ph, f, W)
        ph, f = o32.frame(screens, x, y, sc, sidx, salt, 0.01, 0.0, 1.6e-6, W)
        o32.output_sci(ph, f, W)
    return (time.perf_counter() - t0) / nsteps


def fft_calibration(n: int = 1024, reps: int = 5) -> dict:
    """The port's 2-D FFT against numpy's pocketfft on one thread."""
    o32 = orc.Oracle(32)
    o32.set_threads(1)
    a = (np.random.default_rng(0).standard_normal((n, n)) + 1j).astype(np.complex64)
    o32.fft2d(a, -1)
    t0 = time.perf_counter()
    for _ in range(reps):
        o32.fft2d(a, -1)
    tp = (time.perf_counter() - t0) / reps
    np.fft.fft2(a)
    t0 = time.perf_counter()
    for _ in range(reps):
        np.fft.fft2(a)
    tn = (time.perf_counter() - t0) / reps
    return {"n": n, "port_ms": round(tp * 1e3, 2), "numpy_pocketfft_ms": round(tn * 1e3, 2)}


def main():
    if not ATMREF.exists():
        print(json.dumps({"unavailable": f"{ATMREF} not built (run oracle/ref/build_ref.py where the reference is mounted)"}))
        return
    wl, rows = profile()
    o32 = orc.Oracle(32)
    o32.set_threads(os.cpu_count() or 1)
    M = wl["M"]
    screens = []
    for l in range(len(rows)):
        u, g = o32.screen_noise(1000 + l, 0, M)
        screens.append(o32.master_screen(u, g, 20.0 / 0.01, 0.01 / 0.01)[0].astype(np.float32))
    sizes = [int(a) for a in sys.argv[1:]] or [256, 512, 1024]
    out = {"host": os.uname().machine, "cores_used": 1, "profile": "7 layers (batched benchmark)", "master": M,
           "per_step": "one lambda-ref frame + one science frame", "grids": {}}
    for W in sizes:
        tr = time_reference(W, screens, rows)
        tp = time_port(W, screens, wl)
        out["grids"][str(W)] = {"reference_loop_s_per_step": round(tr, 4), "port_s_per_step": round(tp, 4),
                                "port_over_reference": round(tp / tr, 3)}
    out["fft"] = fft_calibration()
    print(json.dumps(out))


if __name__ == "__main__":
    main()
