"""Precision study: the multi-layer workload (7 layers 0-16 km, 512^2 pupils,
wavelengths 0.5 / 0.8 / 1.25 / 2.2 um, on axis) with the propagation's FFT
stages in FP32 and in FP16 (per-stage power-of-two scaling); every frame is
compared with the FP64 oracle on the same screens.

By default a few frames on 1024^2 screens keep the test short;
ATMWFS_PRECISION_FRAMES=500 ATMWFS_PRECISION_M=2048 runs the full study and
ATMWFS_PRECISION_REPORT=<file> writes its numbers (JSON).

Bars: FP32, every frame within 0.05 nm rms wrapped OPD error and 1e-4
relative amplitude variance; FP16, the mean wrapped OPD error of every
wavelength within 1.5 nm rms, every frame within 3 nm, amplitude variance
within 1e-2 relative.  (FP16 rounding leaves a phase error of a few
milliradians, so its error in nm grows with the wavelength: about 0.3 nm at
0.5 um and 1.1 nm at 2.2 um on average.)"""
import json
import os
import time

import numpy as np
import pytest

from series_case import Case, make_screens, metrics, run_gpu, run_oracle

pytestmark = pytest.mark.gpu

LAMS = [0.5e-6, 0.8e-6, 1.25e-6, 2.2e-6]


def _case(M):
    rng = np.random.default_rng(0)
    return Case(alt=[0.0, 500.0, 1000.0, 2000.0, 4000.0, 8000.0, 16000.0],
                cn2=[0.45, 0.15, 0.10, 0.10, 0.08, 0.07, 0.05], speed=list(rng.uniform(5.0, 30.0, 7)),
                direction=list(rng.uniform(0.0, 2 * np.pi, 7)), M=M, W=512, Wout=512, fresnel_bin=100.0,
                sci=[(l, 0.0, 0.0) for l in LAMS], ref=False, seed=11)


def _gpu_frames(case, screens, nsteps, fp16):
    """GPU frames as series_case.run_gpu, with the FFT precision selected."""
    from atmosphericturbulencesimul_gb300 import Series
    from series_case import instances
    inst = instances(case)
    s = Series(case.alt, case.cn2, case.speed, case.direction, master_size=case.M, instances=inst,
               pupil_scale=case.pupil, time_step=case.dt, fresnel_bin=case.fresnel_bin, fft_fp16=int(fp16))
    for l, sc in enumerate(screens):
        s.load_screen(l, sc)
    frames = s.run_frames(nsteps)
    # throughput on resident state
    import torch
    s.run(3)
    st = torch.cuda.ExternalStream(s.stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    s.run(20)
    e1.record(st)
    torch.cuda.synchronize()
    fps = 20 * len(inst) / (e0.elapsed_time(e1) * 1e-3)
    s.close()
    return inst, frames, fps


def test_precision_fp32_and_fp16(lib, oracle64):
    nframes = int(os.environ.get("ATMWFS_PRECISION_FRAMES", "8"))
    M = int(os.environ.get("ATMWFS_PRECISION_M", "1024"))
    nsteps = max(1, nframes // len(LAMS))
    case = _case(M)
    screens = make_screens(case, oracle64)
    t0 = time.time()
    _, res, _, _ = run_oracle(case, oracle64, screens, nsteps)
    t_oracle = time.time() - t0
    report = {"workload": f"7 layers, {M}^2 screens, 512^2 pupils, 4 wavelengths, on axis",
              "frames": nsteps * len(LAMS), "oracle_s": round(t_oracle, 1)}
    for name, fp16 in (("fp32", False), ("fp16", True)):
        inst, frames, fps = _gpu_frames(case, screens, nsteps, fp16)
        per = {"wrapped_rms_nm": [], "opd_rms_err_nm": [], "amp_max_err": [], "amp_var_rel": [], "flip_frac": []}
        per_lam = {l: [] for l in LAMS}
        for i, I in enumerate(inst):
            for s in range(nsteps):
                m = metrics(frames[i][0][s], frames[i][1][s], res[s][i][0], res[s][i][1], I.lam)
                for k in per:
                    per[k].append(m[k])
                per_lam[I.lam].append(m["wrapped_rms_nm"])
        report[name] = {"frames_per_s": round(fps, 1),
                        "wrapped_opd_rms_nm": {"mean": float(np.mean(per["wrapped_rms_nm"])),
                                               "max": float(np.max(per["wrapped_rms_nm"]))},
                        "opd_rms_err_nm_mean": float(np.mean(per["opd_rms_err_nm"])),
                        "amp_var_rel": {"mean": float(np.mean(per["amp_var_rel"])),
                                        "max": float(np.max(per["amp_var_rel"]))},
                        "amp_max_err": float(np.max(per["amp_max_err"])),
                        "flip_frac_max": float(np.max(per["flip_frac"])),
                        "wrapped_opd_rms_nm_per_lambda_um": {f"{l * 1e6:.2f}": float(np.mean(v))
                                                             for l, v in per_lam.items()}}
    path = os.environ.get("ATMWFS_PRECISION_REPORT")
    if path:
        with open(path, "w") as f:
            json.dump(report, f, indent=1)
    print(json.dumps(report))
    assert report["fp32"]["wrapped_opd_rms_nm"]["max"] < 0.05, report
    assert report["fp32"]["amp_var_rel"]["max"] < 1e-4, report
    assert report["fp16"]["wrapped_opd_rms_nm"]["max"] < 3.0, report
    assert max(report["fp16"]["wrapped_opd_rms_nm_per_lambda_um"].values()) < 1.5, report
    assert report["fp16"]["amp_var_rel"]["max"] < 1e-2, report
