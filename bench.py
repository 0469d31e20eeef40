#!/usr/bin/env python3
"""Wavefront-series benchmark: frames/s per (wavelength, direction) instance.

Default workload ("batched"): the 7-layer profile (0, 0.5, 1, 2, 4, 8, 16 km;
Cn2 0.45/0.15/0.10/0.10/0.08/0.07/0.05; seeded winds 5-30 m/s, seeded
directions), 2048^2 float32 master screens, 16 wavelengths log-spaced
0.5-2.4 um x 9 directions (3 x 3 grid, 10 arcsec spacing) = 144 instances
with seeded propagation grids from {256, 512, 1024}, science output with
the bin unwrap; one step = one frame of every instance.

  value : frames/s with screens and state resident in HBM (CUDA events on
          the engine stream around K steps);
  e2e   : the same through the C ABI with host buffers: per-step H2D of the
          layer positions and D2H of every frame (pha + amp) into pinned memory.
Multi-GPU (torchrun): every rank runs its own replica of the workload
(weak scaling, no collective on the data path).

--impl reference times the reference's float path as restated by the CPU
oracle port (the reference itself needs FFTW/GSL/cfitsio, absent here) on
all host cores, on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
import csv
import io
import json
import os
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

ARCSEC = np.pi / 180.0 / 3600.0


def workload(name: str, seed: int = 0) -> dict:
    rng = np.random.default_rng(seed)
    alt = [0.0, 500.0, 1000.0, 2000.0, 4000.0, 8000.0, 16000.0]
    cn2 = [0.45, 0.15, 0.10, 0.10, 0.08, 0.07, 0.05]
    speed = list(rng.uniform(5.0, 30.0, 7))
    direction = list(rng.uniform(0.0, 2 * np.pi, 7))
    base = dict(alt=alt, cn2=cn2, speed=speed, direction=direction, M=2048, pupil=0.01, dt=0.001,
                lam_ref=0.5e-6, seeing=0.5e-6 / 0.15 / ARCSEC, fresnel_bin=100.0, L0=20.0, l0=0.01)
    if name == "batched":
        lams = list(0.5e-6 * (2.4 / 0.5) ** (np.arange(16) / 15.0))
        dirs = [(dx * 10 * ARCSEC, dy * 10 * ARCSEC) for dy in (-1, 0, 1) for dx in (-1, 0, 1)]
        sizes = list(rng.choice([256, 512, 1024], size=len(lams) * len(dirs)))
        inst = []
        k = 0
        for d in dirs:
            for lam in lams:
                inst.append(dict(lam=float(lam), src=d, W=int(sizes[k])))
                k += 1
        base.update(name="batched: 7 layers, 2048^2 screens, 16 lambda x 9 directions, W mixed 256/512/1024",
                    inst=inst, steps_nominal=5000)
    elif name == "single":
        # one turbulent layer at 5 km over a Cn2 = 0 layer at the ground, so
        # that the field is propagated to the ground (the reference never
        # propagates below its lowest super-layer)
        base.update(alt=[0.0, 5000.0], cn2=[0.0, 1.0], speed=[0.0, 10.0], direction=[0.0, np.deg2rad(30.0)], M=1024,
                    inst=[dict(lam=1.6e-6, src=(0.0, 0.0), W=256)], steps_nominal=1000,
                    name="single: 1 layer at 5 km, 1024^2 screen, 256^2 pupil, 1.6 um")
    elif name == "multilayer":
        inst = [dict(lam=l, src=(0.0, 0.0), W=512) for l in (0.5e-6, 0.8e-6, 1.25e-6, 2.2e-6)]
        base.update(name="multilayer: 7 layers, 2048^2 screens, 512^2 pupils, 4 lambda, on-axis", inst=inst,
                    steps_nominal=2000)
    elif name == "w1024":
        inst = [dict(lam=l, src=(0.0, 0.0), W=1024) for l in (0.5e-6, 0.8e-6, 1.25e-6, 2.2e-6)]
        base.update(name="w1024: 7 layers, 2048^2 screens, 1024^2 pupils, 4 lambda, on-axis", inst=inst,
                    steps_nominal=2000)
    elif name == "prof1024":
        lams = list(0.5e-6 * (2.4 / 0.5) ** (np.arange(16) / 15.0))
        inst = [dict(lam=float(l), src=(0.0, 0.0), W=1024) for l in lams]
        base.update(name="prof1024: 7 layers, 2048^2 screens, 1024^2 pupils, 16 lambda (profiling case)", inst=inst,
                    steps_nominal=100)
    else:
        raise SystemExit(f"unknown workload {name}")
    return base


def num_hops(wl: dict) -> int:
    """Propagation hops per frame of the workload's profile (host grouping)."""
    from atmosphericturbulencesimul_gb300.engine import layer_planes
    return len(layer_planes(wl["alt"], wl["cn2"], wl["fresnel_bin"])[3])


def make_series(wl: dict, ring: int = 1, fft_fp16: bool = False):
    from atmosphericturbulencesimul_gb300 import MODE_SCI, InstanceSpec, Series, master_screen
    from atmosphericturbulencesimul_gb300.refractivity import scoeff
    L = len(wl["alt"])
    specs = [InstanceSpec(lam=I["lam"], mode=MODE_SCI, src_x=I["src"][0], src_y=I["src"][1], wf_raw_size=I["W"],
                          wf_size=I["W"], scoeff=scoeff(wl["lam_ref"], I["lam"], L)) for I in wl["inst"]]
    s = Series(wl["alt"], wl["cn2"], wl["speed"], wl["direction"], master_size=wl["M"], instances=specs,
               pupil_scale=wl["pupil"], time_step=wl["dt"], fresnel_bin=wl["fresnel_bin"], ring=ring,
               fft_fp16=int(fft_fp16))
    M = wl["M"]
    screens = []
    for l in range(L):
        s1, _, _ = master_screen(1000 + l, M, wl["L0"] / wl["pupil"], wl["l0"] / wl["pupil"])
        screens.append(s1)
        s.load_screen(l, s1)
    s.normalize(np.float32(wl["lam_ref"]), np.float32(wl["seeing"]))
    return s, screens


class ClockSampler:
    """nvidia-smi clock / throttle sampling during the timed region: samples
    every 20 ms from before the region (the tool takes a moment to start) to
    after it; only samples stamped inside a region count (mark() opens and
    closes one)."""
    Q = ("timestamp,index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.regions = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "20"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            time.sleep(1.0)  # the first samples come after the tool has started
        except Exception:
            self.proc = None
        return self

    def mark(self, start: bool) -> None:
        import datetime
        now = datetime.datetime.now()
        if start:
            self.regions.append([now, None])
        elif self.regions:
            self.regions[-1][1] = now

    def __exit__(self, *exc):
        self.out = ""
        if self.proc:
            time.sleep(0.1)
            self.proc.terminate()
            try:
                self.out, _ = self.proc.communicate(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self) -> dict:
        import datetime
        rows = [r for r in csv.reader(io.StringIO(getattr(self, "out", "") or "")) if len(r) >= 10]
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"]}

        def stamp(r):
            try:
                return datetime.datetime.strptime(r[0].strip(), "%Y/%m/%d %H:%M:%S.%f")
            except ValueError:
                return None
        inside = [r for r in rows if stamp(r) and any(a <= stamp(r) <= (b or a) for a, b in self.regions)]
        use = inside or rows
        sm = [float(r[2]) for r in use if r[2].strip().replace(".", "").isdigit()]
        mx = [float(r[3]) for r in use if r[3].strip().replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in use for k in range(4) if r[6 + k].strip().lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(use),
                "window": "inside the timed regions" if inside else "whole sampling span (none stamped inside)"}


def peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": d["hbm_gbs"], "bf16_tflops": d.get("bf16_tflops"), "source": "measured"}
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "source": "fallback"}


def surrogate_section(pairs: int = 50000) -> dict:
    """The learned surrogate at 256^2 (7 layers): inference frames/s and
    tensor-core roofline, and its held-out error against the plain Fresnel
    path beside that of the geometric field.  Uses the model file named by
    ATMWFS_FNO_MODEL when present, else trains one on `pairs` plain-path pairs."""
    import torch
    from atmosphericturbulencesimul_gb300 import fno as F
    t0 = time.time()
    path = os.environ.get("ATMWFS_FNO_MODEL")
    src = None
    if path and os.path.exists(path):
        model = F.Surrogate(path=path)
        how = f"model file {os.path.basename(path)}"
    else:
        model = F.Surrogate(F.FnoConfig(), seed=0)
        src = F.PairSource(count=32, grid=256, seed=1)
        F.train(model, src, pairs, batch=8, lr=1e-3)
        how = f"trained here on {pairs} plain-path pairs"
    t_train = time.time() - t0
    test = F.PairSource(count=32, grid=256, seed=1001)
    ev = F.evaluate(model, test, steps=2, batch=8)
    ev_fp64 = surrogate_vs_fp64(model, test)
    # inference throughput on resident inputs, batch 16
    x, *_ = test.step()
    xb = torch.cat([x, x])[:16].contiguous()
    out = torch.empty((16, 2, 256, 256), device="cuda")
    for _ in range(3):
        model.forward(xb, out)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record()
    reps = 10
    torch.cuda.nvtx.range_push("timed")  # profilers can select the timed batches
    for _ in range(reps):
        model.forward(xb, out)
    e1.record()
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    ms = e0.elapsed_time(e1) / reps
    fps = 16 / (ms * 1e-3)
    # the plain path on the same 32 instances at 256^2
    s = test.series
    s.run(3)
    e0.record(torch.cuda.ExternalStream(s.stream))
    s.run(20)
    e1.record(torch.cuda.ExternalStream(s.stream))
    torch.cuda.synchronize()
    plain_fps = 20 * test.count / (e0.elapsed_time(e1) * 1e-3)
    pk = peaks()
    tflops = F.frame_flops(model.cfg) * fps / 1e12
    gbs = F.frame_bytes(model.cfg) * fps / 1e9
    # the products are thin (K or N of 64..256 against 65536 pixels): their
    # arithmetic intensity is far below the BF16 ridge, so HBM bounds them
    roof = {"bound": "hbm", "achieved": round(gbs, 1), "peak": pk["hbm_gbs"], "unit": "GB/s",
            "frac": round(gbs / pk["hbm_gbs"], 4), "bytes_per_frame": F.frame_bytes(model.cfg),
            "tensor": {"achieved": round(tflops, 2), "peak": pk.get("bf16_tflops"), "unit": "TFLOP/s",
                       "frac": round(tflops / pk["bf16_tflops"], 4) if pk.get("bf16_tflops") else None,
                       "flops_per_frame": F.frame_flops(model.cfg)},
            "intensity_flop_per_byte": round(F.frame_flops(model.cfg) / F.frame_bytes(model.cfg), 1),
            "peak_source": pk["source"]}
    res = {"value": round(fps, 1), "unit": "frames/s", "grid": 256, "batch": 16, "ms_per_batch": round(ms, 3),
           "model": {k: v for k, v in model.cfg.__dict__.items()}, "params": model.num_params, "weights": "bf16 (fp32 master)",
           "how": how, "setup_s": round(t_train, 1), "roofline": roof, "plain_same_grid_fps": round(plain_fps, 1),
           "error_vs_plain": {k: {m: round(v, 5) for m, v in d.items()} for k, d in ev.items()},
           "error_vs_fp64": ev_fp64,
           "error_note": "held-out seeds; 'model' = surrogate, 'geometric' = exp(i phi) without diffraction; "
                         "opd_wrms_nm weights the wrapped phase error by the plain path's intensity"}
    test.close()
    if src:
        src.close()
    model.close()
    return res


def surrogate_vs_fp64(model, test, n: int = 8) -> dict:
    """Held-out frames of the surrogate and of the plain FP32 path against the
    FP64 oracle's field (same screens, positions and Scoeff as the engine that
    made the surrogate's inputs): wrapped OPD rms (nm) and amplitude rms,
    averaged over the first n instances of one more step.  The checker runs
    outside every timed region."""
    import torch
    from atmosphericturbulencesimul_gb300 import fno as F
    from oracle import oracle as orc
    o64 = orc.Oracle(64)
    o64.set_threads(os.cpu_count() or 1)
    x, _, phi, amp, pha, lam = test.step()
    out = model.forward(x[:n].contiguous())
    a_m, p_m = F.assemble(out, phi[:n].contiguous())
    torch.cuda.synchronize()
    s = test.series
    screens = [s.read_screen(l) for l in range(test.L)]
    salt, sidx = o64.superlayers(test.alt, np.asarray(test.cn2) / np.sum(test.cn2), test.fresnel_bin)
    acc = {"surrogate": [], "plain": []}
    for i in range(n):
        xi, yi = s.positions(i)
        sc = np.asarray(s.instances[i].scoeff, np.float32).astype(np.float64)
        li = float(s.instances[i].lam)
        _, fld = o64.frame(screens, xi, yi, sc, sidx, salt, float(np.float32(test.pupil)), 0.0, li, test.G)
        ao, po = np.abs(fld), np.angle(fld)
        nm = li / (2 * np.pi) * 1e9
        for key, (a, p_) in (("surrogate", (a_m[i], p_m[i])), ("plain", (amp[i], pha[i]))):
            a = a.double().cpu().numpy()
            d = np.angle(np.exp(1j * (p_.double().cpu().numpy() - po)))
            acc[key].append((float(np.sqrt(np.mean(d ** 2)) * nm), float(np.sqrt(np.mean((a - ao) ** 2)))))
    return {k: {"opd_wrapped_rms_nm": float(f"{np.mean([e[0] for e in v]):.4g}"),
                "amp_rms": float(f"{np.mean([e[1] for e in v]):.4g}"), "frames": n} for k, v in acc.items()}


def launch_gap_section(wl: dict, steps: int = 50) -> dict:
    """Launch gaps of the smallest grid class: its instances alone in a
    context, the device time of whole steps (one graph each) against the sum
    of its kernels timed one by one.  The difference is what launching the
    step's kernels as separate graph nodes costs on the class whose kernels
    are shortest."""
    import torch
    W = min(I["W"] for I in wl["inst"])
    sub = dict(wl, inst=[I for I in wl["inst"] if I["W"] == W])
    s, _ = make_series(sub)
    s.run(5)
    st = torch.cuda.ExternalStream(s.stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.synchronize()
    e0.record(st)
    s.run(steps)
    e1.record(st)
    torch.cuda.synchronize()
    step_ms = e0.elapsed_time(e1) / steps
    npl = len(s.planes()[0])
    kern = [s.time_pass(k, 0, reps=20)["ms"] for k in range(0, npl + 3)]
    s.close()
    # the phase sum runs on its own branch beside the passes; the windows, the
    # passes, the unwrap and the apply are serial
    serial = kern[npl + 1] + sum(kern[1:npl + 1]) + kern[npl + 2]
    return {"grid": W, "instances": len(sub["inst"]), "step_ms": round(step_ms, 4),
            "kernels_ms": {"windows": round(kern[npl + 1], 4), "phase_sum": round(kern[0], 4),
                           "passes": round(sum(kern[1:npl + 1]), 4), "unwrap_apply": round(kern[npl + 2], 4)},
            "serial_kernels_ms": round(serial, 4),
            "gap_ms": round(step_ms - serial, 4), "gap_frac": round((step_ms - serial) / step_ms, 3),
            "note": "step = windows, then the passes beside the phase sum, then unwrap, apply and the step "
                    "counter (the counter's 2-3 us counts in the gap)"}


def rows_section() -> dict:
    """The rows around the series, each timed on resident data with CUDA
    events after warm-up: exposure PSFs (W = 512 frames into 1024^2 PSFs),
    the 8192^2 2-D transform behind large master screens, and refraction ray
    traces (GPU table form against the host trace)."""
    import torch
    from atmosphericturbulencesimul_gb300 import _lib, psf as P
    from atmosphericturbulencesimul_gb300.mkwfs import refraction_table
    lib = _lib.load()
    pk = peaks()
    out = {}
    ev = lambda: (torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
    # exposure PSFs: 64 frames per call, amplitude = one pupil
    W, nf = 512, 64
    g = torch.Generator(device="cuda").manual_seed(3)
    pha = torch.randn((nf, W, W), device="cuda", generator=g)
    amp = torch.ones((W, W), device="cuda")
    acc = torch.zeros((2 * W, 2 * W), device="cuda")
    for _ in range(3):
        P.expo_accumulate_dev(pha, amp, acc)
    e0, e1 = ev()
    torch.cuda.synchronize()
    e0.record()
    reps = 10
    for _ in range(reps):
        P.expo_accumulate_dev(pha, amp, acc)
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / reps
    N = 2 * W
    batch = max(1, min(64, (256 << 20) // (N * N * 8)))
    bpf = 4.0 * W * W + 2 * 16.0 * W * W + 2 * 4.0 * N * N / batch    # phase in, intermediate out + in, accumulator
    gbs = bpf * nf / (ms * 1e-3) / 1e9
    out["psf_expo"] = {"value": round(nf / (ms * 1e-3), 1), "unit": "frames/s", "frame": f"{W}^2 -> {N}^2 PSF",
                       "ms_per_call": round(ms, 4), "frames_per_call": nf,
                       "roofline": {"bound": "hbm", "achieved": round(gbs, 1), "peak": pk["hbm_gbs"], "unit": "GB/s",
                                    "frac": round(gbs / pk["hbm_gbs"], 4), "bytes_per_frame": bpf}}
    del pha, acc
    # 8192^2 complex transform (master screens of that size)
    M = 8192
    a = torch.randn((M, M, 2), device="cuda")
    b = torch.empty_like(a)
    for _ in range(2):
        _lib.check(lib.atmwfs_fft2d_dev(a.data_ptr(), b.data_ptr(), M, -1, None))
    e0, e1 = ev()
    torch.cuda.synchronize()
    e0.record()
    for _ in range(5):
        _lib.check(lib.atmwfs_fft2d_dev(a.data_ptr(), b.data_ptr(), M, -1, None))
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1) / 5
    byt = 4 * 2 * 8.0 * M * M
    out["fft2d_8192"] = {"value": round(ms, 3), "unit": "ms", "higher_is_better": False,
                         "roofline": {"bound": "hbm", "achieved": round(byt / (ms * 1e-3) / 1e9, 1),
                                      "peak": pk["hbm_gbs"], "unit": "GB/s",
                                      "frac": round(byt / (ms * 1e-3) / 1e9 / pk["hbm_gbs"], 4), "bytes": byt,
                                      "note": "rows, transpose, rows, transpose: four read+write passes"}}
    del a, b
    # refraction: tables of 16 wavelengths x nz zenith angles, FP64 traces,
    # on the GPU (one ray per thread) and on every host core
    alt = np.arange(10001) * 10.0
    lams = 0.4e-6 * (2.4 / 0.4) ** (np.arange(16) / 15.0)
    Ntab = np.stack([(2.7e-4 * (1 + 0.0056 / (l * 1e6) ** 2) * np.exp(-alt / 8000.0)).astype(np.float32) for l in lams])
    threads = os.cpu_count() or 1
    refraction_table(lams[:1], [0.1], 0.0, Ntab[:1], None, 10.0, where="gpu")
    scan = []
    for nz in (64, 256, 1024, 4096):
        za = np.linspace(0.0, np.deg2rad(75.0), nz)
        t0 = time.perf_counter()
        refraction_table(lams, za, 0.0, Ntab, None, 10.0, where="gpu")
        t_gpu = time.perf_counter() - t0
        # the host on a sample of the same table (every 16th zenith angle)
        sub = za[::max(1, nz // 64)]
        t0 = time.perf_counter()
        refraction_table(lams, sub, 0.0, Ntab, None, 10.0, where="host", host_threads=threads)
        t_host = time.perf_counter() - t0
        scan.append({"rays": 16 * nz, "gpu_rays_per_s": round(16 * nz / t_gpu, 1),
                     "host_rays_per_s": round(16 * len(sub) / t_host, 1)})
    out["refraction"] = {"value": scan[0]["gpu_rays_per_s"], "unit": "rays/s", "rays": scan[0]["rays"],
                         "cpu": {"value": scan[0]["host_rays_per_s"], "unit": "rays/s", "cores": threads,
                                 "sample": "the same table model; host rays on every thread"},
                         "scan": scan,
                         "note": "FP64 traces, wall time of the call; one ray per GPU thread (one warp per block); "
                                 "refraction_table(where='auto') takes the host below the crossover of this scan"}
    return out


def cpu_screens(wl: dict, threads: int):
    """The workload's master screens synthesised, renormalised and weighted on
    the CPU by the oracle (same Philox seeds as the GPU arm)."""
    from oracle import oracle as orc
    o32 = orc.Oracle(32)
    o32.set_threads(threads)
    M = wl["M"]
    screens = []
    for l in range(len(wl["alt"])):
        u, g = o32.screen_noise(1000 + l, 0, M)
        screens.append(o32.master_screen(u, g, wl["L0"] / wl["pupil"], wl["l0"] / wl["pupil"])[0].astype(np.float32))
    cn2 = np.asarray(wl["cn2"], float)
    orc.r0_renormalise(o32, screens, np.float32(wl["lam_ref"]), np.float32(wl["seeing"]), np.float32(wl["pupil"]),
                       cn2 / cn2.sum(), np.float32(0.0))
    return screens


class CpuSeries:
    """The workload on the host cores with the oracle's float port of the
    reference's WFprecision=0 loop (AtmosphericTurbulence.c:2561 onward:
    positions, window sampling, hops, outputs and the science unwrap of every
    instance).  The reference runs one frame at a time in one thread; here the
    instances of a step run one per host thread (each frame single-threaded),
    the largest grids first."""

    def __init__(self, wl: dict, screens, threads: int):
        import concurrent.futures as cf
        from oracle import oracle as orc
        from atmosphericturbulencesimul_gb300.refractivity import scoeff
        self.orc = orc
        self.o32 = orc.Oracle(32)
        self.wl, self.screens, self.threads = wl, screens, threads
        L = len(wl["alt"])
        cn2 = np.asarray(wl["cn2"]) / np.sum(wl["cn2"])
        self.salt, self.sidx = self.o32.superlayers(wl["alt"], cn2, wl["fresnel_bin"])
        self.state = []
        for I in wl["inst"]:
            x, y, vx, vy = orc.init_positions(wl["M"], wl["alt"], wl["speed"], wl["direction"], wl["pupil"], *I["src"])
            self.state.append([x, y, [0] * L, [0] * L, vx, vy,
                               scoeff(wl["lam_ref"], I["lam"], L).astype(np.float64)])
        self.order = sorted(range(len(wl["inst"])), key=lambda i: -wl["inst"][i]["W"])
        # one frame per thread; with fewer instances than threads each frame
        # spreads over its share of the threads (OpenMP inside the frame)
        self.workers = min(threads, len(wl["inst"]))
        self.per_frame = max(1, threads // self.workers)
        self.pool = cf.ThreadPoolExecutor(max_workers=self.workers)

    def _frame(self, i: int, x, y, threads: int = 1) -> None:
        # the OpenMP team size is a per-thread setting: one thread per frame
        self.o32.set_threads(threads)
        I = self.wl["inst"][i]
        ph, fld = self.o32.frame(self.screens, x, y, self.state[i][6], self.sidx, self.salt,
                                 float(np.float32(self.wl["pupil"])), 0.0, I["lam"], I["W"])
        self.o32.output_sci(ph, fld, I["W"])

    def step(self) -> None:
        """One frame of every instance."""
        jobs = []
        for i in self.order:
            st = self.state[i]
            self.orc.step_positions(st[0], st[1], st[2], st[3], st[4], st[5], self.wl["dt"], self.wl["M"])
            jobs.append(self.pool.submit(self._frame, i, st[0].copy(), st[1].copy(), self.per_frame))
        for j in jobs:
            j.result()

    def single_core(self) -> tuple[float, str]:
        """Frames/s of one host core over the workload's mix, from one timed
        frame per grid class (the reference's own one-thread loop)."""
        t_class = {}
        for W in sorted({I["W"] for I in self.wl["inst"]}):
            i = next(k for k, I in enumerate(self.wl["inst"]) if I["W"] == W)
            t0 = time.perf_counter()
            self.pool.submit(self._frame, i, self.state[i][0].copy(), self.state[i][1].copy()).result()
            t_class[W] = time.perf_counter() - t0
        counts = {W: sum(1 for I in self.wl["inst"] if I["W"] == W) for W in t_class}
        fps = len(self.wl["inst"]) / sum(counts[W] * t_class[W] for W in t_class)
        return fps, ", ".join(f"{W}^2 {t_class[W]*1e3:.0f} ms" for W in t_class)

    def close(self) -> None:
        self.pool.shutdown()


def cpu_step_sample(wl: dict, threads: int, min_s: float = 10.0) -> tuple[float, str]:
    """The CPU baseline of the GPU arm's line: whole steps of the workload
    (every instance, one frame each) on `threads` host threads, as many as
    fit in about `min_s` seconds (at least one)."""
    cs = CpuSeries(wl, cpu_screens(wl, threads), threads)
    cs.step()  # warm-up
    t0 = time.perf_counter()
    nsteps = 0
    while nsteps == 0 or time.perf_counter() - t0 < min_s:
        cs.step()
        nsteps += 1
    t = time.perf_counter() - t0
    cs.close()
    n = nsteps * len(wl["inst"])
    how = ("one instance per host thread" if cs.per_frame == 1 else
           f"{cs.workers} instance(s) at a time, {cs.per_frame} threads per frame")
    return n / t, f"{nsteps} whole step(s) of the workload ({n} frames, {t:.2f} s), {how}"


def accuracy_section(s, wl: dict) -> dict:
    """Error of the benchmarked frames against the FP64 oracle.  After the
    timed steps, one more step is run into host buffers; for one instance of
    every grid class (and the shortest and longest wavelengths) the FP64
    oracle recomputes the frame from the engine's own screens (read back
    after renormalisation), positions and Scoeff.  Outside every timed region."""
    from oracle import oracle as orc
    o64 = orc.Oracle(64)
    o64.set_threads(os.cpu_count() or 1)
    frames = s.run_frames(1)
    L = len(wl["alt"])
    screens = [s.read_screen(l) for l in range(L)]
    cn2 = np.asarray(wl["cn2"]) / np.sum(wl["cn2"])
    salt, sidx = o64.superlayers(wl["alt"], cn2, wl["fresnel_bin"])
    inst = wl["inst"]
    pick = {}
    for i, I in enumerate(inst):
        pick.setdefault(I["W"], i)
    lam_sorted = sorted(range(len(inst)), key=lambda i: inst[i]["lam"])
    chosen = sorted(set(pick.values()) | {lam_sorted[0], lam_sorted[-1]})
    rows = []
    for i in chosen:
        I = inst[i]
        x, y = s.positions(i)
        sc = np.asarray(s.instances[i].scoeff, np.float32).astype(np.float64)
        ph, fld = o64.frame(screens, x, y, sc, sidx, salt, float(np.float32(wl["pupil"])), 0.0, I["lam"], I["W"])
        pha_o, amp_o, _, _ = o64.output_sci(ph, fld, I["W"])
        pha_g, amp_g = frames[i][0][0].astype(np.float64), frames[i][1][0].astype(np.float64)
        d = pha_g - pha_o
        wrapped = np.angle(np.exp(1j * d))
        nm = I["lam"] / (2 * np.pi) * 1e9
        rows.append({"instance": i, "W": I["W"], "lambda_um": round(I["lam"] * 1e6, 4),
                     "opd_rms_err_nm": float(np.sqrt(np.mean(d ** 2)) * nm),
                     "opd_wrapped_rms_err_nm": float(np.sqrt(np.mean(wrapped ** 2)) * nm),
                     "jump_frac": float(np.mean(np.abs(d - wrapped) > 1.0)),
                     "amp_var_rel": float(abs(amp_g.var() - amp_o.var()) / max(amp_o.var(), 1e-30)),
                     "amp_max_err": float(np.abs(amp_g - amp_o).max())})
    worst = {k: max(r[k] for r in rows) for k in ("opd_rms_err_nm", "opd_wrapped_rms_err_nm", "jump_frac",
                                                   "amp_var_rel", "amp_max_err")}
    return {"against": "FP64 oracle (same screens, positions and Scoeff as the engine)",
            "frames": len(rows), "worst": {k: float(f"{v:.4g}") for k, v in worst.items()},
            "per_frame": [{k: (float(f"{v:.4g}") if isinstance(v, float) else v) for k, v in r.items()} for r in rows]}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None,
                    help="timed steps (default 200 on the GPU, 10 for the CPU reference arm)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="batched")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-accuracy", action="store_true", help="skip the error check against the FP64 oracle")
    ap.add_argument("--fft-fp16", action="store_true", help="FFT stages in FP16 with per-stage scaling")
    ap.add_argument("--no-surrogate", action="store_true")
    ap.add_argument("--surrogate-only", action="store_true",
                    help="time only the surrogate section (profiling); prints its JSON object")
    ap.add_argument("--surrogate-pairs", type=int, default=50000,
                    help="training pairs of the surrogate section (50k: the specified training set)")
    ap.add_argument("--no-rows", action="store_true", help="skip the PSF / large-transform / refraction section")
    ap.add_argument("--rows-only", action="store_true", help="time only that section (profiling)")
    args = ap.parse_args()
    if args.steps is None:
        args.steps = 10 if args.impl == "reference" else 200
    if args.surrogate_only:
        print(json.dumps(surrogate_section(args.surrogate_pairs)))
        return
    if args.rows_only:
        print(json.dumps(rows_section()))
        return
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    wl = workload(args.workload)
    metric = "wavefront frames/s (7 layers,1024^2,per lambda-dir) surrogate vs plain at <=1nm rms"
    cfg = {"workload": wl["name"], "instances": len(wl["inst"]), "layers": len(wl["alt"]),
           "master": wl["M"], "grids": {str(W): sum(1 for i in wl["inst"] if i["W"] == W)
                                         for W in sorted({i["W"] for i in wl["inst"]})},
           "hops": num_hops(wl),
           "path": "plain (Fresnel, FP16 FFT stages)" if args.fft_fp16 else "plain (Fresnel, FP32)",
           "l2": "inputs larger than L2 (screens + fields > 1 GB)" if len(wl["inst"]) > 8 else
                 "small workload: inputs not larger than L2",
           "parallelism": f"replicas x{args.gpus}"}
    dtype = "f16/f32" if args.fft_fp16 else "f32"

    if args.impl == "reference":
        if rank != 0:
            return
        # the CPU arm: no GPU work at all, inputs made by the oracle too;
        # every step is a whole step of the workload (one frame per instance)
        threads = os.cpu_count() or 1
        cs = CpuSeries(wl, cpu_screens(wl, threads), threads)
        for _ in range(args.warmup):
            cs.step()
        t0 = time.perf_counter()
        for _ in range(args.steps):
            cs.step()
        t = time.perf_counter() - t0
        v = args.steps * len(wl["inst"]) / t
        one, one_sample = cs.single_core()
        cs.close()
        line = {"metric": metric, "value": v, "unit": "frames/s", "n_gpus": args.gpus, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded screens)",
                "config": cfg, "impl": "reference",
                "cpu_baseline": {"value": v, "unit": "frames/s", "cores": threads, "kind": "port",
                                 "sample": f"{args.steps} whole steps of the workload after {args.warmup} warm-up "
                                           f"steps, " + ("one instance per host thread" if cs.per_frame == 1 else
                                                         f"{cs.workers} instance(s) at a time, {cs.per_frame} "
                                                         f"threads per frame"),
                                 "single_core": {"value": round(one, 4), "unit": "frames/s",
                                                 "sample": "one frame per grid class on one thread (" + one_sample
                                                           + "), weighted by the workload's mix"}},
                "e2e": {"value": v, "unit": "frames/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(line))
        return

    import torch
    from atmosphericturbulencesimul_gb300.replicas import aggregate
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    # two device output slots: the e2e copies of a step overlap the next step
    s, screens = make_series(wl, ring=2, fft_fp16=args.fft_fp16)
    ninst = len(wl["inst"])
    L = len(wl["alt"])
    # warm-up (also captures the step graph)
    s.run(args.warmup)
    stream = torch.cuda.ExternalStream(s.stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def barrier():
        torch.cuda.synchronize()
        if dist:
            dist.barrier()

    # device-resident throughput
    barrier()
    ff = s.frame_floats
    nslots = 2
    pha_h = torch.empty(nslots * ff, dtype=torch.float32, pin_memory=True)
    amp_h = torch.empty(nslots * ff, dtype=torch.float32, pin_memory=True)
    # the clock sampler polls the driver every 20 ms: it runs around the
    # device-resident steps only, since its queries can slow the host-driven
    # copies of the end-to-end run
    with ClockSampler(local) as clk:
        barrier()
        clk.mark(True)
        torch.cuda.nvtx.range_push("timed")  # profilers can select the timed steps
        e0.record(stream)
        s.run(args.steps)
        e1.record(stream)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
        clk.mark(False)
    # end to end through the C ABI with host buffers; its own warm-up steps
    # first (the copy stream, its events and the copy kernel are set up on
    # the first call with a sink)
    s.run(args.warmup, pha_ptr=pha_h.data_ptr(), amp_ptr=amp_h.data_ptr(), nslots=nslots)
    barrier()
    w0 = time.perf_counter()
    s.run(args.steps, pha_ptr=pha_h.data_ptr(), amp_ptr=amp_h.data_ptr(), nslots=nslots)
    torch.cuda.synchronize()
    w1 = time.perf_counter()
    # max over ranks of the device time, frames of all ranks
    t, _, value = aggregate(e0.elapsed_time(e1) / 1e3, args.steps * ninst, device="cuda")
    _, _, e2e = aggregate(w1 - w0, args.steps * ninst, device="cuda")

    # roofline of the dominant pass (timed live on the engine stream)
    npl = len(s.planes()[0])
    passes = []
    for c in range(s.num_classes()):
        for k in range(0, npl + 2):
            r = s.time_pass(k, c, reps=5)
            r.update(k=k, c=c)
            if k == npl + 1 and r["bytes"] == 0:
                continue  # this class computes no windows
            passes.append(r)
    # group launches by kernel (grid size, pass kind); the dominant kernel has
    # the largest total time per step
    def kind(k):
        return ("phase-sum" if k == 0 else "windows" if k == npl + 1 else "first" if k == 1 else "last" if k == npl
                else "mid")
    groups = {}
    for p in passes:
        g = groups.setdefault((p["n"], kind(p["k"])), {"ms": 0.0, "bytes": 0.0, "launches": 0, "count": p["count"]})
        g["ms"] += p["ms"]
        g["bytes"] += p["bytes"]
        g["launches"] += 1
    tot = sum(g["ms"] for g in groups.values())
    (dn, dkind), dom = max(groups.items(), key=lambda kv: kv[1]["ms"])
    pk = peaks()
    achieved = (dom["bytes"] / dom["launches"]) / (dom["ms"] / dom["launches"] * 1e-3) / 1e9
    traffic = None
    tf = ROOT / "profiles" / "traffic.json"
    if tf.exists():
        try:
            traffic = json.loads(tf.read_text()).get(f"{dkind}_n{dn}")
        except Exception:
            traffic = None
    roof = {"bound": "hbm", "achieved": round(achieved, 1), "peak": pk["hbm_gbs"], "unit": "GB/s",
            "frac": round(achieved / pk["hbm_gbs"], 4), "traffic": traffic,
            "kernel": f"k_pass {dkind} pass, N={dn} ({dom['count']} instances per launch, {dom['launches']} launches per step)",
            "algorithmic_bytes_per_launch": dom["bytes"] / dom["launches"],
            "ms_per_launch": round(dom["ms"] / dom["launches"], 4), "share_of_step": round(dom["ms"] / tot, 3),
            "peak_source": pk["source"]}
    # the whole step against the path's per-frame byte model W^2 (4 L + 4 e P + 8) (layer windows read once,
    # two field round trips per hop, outputs written once; e = 8 B per complex element), summed over the
    # step's instances; this engine does one field round trip per hop, so the model overstates its bytes
    hops = num_hops(wl)
    e_el = 4 if args.fft_fp16 else 8
    model_step = sum(float(I["W"]) ** 2 * (4 * L + 4 * e_el * hops + 8) for I in wl["inst"])
    ms_step = 1e3 * t / args.steps
    roof["path_model"] = {"bytes_per_step": model_step, "ms_per_step": round(ms_step, 4),
                          "achieved": round(model_step / (ms_step * 1e-3) / 1e9, 1),
                          "frac": round(model_step / (ms_step * 1e-3) / 1e9 / pk["hbm_gbs"], 4),
                          "bytes_per_frame_1024": 1024.0 ** 2 * (4 * L + 4 * e_el * hops + 8)}
    # kernel nodes of the engine's captured step graph (windows, phase sums, passes, unwrap, apply, counter)
    launches = s.step_kernels()
    cfg["tiles"] = {str(ci["n"]): {"cfg": ci["cfg"], "radices": ci["radices"], "rows_per_cta": ci["rows_per_cta"],
                                   "tuned_ms": [round(x, 4) for x in ci["tuned_ms"]]}
                    for ci in (s.class_info(c) for c in range(s.num_classes()))}
    cfg["pass_ms"] = {f"n{p['n']}_k{p['k']}": round(p["ms"], 4) for p in passes}

    line = {"metric": metric, "value": round(value, 2), "unit": "frames/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(1e3 * t / args.steps, 4), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": dtype, "data": "synthetic (seeded Philox screens)",
            "config": cfg, "clocks": clk.summary(),
            "e2e": {"value": round(e2e, 2), "unit": "frames/s", "h2d_bytes_per_step": ninst * L * 16,
                    "d2h_bytes_per_step": 2 * ff * 4},
            "gpu_launches": launches * args.steps, "roofline": roof}
    if rank == 0 and not args.no_accuracy:
        line["error_vs_fp64"] = accuracy_section(s, wl)
    s.close()
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        fps, sample = cpu_step_sample(wl, threads)
        line["cpu_baseline"] = {"value": round(fps, 4), "unit": "frames/s", "cores": threads, "kind": "port",
                                "sample": sample}
    if rank == 0 and not args.no_surrogate:
        line["surrogate"] = surrogate_section(args.surrogate_pairs)
    if rank == 0 and world == 1 and not args.no_rows:
        line["rows"] = rows_section()
        if len({I["W"] for I in wl["inst"]}) > 1:
            line["rows"]["launch_gaps"] = launch_gap_section(wl)
    if rank == 0:
        print(json.dumps(line))
    if dist:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
