"""The reference-written golden cases of tests/golden/ (made by
tests/golden/make_golden.py from the reference's own code): their
parameters, and the same series re-run through the FP64 oracle or the GPU
engine from the reference's raw master screens."""
from __future__ import annotations

from dataclasses import dataclass
from pathlib import Path

import numpy as np

from oracle import oracle as orc

GOLDEN = Path(__file__).resolve().parent / "golden"
CASES = ["mkwfs", "mkwfs_b", "mkwfs_c", "mkwfs_d"]


@dataclass
class Golden:
    name: str
    M: int
    W: int
    Wout: int
    nframes: int
    lam_ref: float      # TURBULENCE_REF_WAVEL as the reference holds it (float)
    slam: float         # SLAMBDA [m] = 1e-6 x the float argument in um, as the reference forms it
    slam_um: float      # that argument
    seeing: float
    pupil: float
    dt: float
    fbin: float
    seed: int
    zangle: float
    src: tuple
    alt: np.ndarray
    cn2: np.ndarray
    speed: np.ndarray
    direction: np.ndarray
    outer: np.ndarray   # L0 [m]
    inner: np.ndarray   # l0 [m]
    screens: np.ndarray  # raw master screens the reference synthesised and saved
    scoeff: np.ndarray
    roffset: np.ndarray
    precision: int       # 0: float files, 1: double files
    ntspan: int          # time spans (files per wavelength)
    amplitude: int       # WAVEFRONT_AMPLITUDE
    cubes: dict          # ref_pha, sci_pha (+ ref_amp, sci_amp): (ntspan * nframes, Wout, Wout)
    conf: str            # WFsim.conf the reference read
    prof: str            # its turbulence profile file
    logprof: np.ndarray  # the layer table the reference printed (normalised Cn2, 6 decimals)

    @property
    def frames(self) -> int:
        return self.nframes * self.ntspan


def load(name: str) -> Golden:
    g = np.load(GOLDEN / f"{name}.npz")
    p = g["params"]
    prof = g["profile"]
    return Golden(name=name, M=int(p[0]), W=int(p[1]), Wout=int(p[2]), nframes=int(p[3]),
                  lam_ref=float(np.float32(p[4] * 1e-6)), slam=1.0e-6 * float(np.float32(p[5])), slam_um=float(np.float32(p[5])), seeing=float(p[6]),
                  pupil=float(p[7]), dt=float(p[8]), fbin=float(p[9]), seed=int(p[10]), zangle=float(p[11]),
                  src=(float(p[12]), float(p[13])), alt=prof[:, 0].copy(), cn2=prof[:, 1].copy(),
                  speed=prof[:, 2].copy(), direction=prof[:, 3].copy(), outer=prof[:, 4].copy(),
                  inner=prof[:, 5].copy(), screens=g["screens"].astype(np.float32), scoeff=g["scoeff"].copy(),
                  roffset=g["roffset"].copy(), precision=int(p[14]), ntspan=int(p[15]), amplitude=int(p[16]),
                  cubes={k: g[k] for k in ("ref_pha", "ref_amp", "sci_pha", "sci_amp") if k in g},
                  conf=str(g["conf"]), prof=str(g["prof"]), logprof=g["logprof"])


def normalised_screens(gc: Golden, o32) -> list[np.ndarray]:
    """The reference's r0 renormalisation and Cn2 / cos z weights, float storage."""
    screens = [s.copy() for s in gc.screens]
    cn2 = gc.cn2 * (1.0 / gc.cn2.sum())
    orc.r0_renormalise(o32, screens, np.float32(gc.lam_ref), np.float32(gc.seeing), np.float32(gc.pupil), cn2,
                       np.float32(gc.zangle))
    return screens


def run_oracle(gc: Golden, o64, o32) -> dict:
    """The series through the FP64 oracle: {key: (frames, Wout, Wout)}."""
    screens = normalised_screens(gc, o32)
    cn2 = gc.cn2 * (1.0 / gc.cn2.sum())
    amp = gc.amplitude
    salt, sidx = o64.superlayers(list(gc.alt), cn2, gc.fbin)
    out = {k: [] for k in gc.cubes}
    for key, lam, sc in (("ref", gc.lam_ref, None), ("sci", gc.slam, gc.scoeff)):
        x, y, vx, vy = orc.init_positions(gc.M, gc.alt, gc.speed, gc.direction, gc.pupil, gc.src[0], gc.src[1],
                                          roffset=gc.roffset)
        cx, cy = [0] * len(x), [0] * len(x)
        for _ in range(gc.frames):
            orc.step_positions(x, y, cx, cy, vx, vy, gc.dt, gc.M)
            phasum, fld = o64.frame(screens, x, y, sc, sidx, salt, float(np.float32(gc.pupil)),
                                    float(np.float32(gc.zangle)), lam, gc.W, amp, amp)
            if key == "sci" and amp:
                pha, a, _, _ = o64.output_sci(phasum, fld, gc.Wout, amp)
            else:
                pha, a = o64.output_ref(phasum, fld, gc.Wout, amp)
            out[key + "_pha"].append(pha)
            if amp:
                out[key + "_amp"].append(a)
    return {k: np.stack(v) for k, v in out.items()}


def run_gpu(gc: Golden) -> dict:
    """The series through the C ABI: raw screens loaded, renormalised on the
    GPU, one lambda_ref instance and one science instance."""
    from atmosphericturbulencesimul_gb300 import MODE_PHASE, MODE_REF, MODE_SCI, InstanceSpec, Series
    amp = gc.amplitude
    inst = [InstanceSpec(lam=gc.lam_ref, mode=MODE_REF if amp else MODE_PHASE, src_x=gc.src[0], src_y=gc.src[1],
                         wf_raw_size=gc.W, wf_size=gc.Wout, roffset=gc.roffset),
            InstanceSpec(lam=gc.slam, mode=MODE_SCI if amp else MODE_PHASE, src_x=gc.src[0], src_y=gc.src[1],
                         wf_raw_size=gc.W, wf_size=gc.Wout, scoeff=gc.scoeff.astype(np.float32), roffset=gc.roffset)]
    s = Series(gc.alt, gc.cn2, gc.speed, gc.direction, master_size=gc.M, instances=inst, pupil_scale=gc.pupil,
               time_step=gc.dt, fresnel_bin=gc.fbin, zangle=gc.zangle, amplitude=amp, fresnel=amp)
    try:
        for l, sc in enumerate(gc.screens):
            s.load_screen(l, sc)
        s.normalize(np.float32(gc.lam_ref), np.float32(gc.seeing))
        frames = s.run_frames(gc.frames)
    finally:
        s.close()
    out = {"ref_pha": frames[0][0], "sci_pha": frames[1][0]}
    if amp:
        out.update(ref_amp=frames[0][1], sci_amp=frames[1][1])
    return out


def compare(got: dict, gc: Golden, lim: dict) -> None:
    """Assert every frame of `got` against the reference's cubes within `lim`."""
    for key, lam in (("ref", gc.lam_ref), ("sci", gc.slam)):
        for f in range(gc.frames):
            ga = got.get(key + "_amp")
            ra = gc.cubes.get(key + "_amp")
            e = frame_errors(got[key + "_pha"][f], None if ga is None else ga[f], gc.cubes[key + "_pha"][f],
                             None if ra is None else ra[f], lam)
            assert e["wrapped_rms_nm"] < lim["wrapped_rms_nm"], (gc.name, key, f, e)
            assert e.get("wrapped_max_nm", 0) < lim.get("wrapped_max_nm", 1e30), (gc.name, key, f, e)
            assert e["flip_frac"] <= lim["flip_frac"], (gc.name, key, f, e)
            assert e["opd_rms_rel"] < lim["opd_rms_rel"] or e["flip_frac"] > 0, (gc.name, key, f, e)
            if ga is not None:
                assert e["amp_max_err"] < lim["amp_max_err"], (gc.name, key, f, e)
                assert e["amp_var_rel"] < lim["amp_var_rel"], (gc.name, key, f, e)


def frame_errors(pha, amp, gpha, gamp, lam) -> dict:
    d = pha.astype(np.float64) - gpha.astype(np.float64)
    w = np.angle(np.exp(1j * d))
    nm = lam / (2 * np.pi) * 1e9
    e = {
        "wrapped_rms_nm": float(np.sqrt(np.mean(w ** 2)) * nm),
        "wrapped_max_nm": float(np.abs(w).max() * nm),
        "flip_frac": float((np.abs(d - w) > 1.0).mean()),
        "opd_rms_rel": float(abs(pha.std() - gpha.std()) / gpha.std()),
    }
    if amp is not None:
        e["amp_max_err"] = float(np.abs(amp.astype(np.float64) - gamp).max())
        e["amp_var_rel"] = float(abs(amp.var() - gamp.var()) / gamp.var())
    return e
