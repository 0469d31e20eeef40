"""Seeded small wavefront-series cases run through the GPU engine and the
FP64 oracle with identical inputs (screens, positions, Scoeff), plus the
error metrics used by the parity tests."""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np

from oracle import oracle as orc


@dataclass
class Case:
    alt: list
    cn2: list
    speed: list
    direction: list
    M: int = 256
    W: int = 128
    Wout: int = 128
    fresnel_bin: float = 100.0
    pupil: float = 0.01
    dt: float = 0.001
    zangle: float = 0.0
    lam_ref: float = 0.5e-6
    seeing: float = 0.6875
    # science instances: (lambda, src_x, src_y) on the case's grid, or
    # (lambda, src_x, src_y, W, Wout) on a grid of their own
    sci: list = field(default_factory=lambda: [(1.6e-6, 0.0, 0.0)])
    ref: bool = True
    amplitude: int = 1
    fresnel: int = 1
    seed: int = 7
    air_index: bool = False   # hops with lambda / n(air) (atmwfs_instance.hop_n)
    flat_scoeff: bool = False  # one Scoeff for all layers (a fixed gas mixture, as refractivity.scoeff)


def make_screens(case: Case, o64) -> list[np.ndarray]:
    """Seeded master screens (the oracle's synthesis of Philox noise), then the
    reference's r0 renormalisation and Cn2 weights in float storage."""
    L = len(case.alt)
    o32 = orc.Oracle(32)
    screens = []
    for l in range(L):
        u, g = o64.screen_noise(case.seed, l, case.M)
        s1, _, _ = o32.master_screen(u, g, 20.0 / case.pupil, 0.01 / case.pupil)
        screens.append(s1.astype(np.float32))
    cn2 = np.asarray(case.cn2, float)
    cn2 = cn2 * (1.0 / cn2.sum())
    orc.r0_renormalise(o32, screens, np.float32(case.lam_ref), np.float32(case.seeing), np.float32(case.pupil), cn2,
                       np.float32(case.zangle))
    return screens


def scoeff_for(case: Case, lam: float) -> np.ndarray:
    """A deterministic stand-in for CONF_LAMBDA/SLAMBDA * N(h,lam)/N(h,lam_ref):
    the vacuum ratio times a mild altitude-dependent dispersion factor."""
    L = len(case.alt)
    if case.flat_scoeff:
        return np.full(L, np.float32(np.float32(case.lam_ref) / lam * (1.0 - 1e-3 * (1.0 - case.lam_ref / lam))),
                       np.float32)
    disp = 1.0 - 2e-3 * (1.0 - case.lam_ref / lam) * np.exp(-np.asarray(case.alt) / 8000.0)
    return (np.float32(case.lam_ref) / lam * disp).astype(np.float32) * np.ones(L, np.float32)


def instances(case: Case):
    from atmosphericturbulencesimul_gb300 import MODE_PHASE, MODE_REF, MODE_SCI, InstanceSpec
    from atmosphericturbulencesimul_gb300.refractivity import hop_air_index
    out = []
    if case.ref:
        mode = MODE_REF if case.amplitude else MODE_PHASE
        out.append(InstanceSpec(lam=float(np.float32(case.lam_ref)), mode=mode, wf_raw_size=case.W, wf_size=case.Wout))
    for entry in case.sci:
        lam, sx, sy = entry[:3]
        W, Wout = (entry[3], entry[4]) if len(entry) > 3 else (case.W, case.Wout)
        mode = MODE_SCI if case.amplitude else MODE_PHASE
        out.append(InstanceSpec(lam=lam, mode=mode, src_x=sx, src_y=sy, wf_raw_size=W, wf_size=Wout,
                                scoeff=scoeff_for(case, lam)))
    if case.air_index:
        for I in out:
            I.hop_n = hop_air_index(case.alt, case.cn2, case.fresnel_bin, I.lam, amplitude=case.amplitude,
                                    fresnel=case.fresnel, zangle=case.zangle)
    return out


def run_gpu(case: Case, screens, nsteps: int, ring: int = 1, specs=None):
    from atmosphericturbulencesimul_gb300 import Series
    inst = instances(case) if specs is None else specs
    s = Series(case.alt, case.cn2, case.speed, case.direction, master_size=case.M, instances=inst,
               pupil_scale=case.pupil, time_step=case.dt, fresnel_bin=case.fresnel_bin, zangle=case.zangle,
               amplitude=case.amplitude, fresnel=case.fresnel, ring=ring)
    for l, sc in enumerate(screens):
        s.load_screen(l, sc)
    frames = s.run_frames(nsteps)
    pos = [s.positions(i) for i in range(len(inst))]
    planes = s.planes()
    s.close()
    return inst, frames, pos, planes


def run_oracle(case: Case, o64, screens, nsteps: int, specs=None):
    """Per step, per instance (pha, amp) from the FP64 oracle."""
    inst = instances(case) if specs is None else specs
    cn2 = np.asarray(case.cn2, float)
    cn2 = cn2 * (1.0 / cn2.sum())
    salt, sidx = o64.superlayers(case.alt, cn2, case.fresnel_bin)
    res = []
    states = []
    for I in inst:
        x, y, vx, vy = orc.init_positions(case.M, case.alt, case.speed, case.direction, case.pupil, I.src_x, I.src_y)
        states.append([x, y, [0] * len(x), [0] * len(x), vx, vy])
    for _ in range(nsteps):
        step = []
        for I, st in zip(inst, states):
            orc.step_positions(st[0], st[1], st[2], st[3], st[4], st[5], case.dt, case.M)
            sc = None if I.scoeff is None else I.scoeff.astype(np.float64)
            phasum, fld = o64.frame(screens, st[0], st[1], sc, sidx, salt, float(np.float32(case.pupil)),
                                    float(np.float32(case.zangle)), I.lam, I.wf_raw_size, case.amplitude, case.fresnel,
                                    hop_n=I.hop_n)
            from atmosphericturbulencesimul_gb300 import MODE_SCI
            if I.mode == MODE_SCI:
                pha, amp, _, _ = o64.output_sci(phasum, fld, I.wf_size, case.amplitude)
            else:
                pha, amp = o64.output_ref(phasum, fld, I.wf_size, case.amplitude)
            step.append((pha, amp))
        res.append(step)
    final_pos = [(st[0].copy(), st[1].copy()) for st in states]
    return inst, res, final_pos, (salt, sidx)


def metrics(pha_g, amp_g, pha_o, amp_o, lam):
    """Error metrics of one frame against the oracle."""
    d = pha_g.astype(np.float64) - pha_o.astype(np.float64)
    wrapped = np.angle(np.exp(1j * d))
    flips = np.abs(d - wrapped) > 1.0
    nm = lam / (2 * np.pi) * 1e9
    opd_g = pha_g.astype(np.float64) * lam / (2 * np.pi)
    opd_o = pha_o.astype(np.float64) * lam / (2 * np.pi)
    return {
        "wrapped_rms_nm": float(np.sqrt(np.mean(wrapped ** 2)) * nm),
        "opd_rms_err_nm": float(np.sqrt(np.mean(d ** 2)) * nm),
        "flip_frac": float(flips.mean()),
        "amp_max_err": float(np.max(np.abs(amp_g.astype(np.float64) - amp_o))),
        "opd_rms_rel": float(abs(opd_g.std() - opd_o.std()) / max(opd_o.std(), 1e-30)),
        "amp_var_rel": float(abs(amp_g.var() - amp_o.var()) / max(amp_o.var(), 1e-30)),
    }


def compare(case: Case, o64, nsteps: int, wrapped_nm: float = 0.05, flip: float = 2e-3, amp_var: float = 1e-3,
            screens=None, specs=None):
    """Run `case` for `nsteps` on the GPU and in the FP64 oracle from the same
    screens (and instance list `specs`, default instances(case)) and assert
    the parity bars on every frame:
      * layer positions equal bit for bit (the reference's sequential update);
      * wrapped phase error < `wrapped_nm` nm rms, amplitude error < 2e-3;
      * a 2 pi jump of the unwrapped phase on fewer than `flip` of the pixels;
      * relative OPD rms within 1e-4 (frames without a jump), relative
        amplitude variance within `amp_var` (frames with a variance above 1e-6).
    Returns the metrics of every frame, with the instance's grid and step."""
    if screens is None:
        screens = make_screens(case, o64)
    inst_g, frames, pos_g, _ = run_gpu(case, screens, nsteps, specs=specs)
    inst_o, res, pos_o, _ = run_oracle(case, o64, screens, nsteps, specs=specs)
    for (xg, yg), (xo, yo) in zip(pos_g, pos_o):
        assert np.array_equal(xg, xo) and np.array_equal(yg, yo)
    out = []
    for i, I in enumerate(inst_g):
        for s in range(nsteps):
            pha_g, amp_g = frames[i][0][s], frames[i][1][s]
            pha_o, amp_o = res[s][i]
            m = metrics(pha_g, amp_g, pha_o, amp_o, I.lam)
            m.update(inst=i, step=s, W=I.wf_raw_size, Wout=I.wf_size or I.wf_raw_size, mode=I.mode)
            out.append(m)
            assert m["wrapped_rms_nm"] < wrapped_nm, m
            assert m["amp_max_err"] < 2e-3, m
            assert m["flip_frac"] < flip, m
            assert m["opd_rms_rel"] < 1e-4 or m["flip_frac"] > 0, m
            if amp_o.var() > 1e-6:
                assert m["amp_var_rel"] < amp_var, m
    return out


def worst(ms: list) -> dict:
    """Largest value of every error metric over a list of frame metrics."""
    keys = ["wrapped_rms_nm", "opd_rms_err_nm", "flip_frac", "amp_max_err", "opd_rms_rel", "amp_var_rel"]
    return {k: max(m[k] for m in ms) for k in keys}
