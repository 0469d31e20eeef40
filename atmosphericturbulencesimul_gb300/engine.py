"""Python front end of the GB300 wavefront-series engine.

Mirrors the reference's operators on top of the C ABI:

* :class:`Series` -- make_AtmosphericTurbulence_wavefront_series
  (src/AtmosphericTurbulence/AtmosphericTurbulence.c:1433-4455) split into
  set-up, screen loading, r0 renormalisation and the frame loop;
* :func:`fresnel` -- Fresnel_propagate_wavefront (src/WFpropagate/WFpropagate.c:68-152);
* :func:`fft2d` -- do2dfft / do2dffti (src/fft/fft.c:1298-1315);
* :func:`master_screen` -- make_master_turbulence_screen (AtmosphericTurbulence.c:643-855).
"""
from __future__ import annotations

import ctypes as C
from dataclasses import dataclass, field

import numpy as np

from . import _lib
from ._lib import MODE_PHASE, MODE_REF, MODE_SCI, NUM_TILE_CFG, check

__all__ = ["Series", "InstanceSpec", "layer_planes", "fresnel", "fft2d", "master_screen", "MODE_REF", "MODE_SCI", "MODE_PHASE"]


def _f32p(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def _f64p(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_double))


@dataclass
class InstanceSpec:
    """One (wavelength, direction, output-mode) instance."""
    lam: float                      # propagation wavelength in vacuum [m]
    mode: int = MODE_SCI
    src_x: float = 0.0              # source offset [rad]
    src_y: float = 0.0
    wf_raw_size: int = 256          # propagation grid
    wf_size: int | None = None      # output crop (default: wf_raw_size)
    scoeff: np.ndarray | None = None   # per-layer phase multiplier (float32)
    roffset: np.ndarray | None = None  # per-layer refraction offset [m]
    hop_n: np.ndarray | None = None    # per-hop air index (optional lambda / n hops); None = vacuum lambda


class Series:
    """A configured wavefront series on the GPU."""

    def __init__(self, alt, cn2, speed, direction, *, master_size: int, instances: list[InstanceSpec],
                 pupil_scale: float, time_step: float, fresnel_bin: float = 0.0, zangle: float = 0.0,
                 amplitude: int = 1, fresnel: int = 1, realtime: int = 0, realtime_factor: float = 1.0,
                 ring: int = 1, fft_fp16: int = 0):
        self._lib = _lib.load()
        self.L = len(alt)
        self._keep = []
        arr = lambda v: self._hold(np.ascontiguousarray(v, dtype=np.float64))
        self.alt, self.cn2, self.speed, self.dir = arr(alt), arr(cn2), arr(speed), arr(direction)
        self.instances = list(instances)
        insts = (_lib.Instance * len(instances))()
        for k, s in enumerate(instances):
            I = insts[k]
            I.lambda_ = float(s.lam)
            I.mode = int(s.mode)
            I.src_x = float(s.src_x)
            I.src_y = float(s.src_y)
            I.wf_raw_size = int(s.wf_raw_size)
            I.wf_size = int(s.wf_size or s.wf_raw_size)
            if s.scoeff is not None:
                I.scoeff = _f32p(self._hold(np.ascontiguousarray(s.scoeff, np.float32)))
            if s.roffset is not None:
                I.roffset = _f64p(self._hold(np.ascontiguousarray(s.roffset, np.float64)))
            if s.hop_n is not None:
                I.hop_n = _f64p(self._hold(np.ascontiguousarray(s.hop_n, np.float64)))
        p = _lib.Params()
        p.nlayers = self.L
        p.alt, p.cn2, p.speed, p.dir = _f64p(self.alt), _f64p(self.cn2), _f64p(self.speed), _f64p(self.dir)
        p.fresnel_bin = float(fresnel_bin)
        p.zangle = float(zangle)
        p.pupil_scale = float(pupil_scale)
        p.time_step = float(time_step)
        p.master_size = int(master_size)
        p.amplitude = int(amplitude)
        p.fresnel = int(fresnel)
        p.realtime = int(realtime)
        p.realtime_factor = float(realtime_factor)
        p.ninst = len(instances)
        p.inst = insts
        p.ring = int(ring)
        p.fft_fp16 = int(fft_fp16)
        ctx = C.c_void_p()
        check(self._lib.atmwfs_create(C.byref(p), C.byref(ctx)))
        self._ctx = ctx
        self.master_size = int(master_size)
        self.frame_floats = int(self._lib.atmwfs_frame_floats(ctx))
        self.frame_offsets = [int(self._lib.atmwfs_frame_offset(ctx, i)) for i in range(len(instances))]
        self.wf_sizes = [int(s.wf_size or s.wf_raw_size) for s in instances]

    def _hold(self, a):
        self._keep.append(a)
        return a

    # -- set-up ------------------------------------------------------------
    def load_screen(self, layer: int, screen: np.ndarray) -> None:
        s = np.ascontiguousarray(screen, np.float32)
        check(self._lib.atmwfs_load_screen(self._ctx, layer, _f32p(s), s.shape[0]))

    def load_screen_dev(self, layer: int, ptr: int, M: int) -> None:
        check(self._lib.atmwfs_load_screen_dev(self._ctx, layer, C.c_void_p(ptr), M))

    def read_screen(self, layer: int) -> np.ndarray:
        """The layer's screen as the frames use it (renormalised and weighted
        once normalize() has run)."""
        out = np.empty((self.master_size, self.master_size), np.float32)
        check(self._lib.atmwfs_read_screen(self._ctx, layer, _f32p(out)))
        return out

    def normalize(self, lambda_ref: float, seeing_arcsec: float) -> tuple[float, float]:
        r0 = np.zeros(2)
        check(self._lib.atmwfs_normalize_screens(self._ctx, lambda_ref, seeing_arcsec, _f64p(r0)))
        return float(r0[0]), float(r0[1])

    # -- frame loop ----------------------------------------------------------
    def run(self, nsteps: int, pha: np.ndarray | None = None, amp: np.ndarray | None = None,
            pha_ptr: int | None = None, amp_ptr: int | None = None, nslots: int = 0) -> None:
        """Advance nsteps steps.  Frames go to host arrays (shape [nsteps, frame_floats])
        or raw host or device pointers (nslots frames, reused round-robin);
        with neither they stay on the device."""
        sink = None
        if pha is not None or amp is not None or pha_ptr or amp_ptr:
            sink = _lib.Sink()
            sink.nslots = int(nslots)
            for name, a, ptr in (("pha", pha, pha_ptr), ("amp", amp, amp_ptr)):
                if a is not None:
                    need = (nslots if nslots > 0 else nsteps) * self.frame_floats
                    assert a.dtype == np.float32 and a.flags["C_CONTIGUOUS"] and a.size >= need
                    setattr(sink, name, _f32p(a))
                elif ptr:
                    setattr(sink, name, C.cast(C.c_void_p(ptr), C.POINTER(C.c_float)))
        check(self._lib.atmwfs_run(self._ctx, int(nsteps), C.byref(sink) if sink is not None else None))

    def run_frames(self, nsteps: int):
        """Run nsteps and return per-instance lists of (pha, amp) arrays of shape [nsteps, n, n]."""
        pha = np.empty((nsteps, self.frame_floats), np.float32)
        amp = np.empty((nsteps, self.frame_floats), np.float32)
        self.run(nsteps, pha, amp)
        out = []
        for i, n in enumerate(self.wf_sizes):
            o = self.frame_offsets[i]
            out.append((pha[:, o:o + n * n].reshape(nsteps, n, n), amp[:, o:o + n * n].reshape(nsteps, n, n)))
        return out

    def advance(self, nsteps: int) -> None:
        """Move the windows nsteps steps without propagating (for the surrogate)."""
        check(self._lib.atmwfs_advance(self._ctx, int(nsteps)))

    def frame_offset(self, i: int) -> int:
        return int(self._lib.atmwfs_frame_offset(self._ctx, i))

    def windows_dev(self, i: int, ptr: int, stream: int = 0) -> None:
        """Per-layer phase windows of instance i at the last step into device memory
        (nlayers x W x W floats), on `stream` (0: the engine's)."""
        check(self._lib.atmwfs_windows_dev(self._ctx, i, C.c_void_p(ptr), C.c_void_p(stream) if stream else None))

    def frame_dev(self, i: int) -> tuple[int, int]:
        p, a = C.c_void_p(), C.c_void_p()
        check(self._lib.atmwfs_frame_dev(self._ctx, i, C.byref(p), C.byref(a)))
        return p.value, a.value

    # -- introspection -------------------------------------------------------
    @property
    def steps_done(self) -> int:
        return int(self._lib.atmwfs_steps_done(self._ctx))

    def planes(self):
        n = self._lib.atmwfs_num_planes(self._ctx)
        lo = (C.c_int * n)()
        hi = (C.c_int * n)()
        z = (C.c_double * max(n - 1, 1))()
        check(self._lib.atmwfs_plane_info(self._ctx, lo, hi, z))
        return [(lo[k], hi[k]) for k in range(n)], [z[k] for k in range(n - 1)]

    def positions(self, i: int):
        x = np.zeros(self.L)
        y = np.zeros(self.L)
        check(self._lib.atmwfs_positions(self._ctx, i, _f64p(x), _f64p(y)))
        return x, y

    @property
    def stream(self) -> int:
        return int(self._lib.atmwfs_stream(self._ctx) or 0)

    def step_kernels(self) -> int:
        """Kernel launches per time step (nodes of the captured step graph)."""
        return int(self._lib.atmwfs_step_kernels(self._ctx))

    def num_classes(self) -> int:
        return int(self._lib.atmwfs_num_classes(self._ctx))

    def class_info(self, c: int) -> dict:
        n, no, cnt, rr = C.c_int(), C.c_int(), C.c_int(), C.c_int()
        t = (C.c_double * NUM_TILE_CFG)()
        check(self._lib.atmwfs_class_info(self._ctx, c, C.byref(n), C.byref(no), C.byref(cnt), C.byref(rr), t))
        cfg, rad = C.c_int(), (C.c_int * 3)()
        check(self._lib.atmwfs_class_plan(self._ctx, c, C.byref(cfg), rad))
        return {"n": n.value, "nout": no.value, "count": cnt.value, "rows_per_cta": rr.value,
                "tuned_ms": list(t), "cfg": cfg.value, "radices": [r for r in rad if r > 0]}

    def time_pass(self, k: int, c: int, reps: int = 10):
        """Mean duration [ms] and algorithmic bytes of pass k of grid class c."""
        ms, b = C.c_double(), C.c_double()
        n, cnt = C.c_int(), C.c_int()
        check(self._lib.atmwfs_time_pass(self._ctx, k, c, reps, C.byref(ms), C.byref(b), C.byref(n), C.byref(cnt)))
        return {"ms": ms.value, "bytes": b.value, "n": n.value, "count": cnt.value}

    def last_iters(self, i: int) -> int:
        return int(self._lib.atmwfs_last_iters(self._ctx, i))

    def close(self) -> None:
        if getattr(self, "_ctx", None):
            self._lib.atmwfs_destroy(self._ctx)
            self._ctx = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def layer_planes(alt, cn2, fresnel_bin: float, amplitude: int = 1, fresnel: int = 1, zangle: float = 0.0):
    """Super-layer grouping and propagation planes (host only, no GPU needed).
    Returns (super-layer altitudes, layer -> super-layer index, planes [(lo, hi)], hop distances)."""
    lib = _lib.load()
    alt = np.ascontiguousarray(alt, np.float64)
    cn2 = np.ascontiguousarray(cn2, np.float64)
    L = len(alt)
    ns, npl = C.c_int(), C.c_int()
    salt = np.zeros(L)
    sidx = np.zeros(L, np.int32)
    lo = np.zeros(L, np.int32)
    hi = np.zeros(L, np.int32)
    hz = np.zeros(max(L - 1, 1))
    ip = lambda a: a.ctypes.data_as(C.POINTER(C.c_int))
    check(lib.atmwfs_layer_planes(_f64p(alt), _f64p(cn2), L, fresnel_bin, amplitude, fresnel, zangle, C.byref(ns),
                                  _f64p(salt), ip(sidx), C.byref(npl), ip(lo), ip(hi), _f64p(hz)))
    n = npl.value
    return salt[:ns.value].copy(), sidx, list(zip(lo[:n].tolist(), hi[:n].tolist())), hz[:max(n - 1, 0)].copy()


def fresnel(field_in: np.ndarray, dx: float, z: float, lam: float) -> np.ndarray:
    """Fresnel_propagate_wavefront on an n x n complex64 image (host in, host out)."""
    lib = _lib.load()
    a = np.ascontiguousarray(field_in, np.complex64)
    out = np.empty_like(a)
    check(lib.atmwfs_fresnel(a.ctypes.data_as(C.POINTER(C.c_float)), out.ctypes.data_as(C.POINTER(C.c_float)),
                             a.shape[0], dx, z, lam))
    return out


def fft2d(a: np.ndarray, sign: int = -1) -> np.ndarray:
    """Unnormalised 2-D DFT (sign -1 forward, +1 inverse) of an n x n complex64 image."""
    lib = _lib.load()
    x = np.ascontiguousarray(a, np.complex64)
    out = np.empty_like(x)
    check(lib.atmwfs_fft2d(x.ctypes.data_as(C.POINTER(C.c_float)), out.ctypes.data_as(C.POINTER(C.c_float)),
                           x.shape[0], int(sign)))
    return out


def master_screen(seed: int, M: int, outer_pix: float, inner_pix: float, stream: int = 0):
    """Seeded von Karman master screen pair and the structure-function constants."""
    lib = _lib.load()
    o1 = np.empty((M, M), np.float32)
    o2 = np.empty((M, M), np.float32)
    cf = np.zeros(2)
    check(lib.atmwfs_master_screen(C.c_uint64(seed), stream, M, outer_pix, inner_pix, _f32p(o1), _f32p(o2), _f64p(cf)))
    return o1, o2, cf
