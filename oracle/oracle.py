"""ctypes front end of the CPU oracle (oracle/atmwfs_oracle.c).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and
bench.py's CPU-baseline leg, never by the product.  ``Oracle(64)`` is the FP64
restatement used as the checker; ``Oracle(32)`` is the float-storage port of
the reference's WFprecision=0 path used as the timed CPU baseline.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess
from pathlib import Path

import numpy as np

HERE = Path(__file__).resolve().parent
BUILD = HERE / "build"

_dp = C.POINTER(C.c_double)
_lp = C.POINTER(C.c_long)
_vp = C.c_void_p


def build() -> None:
    """Compile both oracle libraries (make, in-tree)."""
    r = subprocess.run(["make", "-s", "-C", str(HERE)], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + r.stdout + r.stderr)


def _ptr(a: np.ndarray) -> int:
    assert a.flags["C_CONTIGUOUS"]
    return a.ctypes.data


class Oracle:
    def __init__(self, bits: int = 64):
        assert bits in (32, 64)
        path = BUILD / f"liboracle{bits}.so"
        if not path.exists():
            build()
        self.lib = C.CDLL(str(path))
        self.real = np.float64 if bits == 64 else np.float32
        self.cplx = np.complex128 if bits == 64 else np.complex64
        L = self.lib
        L.or_set_threads.argtypes = [C.c_int]
        L.or_fft2d.argtypes = [_vp, C.c_long, C.c_long, C.c_int]
        L.or_permut.argtypes = [_vp, C.c_long, C.c_long]
        L.or_fresnel.argtypes = [_vp, _vp, C.c_long, C.c_double, C.c_double, C.c_double]
        L.or_window.argtypes = [_vp, C.c_long, C.c_double, C.c_double, C.c_long, C.c_double, C.c_int, _vp]
        L.or_superlayers.argtypes = [_dp, _dp, C.c_long, C.c_double, _dp, _lp]
        L.or_superlayers.restype = C.c_long
        L.or_position_step.argtypes = [_dp, _lp, C.c_double, C.c_float, C.c_long]
        L.or_frame.argtypes = [_vp, C.c_long, C.c_long, _dp, _dp, _dp, _lp, _dp, C.c_double, C.c_double, C.c_double,
                               C.c_long, C.c_int, C.c_int, C.c_int, _vp, _vp]
        L.or_frame_n.argtypes = [_vp, C.c_long, C.c_long, _dp, _dp, _dp, _lp, _dp, C.c_double, C.c_double, C.c_double,
                                 C.c_long, C.c_int, C.c_int, C.c_int, _dp, _vp, _vp]
        L.or_output_ref.argtypes = [_vp, _vp, C.c_long, C.c_long, C.c_int, _vp, _vp]
        L.or_output_sci.argtypes = [_vp, _vp, C.c_long, C.c_long, C.c_int, _vp, _vp, _vp]
        L.or_output_sci.restype = C.c_long
        L.or_measure_r0.argtypes = [_vp, C.c_long]
        L.or_measure_r0.restype = C.c_double
        L.or_master_screen.argtypes = [_vp, _vp, C.c_long, C.c_double, C.c_double, _vp, _vp, _dp]
        L.or_philox.argtypes = [C.c_uint64, C.c_uint32, C.c_uint32, C.POINTER(C.c_uint32)]
        L.or_philox4.argtypes = [C.POINTER(C.c_uint32), C.POINTER(C.c_uint32), C.POINTER(C.c_uint32)]
        L.or_screen_noise.argtypes = [C.c_uint64, C.c_uint32, C.c_long, _vp, _vp]
        # PSF consumers (psf_oracle.c)
        L.or_psf_expo_add.argtypes = [_vp, _vp, C.c_long, _vp]
        L.or_chromat_psf.argtypes = [_vp, _vp, C.c_long, C.c_float, C.c_float, C.c_long, C.c_float, _vp]
        L.or_gauss_filter.argtypes = [_vp, C.c_long, C.c_long, C.c_float, C.c_int, _vp]
        L.or_center_psf.argtypes = [_vp, C.c_long, C.c_long, _dp, _dp]
        L.or_measure_fwhm.argtypes = [_vp, C.c_long, C.c_long, C.c_double, C.c_double, C.c_double, C.c_long]
        L.or_measure_fwhm.restype = C.c_double
        L.or_measure_enc_nrj.argtypes = [_vp, C.c_long, C.c_long, C.c_double, C.c_double, C.c_double]
        L.or_measure_enc_nrj.restype = C.c_double

    # -- basic operators -------------------------------------------------
    def set_threads(self, n: int) -> None:
        self.lib.or_set_threads(int(n))

    def fft2d(self, a: np.ndarray, sign: int) -> np.ndarray:
        out = np.ascontiguousarray(a, dtype=self.cplx).copy()
        self.lib.or_fft2d(_ptr(out), out.shape[1], out.shape[0], int(sign))
        return out

    def fresnel(self, a: np.ndarray, dx: float, z: float, lam: float) -> np.ndarray:
        inp = np.ascontiguousarray(a, dtype=self.cplx)
        out = np.empty_like(inp)
        self.lib.or_fresnel(_ptr(inp), _ptr(out), inp.shape[0], dx, z, lam)
        return out

    def window(self, screen: np.ndarray, xpos: float, ypos: float, W: int, scoeff: float = 1.0,
               bicubic: bool = True) -> np.ndarray:
        s = np.ascontiguousarray(screen, dtype=self.real)
        out = np.empty((W, W), np.float64)
        self.lib.or_window(_ptr(s), s.shape[0], xpos, ypos, W, scoeff, int(bicubic), _ptr(out))
        return out

    def superlayers(self, alt, cn2, fresnel_bin: float):
        alt = np.ascontiguousarray(alt, np.float64)
        cn2 = np.ascontiguousarray(cn2, np.float64)
        L = len(alt)
        salt = np.zeros(L)
        sidx = np.zeros(L, np.int64)
        S = self.lib.or_superlayers(alt.ctypes.data_as(_dp), cn2.ctypes.data_as(_dp), L, fresnel_bin,
                                    salt.ctypes.data_as(_dp), sidx.ctypes.data_as(_lp))
        return salt[:S].copy(), sidx

    def position_step(self, pos: float, cnt: int, v: float, dt: float, M: int):
        p = C.c_double(pos)
        c = C.c_long(cnt)
        self.lib.or_position_step(C.byref(p), C.byref(c), v, dt, M)
        return p.value, c.value

    def frame(self, screens, xpos, ypos, scoeff, sidx, salt, dx, zangle, lam, W, amplitude=1, fresnel=1,
              bicubic=1, hop_n=None):
        L = len(screens)
        M = screens[0].shape[0]
        arrs = [np.ascontiguousarray(s, dtype=self.real) for s in screens]
        ptrs = (C.c_void_p * L)(*[_ptr(a) for a in arrs])
        xpos = np.ascontiguousarray(xpos, np.float64)
        ypos = np.ascontiguousarray(ypos, np.float64)
        sc = None if scoeff is None else np.ascontiguousarray(scoeff, np.float64)
        sidx = np.ascontiguousarray(sidx, np.int64)
        salt = np.ascontiguousarray(salt, np.float64)
        phasum = np.empty((W, W), self.real)
        field = np.empty((W, W), self.cplx)
        hn = None if hop_n is None else np.ascontiguousarray(hop_n, np.float64)
        self.lib.or_frame_n(C.cast(ptrs, C.c_void_p), M, L, xpos.ctypes.data_as(_dp), ypos.ctypes.data_as(_dp),
                            None if sc is None else sc.ctypes.data_as(_dp), sidx.ctypes.data_as(_lp),
                            salt.ctypes.data_as(_dp), dx, zangle, lam, W, amplitude, fresnel, bicubic,
                            None if hn is None else hn.ctypes.data_as(_dp), _ptr(phasum), _ptr(field))
        return phasum, field

    def output_ref(self, phasum, field, Wout, amplitude=1):
        W = phasum.shape[0]
        pha = np.empty((Wout, Wout), self.real)
        amp = np.empty((Wout, Wout), self.real)
        self.lib.or_output_ref(_ptr(np.ascontiguousarray(phasum, self.real)),
                               _ptr(np.ascontiguousarray(field, self.cplx)), W, Wout, amplitude, _ptr(pha), _ptr(amp))
        return pha, amp

    def output_sci(self, phasum, field, Wout, amplitude=1):
        W = phasum.shape[0]
        pha = np.empty((Wout, Wout), self.real)
        amp = np.empty((Wout, Wout), self.real)
        nb = max(Wout // 20, 1)
        bins = np.zeros((nb, nb), self.real)
        it = self.lib.or_output_sci(_ptr(np.ascontiguousarray(phasum, self.real)),
                                    _ptr(np.ascontiguousarray(field, self.cplx)), W, Wout, amplitude, _ptr(pha),
                                    _ptr(amp), _ptr(bins))
        return pha, amp, bins, it

    def measure_r0(self, screen) -> float:
        s = np.ascontiguousarray(screen, self.real)
        return self.lib.or_measure_r0(_ptr(s), s.shape[0])

    def screen_noise(self, seed: int, stream: int, M: int):
        u = np.empty((M, M), np.float32)
        g = np.empty((M, M), np.float32)
        self.lib.or_screen_noise(C.c_uint64(seed), stream, M, _ptr(u), _ptr(g))
        return u, g

    def master_screen(self, upha, gau, L0pix: float, l0pix: float):
        M = upha.shape[0]
        u = np.ascontiguousarray(upha, self.real)
        g = np.ascontiguousarray(gau, self.real)
        o1 = np.empty((M, M), self.real)
        o2 = np.empty((M, M), self.real)
        cf = np.zeros(2)
        self.lib.or_master_screen(_ptr(u), _ptr(g), M, L0pix, l0pix, _ptr(o1), _ptr(o2), cf.ctypes.data_as(_dp))
        return o1, o2, cf

    def philox4(self, ctr, key):
        c = (C.c_uint32 * 4)(*ctr)
        k = (C.c_uint32 * 2)(*key)
        out = (C.c_uint32 * 4)()
        self.lib.or_philox4(c, k, out)
        return list(out)

    def philox(self, seed: int, c0: int, c1: int):
        out = (C.c_uint32 * 4)()
        self.lib.or_philox(C.c_uint64(seed), c0, c1, out)
        return list(out)


# -- reference-semantics helpers in pure Python (small, exact restatements) --

    # -- PSF consumers ---------------------------------------------------
    def psf_expo(self, amp, pha):
        """Exposure PSF (2W x 2W, centred) of the frames pha[f] with the
        amplitude amp (one W x W image, or one per frame)."""
        pha = np.asarray(pha)
        if pha.ndim == 2:
            pha = pha[None]
        W = pha.shape[-1]
        psf = np.zeros((2 * W, 2 * W), self.real)
        for f in range(pha.shape[0]):
            a = np.ascontiguousarray(amp[f] if np.ndim(amp) == 3 else amp, self.real)
            p = np.ascontiguousarray(pha[f], self.real)
            self.lib.or_psf_expo_add(_ptr(a), _ptr(p), W, _ptr(psf))
        return psf

    def chromat_psf(self, amp, pha, coeff1, coeff2, nbstep, apo):
        a, p = (np.ascontiguousarray(x, self.real) for x in (amp, pha))
        out = np.zeros_like(a)
        self.lib.or_chromat_psf(_ptr(a), _ptr(p), a.shape[0], coeff1, coeff2, nbstep, apo, _ptr(out))
        return out

    def gauss_filter(self, img, sigma=3.0, size=10):
        a = np.ascontiguousarray(img, self.real)
        out = np.zeros_like(a)
        self.lib.or_gauss_filter(_ptr(a), a.shape[1], a.shape[0], sigma, size, _ptr(out))
        return out

    def center_psf(self, img):
        a = np.ascontiguousarray(img, self.real)
        x, y = C.c_double(), C.c_double()
        self.lib.or_center_psf(_ptr(a), a.shape[1], a.shape[0], C.byref(x), C.byref(y))
        return x.value, y.value

    def measure_fwhm(self, img, xc, yc, step=1.0, nb=None):
        a = np.ascontiguousarray(img, self.real)
        return self.lib.or_measure_fwhm(_ptr(a), a.shape[1], a.shape[0], xc, yc, step, nb or a.shape[1] // 2)

    def measure_enc_nrj(self, img, xc, yc, fraction=0.5):
        a = np.ascontiguousarray(img, self.real)
        return self.lib.or_measure_enc_nrj(_ptr(a), a.shape[1], a.shape[0], xc, yc, fraction)

    def psf_measure(self, psf):
        """The exposure loop's measures: (xc, yc, fwhm, ee50) in pixels."""
        g = self.gauss_filter(psf)
        xc, yc = self.center_psf(g)
        return xc, yc, self.measure_fwhm(g, xc, yc), self.measure_enc_nrj(psf, xc, yc)


def scoeff_from_n(lam_ref_f32: float, lam_sci: float, n_sci_f32: float, n_ref_f32: float) -> float:
    """Scoeff = CONF_LAMBDA/SLAMBDA * Nslambda/Nlambda with the reference's
    float operands (AtmosphericTurbulence.c:2661-2663)."""
    return float(lam_ref_f32) / float(lam_sci) * float(n_sci_f32) / float(n_ref_f32)


def init_positions(M, alt, speed, direction, dx_f32, src_x=0.0, src_y=0.0, roffset=None):
    """Start positions and pixel velocities (AtmosphericTurbulence.c:2152-2197)."""
    L = len(alt)
    dx = float(np.float32(dx_f32))
    sx = float(np.float32(src_x))
    sy = float(np.float32(src_y))
    xpos = np.empty(L)
    ypos = np.empty(L)
    vx = np.empty(L)
    vy = np.empty(L)
    for l in range(L):
        xpos[l] = 0.05 * M
        ypos[l] = 0.05 * M
        ypos[l] += (0.0 if roffset is None else roffset[l]) / dx
        xpos[l] += sx * alt[l] / dx
        ypos[l] += sy * alt[l] / dx
        vx[l] = speed[l] * np.cos(direction[l]) / dx
        vy[l] = speed[l] * np.sin(direction[l]) / dx
    return xpos, ypos, vx, vy


def step_positions(xpos, ypos, xcnt, ycnt, vx, vy, dt_f32, M):
    """Non-real-time position update and wrap (AtmosphericTurbulence.c:2700-2756)."""
    dt = float(np.float32(dt_f32))
    for l in range(len(xpos)):
        xpos[l] += vx[l] * dt
        ypos[l] += vy[l] * dt
        while xpos[l] < 0:
            xpos[l] += M
            xcnt[l] += 1
        while xpos[l] > M:
            xpos[l] -= M
            xcnt[l] -= 1
        while ypos[l] < 0:
            ypos[l] += M
            ycnt[l] += 1
        while ypos[l] > M:
            ypos[l] -= M
            ycnt[l] -= 1


def r0_renormalise(orc: "Oracle", screens, lam_ref_f32, seeing_f32, dx_f32, cn2_norm, zangle_f32):
    """r0 measurement, renormalisation and Cn2 weights (AtmosphericTurbulence.c:2240-2363),
    applied in place in the oracle's storage precision.  Returns (r0_before, r0_after)."""
    r0a = float(np.mean([orc.measure_r0(s) for s in screens]))
    target = float(np.float32(lam_ref_f32)) / (float(np.float32(seeing_f32)) / 3600.0 / 180.0 * np.pi) / float(
        np.float32(dx_f32)) * 1
    tmp1 = (r0a / target) ** (5.0 / 6.0)
    for s in screens:
        s[...] = (s.astype(np.float64) * tmp1).astype(s.dtype)
    r0b = float(np.mean([orc.measure_r0(s) for s in screens]))
    z = float(np.float32(zangle_f32))
    for l, s in enumerate(screens):
        s[...] = (s.astype(np.float64) * np.sqrt(cn2_norm[l] / np.cos(z))).astype(s.dtype)
    return r0a, r0b


if __name__ == "__main__":
    build()
    print("oracle built in", BUILD, os.listdir(BUILD))
