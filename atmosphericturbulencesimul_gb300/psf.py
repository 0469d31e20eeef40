"""PSF consumers of the wavefront series (include/atmwfs_psf.h): exposure
PSFs accumulated on the GPU, the chromatic PSF of a pupil, the image
measures of the reference's exposure loop, and the exposure command
(the reference's measure_wavefront_series_expoframes).

All compute goes through libatmwfs.so; there is no CPU fallback."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _lib
from ._lib import check


def _f32(a) -> np.ndarray:
    return np.ascontiguousarray(a, np.float32)


def _fp(a: np.ndarray):
    return a.ctypes.data_as(C.POINTER(C.c_float))


def expo_accumulate(pha: np.ndarray, amp: np.ndarray, psf: np.ndarray | None = None) -> np.ndarray:
    """Exposure PSF of the W x W frames pha[f] (amplitude: one W x W pupil for
    every frame, or one per frame), returned as the reference's 2W x 2W
    centred image; accumulated into psf when given."""
    lib = _lib.load()
    pha = _f32(pha)
    if pha.ndim == 2:
        pha = pha[None]
    nf, W, _ = pha.shape
    amp = _f32(amp)
    stride = W * W if amp.ndim == 3 else 0
    out = np.zeros((2 * W, 2 * W), np.float32) if psf is None else _f32(psf).copy()
    check(lib.atmwfs_psf_expo_accumulate(_fp(amp), stride, _fp(pha), W, nf, _fp(out)))
    return out


def expo_accumulate_dev(pha, amp, acc, stream: int = 0) -> None:
    """Device form (torch tensors): acc (2W x 2W, the accumulator layout) +=
    the frames' PSFs, asynchronous on stream."""
    lib = _lib.load()
    nf, W = (pha.shape[0], pha.shape[-1]) if pha.dim() == 3 else (1, pha.shape[-1])
    stride = W * W if amp.dim() == 3 else 0
    check(lib.atmwfs_psf_expo_accumulate_dev(amp.data_ptr(), stride, pha.data_ptr(), W, nf, acc.data_ptr(), stream))


def expo_image_dev(acc, img, stream: int = 0) -> None:
    """The reference's centred image of an accumulator (torch tensors)."""
    check(_lib.load().atmwfs_psf_expo_image_dev(acc.data_ptr(), acc.shape[-1] // 2, img.data_ptr(), stream))


def chromat_psf(amp: np.ndarray, pha: np.ndarray, coeff1: float, coeff2: float, nbstep: int,
                apo: float = 0.0) -> np.ndarray:
    """PSF_makeChromatPSF: the n x n chromatic PSF of a pupil."""
    lib = _lib.load()
    amp, pha = _f32(amp), _f32(pha)
    n = amp.shape[0]
    out = np.empty((n, n), np.float32)
    check(lib.atmwfs_chromat_psf(_fp(amp), _fp(pha), n, coeff1, coeff2, nbstep, apo, _fp(out)))
    return out


def measure(psf: np.ndarray) -> dict:
    """The exposure loop's measures of a PSF image, in pixels."""
    lib = _lib.load()
    p = _f32(psf)
    v = [C.c_double() for _ in range(4)]
    check(lib.atmwfs_psf_measure(_fp(p), p.shape[0], *[C.byref(x) for x in v]))
    return dict(zip(("fwhm", "ee50", "xcenter", "ycenter"), (x.value for x in v)))


def gauss_filter(img: np.ndarray, sigma: float = 3.0, size: int = 10) -> np.ndarray:
    lib = _lib.load()
    a = _f32(img)
    out = np.empty_like(a)
    check(lib.atmwfs_gauss_filter(_fp(a), a.shape[1], a.shape[0], sigma, size, _fp(out)))
    return out


def center(img: np.ndarray) -> tuple[float, float]:
    lib = _lib.load()
    a = _f32(img)
    x, y = C.c_double(), C.c_double()
    check(lib.atmwfs_center_psf(_fp(a), a.shape[1], a.shape[0], C.byref(x), C.byref(y)))
    return x.value, y.value


def fwhm(img: np.ndarray, xc: float, yc: float, step: float = 1.0, nb_step: int | None = None) -> float:
    lib = _lib.load()
    a = _f32(img)
    v = C.c_float()
    check(lib.atmwfs_measure_fwhm(_fp(a), a.shape[1], a.shape[0], xc, yc, step, nb_step or a.shape[1] // 2,
                                  C.byref(v)))
    return v.value


def enc_nrj(img: np.ndarray, xc: float, yc: float, fraction: float = 0.5) -> float:
    lib = _lib.load()
    a = _f32(img)
    v = C.c_float()
    check(lib.atmwfs_measure_enc_nrj(_fp(a), a.shape[1], a.shape[0], xc, yc, fraction, C.byref(v)))
    return v.value


def expoframes(etime: float, outfile: str | os.PathLike, conf: str | os.PathLike = "WFsim.conf",
               pupil: np.ndarray | None = None, amplitude_on: int = 0) -> float:
    """measure_wavefront_series_expoframes(etime, outfile); returns the FWHM
    (arcsec) of the final partial exposure."""
    lib = _lib.load()
    fw = C.c_double()
    if pupil is not None:
        p = _f32(pupil)
        check(lib.atmwfs_expoframes(os.fsencode(conf), etime, os.fsencode(outfile), _fp(p), p.shape[0], amplitude_on,
                                    C.byref(fw)))
    else:
        check(lib.atmwfs_expoframes(os.fsencode(conf), etime, os.fsencode(outfile), None, 0, amplitude_on,
                                    C.byref(fw)))
    return fw.value
