"""Host side of the series command (include/atmwfs_mkwfs.h): the
configuration file, the turbulence profile, FITS cubes, shared-memory
streams and the driver that replaces the reference's `mkwfs` command
(make_AtmosphericTurbulence_wavefront_series,
src/AtmosphericTurbulence/AtmosphericTurbulence.c:1433)."""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import _lib


def _b(s) -> bytes:
    return os.fsencode(s) if not isinstance(s, bytes) else s


def conf_read(conf_file, keyword: str) -> tuple[bool, str]:
    """read_config_parameter (COREMOD_tools.c:629): (found, content); content is "-" when absent."""
    lib = _lib.load()
    buf = C.create_string_buffer(1000)
    r = lib.atmwfs_conf_read(_b(conf_file), keyword.encode(), buf, len(buf))
    if r < 0:
        _lib.check(4)
    return r == 1, buf.value.decode()


def conf_exists(conf_file, keyword: str) -> bool:
    """read_config_parameter_exists (COREMOD_tools.c:596)."""
    r = _lib.load().atmwfs_conf_exists(_b(conf_file), keyword.encode())
    if r < 0:
        _lib.check(4)
    return r == 1


def load_conf(conf_file="WFsim.conf") -> dict:
    """AtmosphericTurbulence_ReadConf (:1233-1427) -> {field: value} of atmwfs_conf."""
    c = _lib.Conf()
    _lib.check(_lib.load().atmwfs_conf_load(_b(conf_file), C.byref(c)))
    out = {}
    for name, typ in c._fields_:
        v = getattr(c, name)
        out["lambda" if name == "lambda_" else name] = v.decode() if isinstance(v, bytes) else v
    return out


def read_profile(path, site_alt: float = 0.0) -> np.ndarray:
    """The turbulence profile (:1946-2015) as an (L, 8) array: altitude, Cn2,
    speed, direction, outer scale, inner scale, wind sigma, wind outer scale."""
    lib = _lib.load()
    n = C.c_long(0)
    _lib.check(lib.atmwfs_profile_read(_b(path), float(site_alt), None, 0, C.byref(n)))
    out = np.zeros((n.value, 8), np.float64)
    if n.value:
        _lib.check(lib.atmwfs_profile_read(_b(path), float(site_alt), out.ctypes.data_as(C.POINTER(C.c_double)),
                                           n.value, C.byref(n)))
    return out


def make_hv_profile(outfile, wspeed: float, r0: float, sitealt: float, nlayers: int) -> float:
    """The reference's mkHVturbprof: writes `outfile` (and conf_turb.txt in the
    current directory); returns the seeing [arcsec]."""
    see = C.c_double()
    _lib.check(_lib.load().atmwfs_make_hv_profile(float(wspeed), float(r0), float(sitealt), int(nlayers),
                                                  _b(outfile), C.byref(see)))
    return see.value


def fits_write(name, a: np.ndarray) -> None:
    """Write a float32 / float64 image of 1-3 axes (numpy order (z, y, x));
    a leading '!' in the name overwrites."""
    a = np.ascontiguousarray(a)
    bitpix = {np.dtype(np.float32): -32, np.dtype(np.float64): -64}.get(a.dtype)
    if bitpix is None:
        raise TypeError("float32 or float64 image expected")
    ax = (C.c_long * 3)(*a.shape[::-1])
    _lib.check(_lib.load().atmwfs_fits_write(_b(name), a.ctypes.data_as(C.c_void_p), bitpix, a.ndim, ax))


def fits_read(name) -> np.ndarray:
    """Read a primary-HDU image as float32, numpy order (z, y, x)."""
    lib = _lib.load()
    nax = C.c_int(0)
    ax = (C.c_long * 3)()
    _lib.check(lib.atmwfs_fits_read_f32(_b(name), None, 0, C.byref(nax), ax))
    shape = tuple(ax[i] for i in range(nax.value))[::-1]
    out = np.empty(shape, np.float32)
    _lib.check(lib.atmwfs_fits_read_f32(_b(name), out.ctypes.data_as(C.POINTER(C.c_float)), out.size, C.byref(nax),
                                        ax))
    return out


class ShmImage:
    """A stream image /tmp/<name>.im.shm in the reference's layout (NBkw = 0)."""

    def __init__(self, name: str, nx: int, ny: int, dtype=np.float32):
        self._lib = _lib.load()
        self.dtype = np.dtype(dtype)
        code = {np.dtype(np.float32): 3, np.dtype(np.float64): 4}[self.dtype]
        self.shape = (ny, nx)
        h = C.c_void_p()
        _lib.check(self._lib.atmwfs_shm_create(name.encode(), nx, ny, code, C.byref(h)))
        self._h = h

    def write(self, frame: np.ndarray, bump: bool = True) -> None:
        f = np.ascontiguousarray(frame, self.dtype)
        if f.shape != self.shape:
            raise ValueError(f"frame shape {f.shape} != {self.shape}")
        _lib.check(self._lib.atmwfs_shm_write(self._h, f.ctypes.data_as(C.c_void_p), int(bump)))

    def close(self) -> None:
        if self._h:
            self._lib.atmwfs_shm_close(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()


def shm_semwait(name: str, index: int = 0, timeout_s: float = 0.0) -> None:
    """COREMOD_MEMORY_image_set_semwait (COREMOD_memory.c:4246), bounded when timeout_s > 0."""
    _lib.check(_lib.load().atmwfs_shm_semwait(name.encode(), index, float(timeout_s)))


def mkwfs(slambda_um: float, precision: int = 0, conf_file="WFsim.conf", *, refractivity=None, scoeff=None,
          roffset=None, seed: int = 0, verbose: bool = False, semwait_timeout: float = 0.0,
          fresnel_air_index: bool = False) -> None:
    """Run the series command in the current directory (see atmwfs_mkwfs).

    refractivity: optional callable N(alt_m, lambda_m) -> n - 1 (the
    reference's AtmosphereModel_stdAtmModel_N); scoeff / roffset: per-layer
    overrides of the science phase multipliers and refraction offsets [m];
    fresnel_air_index: hops with lambda / n(air) instead of the vacuum lambda."""
    lib = _lib.load()
    o = _lib.MkwfsOpts()
    keep = []
    if refractivity is not None:
        cb = _lib.REFRACTIVITY_FN(lambda alt, lam, user: float(refractivity(alt, lam)))
        keep.append(cb)
        o.refractivity = cb
    if scoeff is not None:
        a = np.ascontiguousarray(scoeff, np.float64)
        keep.append(a)
        o.scoeff = a.ctypes.data_as(C.POINTER(C.c_double))
    if roffset is not None:
        a = np.ascontiguousarray(roffset, np.float64)
        keep.append(a)
        o.roffset = a.ctypes.data_as(C.POINTER(C.c_double))
    o.seed = seed
    o.verbose = int(verbose)
    o.semwait_timeout = float(semwait_timeout)
    o.fresnel_air_index = int(fresnel_air_index)
    _lib.check(lib.atmwfs_mkwfs(_b(conf_file), float(slambda_um), int(precision), C.byref(o)))


def cube_name(prefix: str, tspan: int, slambda_m: float, kind: str) -> str:
    """<prefix>%08ld.%09ld.<kind>.fits: time span and science wavelength in pm (:4351)."""
    return f"{prefix}{tspan:08d}.{int(1.0e12 * slambda_m + 0.5):09d}.{kind}.fits"


__all__ = ["conf_read", "conf_exists", "load_conf", "read_profile", "make_hv_profile", "fits_write", "fits_read", "ShmImage",
           "shm_semwait", "mkwfs", "cube_name"]


def table_model(Ntab: np.ndarray, Ktab: np.ndarray | None, dh: float):
    """N(alt, lam) and K(alt, lam) callables reading tables at altitudes
    k * dh with the reference's interpolation (AtmosphereModel.c:3240-3250)."""
    n = len(Ntab)

    def pos(alt):
        a = float(np.float32(alt))      # the model's float argument, divided in double
        i = int(a / dh)
        if i > n - 3:
            i = n - 2
        i = max(i, 0)
        f = float(np.float32(a / dh - i))
        return i, min(max(f, 0.0), 1.0)

    def N(alt, lam):
        i, f = pos(alt)
        return float(np.float32((1.0 - f) * float(Ntab[i]) + f * float(Ntab[i + 1])))

    def K(alt, lam):
        if Ktab is None:
            return 0.0
        i, f = pos(alt)
        return (1.0 - f) * float(Ktab[i]) + f * float(Ktab[i + 1])

    return N, K


def refraction_path(lam: float, zangle: float, site_alt: float, refractivity, absorption=None,
                    path_file=None) -> tuple[float, float]:
    """AtmosphereModel_RefractionPath on the host with model callables
    refractivity(alt, lam) -> N and absorption(alt, lam) -> 1/m:
    (refraction [arcsec], transmission)."""
    lib = _lib.load()
    ncb = _lib.REFRACTIVITY_FN(lambda a, l, u: float(refractivity(a, l)))
    kcb = _lib.ABSORPTION_FN(lambda a, l, u: float(absorption(a, l))) if absorption else _lib.ABSORPTION_FN()
    r, t = C.c_double(), C.c_double()
    _lib.check(lib.atmwfs_refraction_path(lam, zangle, site_alt, ncb, kcb, None,
                                          os.fsencode(path_file) if path_file else None, C.byref(r), C.byref(t)))
    return r.value, t.value


# Tables with fewer rays than this run on the host cores under where="auto":
# one FP64 ray per GPU thread is a serial chain of double transcendentals,
# and the GPU overtakes 16 Grace cores only once the table fills many warps
# on every SM.  Measured (wall time of the call, GPU / 16 cores, rays/s):
# 1,024 rays 1,776 / 7,122; 4,096 rays 7,104 / 7,421; 16,384 rays
# 27,833 / 7,466; 65,536 rays 64,558 / 7,468.
REFRACTION_GPU_MIN_RAYS = 8192


def refraction_table(lambdas, zangles, site_alt: float, Ntab: np.ndarray, Ktab: np.ndarray | None, dh: float,
                     host_threads: int | None = None, where: str = "auto"):
    """Refraction [arcsec] and transmission of every (wavelength, zenith
    angle) pair; Ntab[i] / Ktab[i] tabulate the model of wavelength i at
    altitudes k * dh.  where: "gpu" (one GPU thread per ray), "host"
    (host_threads CPU threads, 0 or None = all) or "auto" (the host when
    host_threads is given or below REFRACTION_GPU_MIN_RAYS rays).  Returns two [nlambda, nzangle] arrays."""
    lib = _lib.load()
    lam = np.ascontiguousarray(lambdas, np.float64)
    za = np.ascontiguousarray(zangles, np.float64)
    N = np.ascontiguousarray(Ntab, np.float32).reshape(len(lam), -1)
    K = None if Ktab is None else np.ascontiguousarray(Ktab, np.float64).reshape(len(lam), -1)
    r = np.empty((len(lam), len(za)))
    t = np.empty_like(r)
    dp = C.POINTER(C.c_double)
    args = (lam.ctypes.data_as(dp), len(lam), za.ctypes.data_as(dp), len(za), site_alt,
            N.ctypes.data_as(C.POINTER(C.c_float)), None if K is None else K.ctypes.data_as(dp), N.shape[1], dh)
    if where not in ("auto", "gpu", "host"):
        raise ValueError(f"where must be auto, gpu or host, not {where!r}")
    if where == "auto":
        big = len(lam) * len(za) >= REFRACTION_GPU_MIN_RAYS
        where = "gpu" if big and host_threads is None else "host"
    if where == "gpu":
        _lib.check(lib.atmwfs_refraction_table(*args, r.ctypes.data_as(dp), t.ctypes.data_as(dp)))
    else:
        _lib.check(lib.atmwfs_refraction_table_host(*args, int(host_threads or 0), r.ctypes.data_as(dp),
                                                    t.ctypes.data_as(dp)))
    return r, t
