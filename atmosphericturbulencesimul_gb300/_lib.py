"""ctypes binding of libatmwfs.so (the C ABI declared in include/atmwfs.h,
include/atmwfs_mkwfs.h, include/atmwfs_fno.h and include/atmwfs_psf.h).

The library is the only compute path: if it is missing or cannot be loaded
this module raises; there is no CPU fallback.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

LIB_PATH = Path(__file__).resolve().parent / "libatmwfs.so"

OK = 0
STATUS_NAMES = {0: "OK", 1: "ERR_INVALID", 2: "ERR_NOMEM", 3: "ERR_CUDA", 4: "ERR_IO", 5: "ERR_TIMEOUT",
                6: "ERR_STATE", 7: "ERR_NODEVICE"}
MODE_REF, MODE_SCI, MODE_PHASE = 0, 1, 2
NUM_TILE_CFG = 6  # ATMWFS_NUM_TILE_CFG


class AtmwfsError(RuntimeError):
    def __init__(self, status: int, msg: str):
        super().__init__(f"{STATUS_NAMES.get(status, status)}: {msg}")
        self.status = status


class Instance(C.Structure):
    _fields_ = [
        ("lambda_", C.c_double),
        ("mode", C.c_int),
        ("src_x", C.c_float),
        ("src_y", C.c_float),
        ("wf_raw_size", C.c_long),
        ("wf_size", C.c_long),
        ("scoeff", C.POINTER(C.c_float)),
        ("roffset", C.POINTER(C.c_double)),
        ("hop_n", C.POINTER(C.c_double)),
    ]


class Params(C.Structure):
    _fields_ = [
        ("nlayers", C.c_int),
        ("alt", C.POINTER(C.c_double)),
        ("cn2", C.POINTER(C.c_double)),
        ("speed", C.POINTER(C.c_double)),
        ("dir", C.POINTER(C.c_double)),
        ("fresnel_bin", C.c_double),
        ("zangle", C.c_float),
        ("pupil_scale", C.c_float),
        ("time_step", C.c_float),
        ("master_size", C.c_long),
        ("amplitude", C.c_int),
        ("fresnel", C.c_int),
        ("realtime", C.c_int),
        ("realtime_factor", C.c_double),
        ("ninst", C.c_int),
        ("inst", C.POINTER(Instance)),
        ("ring", C.c_int),
        ("fft_fp16", C.c_int),
    ]


class Sink(C.Structure):
    _fields_ = [("pha", C.POINTER(C.c_float)), ("amp", C.POINTER(C.c_float)), ("nslots", C.c_long)]


class Conf(C.Structure):
    """atmwfs_conf: the CONF_* values of the configuration file."""
    _fields_ = [
        ("lambda_", C.c_float),
        ("seeing", C.c_float),
        ("prof_file", C.c_char * 200),
        ("zangle", C.c_float),
        ("source_xpos", C.c_float),
        ("source_ypos", C.c_float),
        ("wfoutput", C.c_int),
        ("wf_file_prefix", C.c_char * 200),
        ("shm_output", C.c_int),
        ("make_swavefront", C.c_int),
        ("swf_write2disk", C.c_int),
        ("swf_file_prefix", C.c_char * 200),
        ("shm_soutput", C.c_int),
        ("shm_sprefix", C.c_char * 100),
        ("shm_soutputm", C.c_int),
        ("pupil_scale", C.c_float),
        ("wfsize", C.c_long),
        ("realtime", C.c_int),
        ("realtime_factor", C.c_double),
        ("wftime_step", C.c_float),
        ("time_span", C.c_float),
        ("nb_tspan", C.c_long),
        ("simtdelay", C.c_long),
        ("waitforsem", C.c_int),
        ("waitsemimname", C.c_char * 100),
        ("skip_existing", C.c_int),
        ("wf_raw_size", C.c_long),
        ("master_size", C.c_long),
        ("wavefront_amplitude", C.c_int),
        ("fresnel_propagation", C.c_int),
        ("fresnel_propagation_bin", C.c_float),
        ("site_alt", C.c_float),
    ]


class FnoCfg(C.Structure):
    _fields_ = [(n, C.c_int) for n in ("nin", "width", "modes", "layers", "proj", "nout", "grid")]


REFRACTIVITY_FN = C.CFUNCTYPE(C.c_float, C.c_float, C.c_float, C.c_void_p)
ABSORPTION_FN = C.CFUNCTYPE(C.c_double, C.c_float, C.c_float, C.c_void_p)


class MkwfsOpts(C.Structure):
    _fields_ = [
        ("refractivity", REFRACTIVITY_FN),
        ("refractivity_user", C.c_void_p),
        ("scoeff", C.POINTER(C.c_double)),
        ("roffset", C.POINTER(C.c_double)),
        ("seed", C.c_ulonglong),
        ("verbose", C.c_int),
        ("semwait_timeout", C.c_double),
        ("fresnel_air_index", C.c_int),
    ]


# (name, restype, argtypes) of every exported entry point
_ctx = C.c_void_p
_fp = C.POINTER(C.c_float)
_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)
SIGNATURES = [
    ("atmwfs_create", C.c_int, [C.POINTER(Params), C.POINTER(_ctx)]),
    ("atmwfs_destroy", None, [_ctx]),
    ("atmwfs_load_screen", C.c_int, [_ctx, C.c_int, _fp, C.c_long]),
    ("atmwfs_load_screen_dev", C.c_int, [_ctx, C.c_int, C.c_void_p, C.c_long]),
    ("atmwfs_read_screen", C.c_int, [_ctx, C.c_int, C.c_void_p]),
    ("atmwfs_normalize_screens", C.c_int, [_ctx, C.c_float, C.c_float, _dp]),
    ("atmwfs_normalize_screens_ext", C.c_int, [_ctx, C.c_float, C.c_float, C.POINTER(_fp), C.c_long, _dp]),
    ("atmwfs_run", C.c_int, [_ctx, C.c_long, C.POINTER(Sink)]),
    ("atmwfs_frame_dev", C.c_int, [_ctx, C.c_int, C.POINTER(C.c_void_p), C.POINTER(C.c_void_p)]),
    ("atmwfs_frame_floats", C.c_size_t, [_ctx]),
    ("atmwfs_frame_offset", C.c_size_t, [_ctx, C.c_int]),
    ("atmwfs_last_iters", C.c_int, [_ctx, C.c_int]),
    ("atmwfs_steps_done", C.c_long, [_ctx]),
    ("atmwfs_num_planes", C.c_int, [_ctx]),
    ("atmwfs_plane_info", C.c_int, [_ctx, _ip, _ip, _dp]),
    ("atmwfs_positions", C.c_int, [_ctx, C.c_int, _dp, _dp]),
    ("atmwfs_layer_planes", C.c_int, [_dp, _dp, C.c_int, C.c_double, C.c_int, C.c_int, C.c_float, _ip, _dp, _ip,
                                      _ip, _ip, _ip, _dp]),
    ("atmwfs_stream", C.c_void_p, [_ctx]),
    ("atmwfs_num_classes", C.c_int, [_ctx]),
    ("atmwfs_class_info", C.c_int, [_ctx, C.c_int, _ip, _ip, _ip, _ip, _dp]),
    ("atmwfs_class_plan", C.c_int, [_ctx, C.c_int, _ip, _ip]),
    ("atmwfs_step_kernels", C.c_int, [_ctx]),
    ("atmwfs_time_pass", C.c_int, [_ctx, C.c_int, C.c_int, C.c_int, _dp, _dp, _ip, _ip]),
    ("atmwfs_fresnel", C.c_int, [_fp, _fp, C.c_long, C.c_double, C.c_double, C.c_double]),
    ("atmwfs_fresnel_dev", C.c_int, [C.c_void_p, C.c_void_p, C.c_long, C.c_double, C.c_double, C.c_double,
                                     C.c_void_p]),
    ("atmwfs_fresnel_noalloc", C.c_int, [C.c_void_p, C.c_void_p, C.c_long, C.c_double, C.c_double, C.c_double,
                                         C.c_void_p]),
    ("atmwfs_fft2d", C.c_int, [_fp, _fp, C.c_long, C.c_int]),
    ("atmwfs_fft2d_dev", C.c_int, [C.c_void_p, C.c_void_p, C.c_long, C.c_int, C.c_void_p]),
    ("atmwfs_master_screen", C.c_int, [C.c_uint64, C.c_uint32, C.c_long, C.c_double, C.c_double, _fp, _fp, _dp]),
    ("atmwfs_last_error", C.c_char_p, []),
    # include/atmwfs_mkwfs.h
    ("atmwfs_conf_read", C.c_int, [C.c_char_p, C.c_char_p, C.c_char_p, C.c_long]),
    ("atmwfs_conf_exists", C.c_int, [C.c_char_p, C.c_char_p]),
    ("atmwfs_conf_load", C.c_int, [C.c_char_p, C.POINTER(Conf)]),
    ("atmwfs_profile_read", C.c_int, [C.c_char_p, C.c_double, _dp, C.c_long, C.POINTER(C.c_long)]),
    ("atmwfs_fits_write", C.c_int, [C.c_char_p, C.c_void_p, C.c_int, C.c_int, C.POINTER(C.c_long)]),
    ("atmwfs_fits_read_f32", C.c_int, [C.c_char_p, _fp, C.c_long, _ip, C.POINTER(C.c_long)]),
    ("atmwfs_shm_create", C.c_int, [C.c_char_p, C.c_long, C.c_long, C.c_int, C.POINTER(C.c_void_p)]),
    ("atmwfs_shm_write", C.c_int, [C.c_void_p, C.c_void_p, C.c_int]),
    ("atmwfs_shm_close", None, [C.c_void_p]),
    ("atmwfs_shm_semwait", C.c_int, [C.c_char_p, C.c_long, C.c_double]),
    ("atmwfs_mkwfs", C.c_int, [C.c_char_p, C.c_float, C.c_long, C.POINTER(MkwfsOpts)]),
    ("atmwfs_make_hv_profile", C.c_int, [C.c_double, C.c_double, C.c_double, C.c_long, C.c_char_p, _dp]),
    ("atmwfs_refraction_path", C.c_int, [C.c_double, C.c_double, C.c_double, REFRACTIVITY_FN, ABSORPTION_FN,
                                         C.c_void_p, C.c_char_p, _dp, _dp]),
    ("atmwfs_refraction_table", C.c_int, [_dp, C.c_long, _dp, C.c_long, C.c_double, _fp, _dp, C.c_long, C.c_double,
                                          _dp, _dp]),
    ("atmwfs_refraction_table_host", C.c_int, [_dp, C.c_long, _dp, C.c_long, C.c_double, _fp, _dp, C.c_long,
                                               C.c_double, C.c_int, _dp, _dp]),
    ("atmwfs_windows_dev", C.c_int, [_ctx, C.c_int, C.c_void_p, C.c_void_p]),
    ("atmwfs_advance", C.c_int, [_ctx, C.c_long]),
    # include/atmwfs_fno.h
    ("atmwfs_fno_create", C.c_int, [C.POINTER(FnoCfg), C.c_uint64, C.POINTER(C.c_void_p)]),
    ("atmwfs_fno_destroy", None, [C.c_void_p]),
    ("atmwfs_fno_get_cfg", C.c_int, [C.c_void_p, C.POINTER(FnoCfg)]),
    ("atmwfs_fno_num_params", C.c_long, [C.c_void_p]),
    ("atmwfs_fno_get_params", C.c_int, [C.c_void_p, _fp]),
    ("atmwfs_fno_set_params", C.c_int, [C.c_void_p, _fp]),
    ("atmwfs_fno_get_grads", C.c_int, [C.c_void_p, _fp]),
    ("atmwfs_fno_zero_grads", C.c_int, [C.c_void_p, C.c_void_p]),
    ("atmwfs_fno_forward", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]),
    ("atmwfs_fno_loss_grad", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, _dp, C.c_void_p]),
    ("atmwfs_fno_adam", C.c_int, [C.c_void_p, C.c_float, C.c_float, C.c_float, C.c_float, C.c_void_p]),
    ("atmwfs_fno_prepare", C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_void_p,
                                     C.c_void_p]),
    ("atmwfs_fno_target", C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p]),
    ("atmwfs_fno_assemble", C.c_int, [C.c_void_p, C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_void_p]),
    ("atmwfs_fno_save", C.c_int, [C.c_void_p, C.c_char_p]),
    ("atmwfs_fno_load", C.c_int, [C.c_char_p, C.POINTER(C.c_void_p)]),
    # include/atmwfs_psf.h
    ("atmwfs_psf_expo_accumulate_dev", C.c_int, [C.c_void_p, C.c_long, C.c_void_p, C.c_long, C.c_long, C.c_void_p,
                                                 C.c_void_p]),
    ("atmwfs_psf_expo_image_dev", C.c_int, [C.c_void_p, C.c_long, C.c_void_p, C.c_void_p]),
    ("atmwfs_psf_expo_load_dev", C.c_int, [C.c_void_p, C.c_long, C.c_void_p, C.c_void_p]),
    ("atmwfs_psf_expo_accumulate", C.c_int, [_fp, C.c_long, _fp, C.c_long, C.c_long, _fp]),
    ("atmwfs_chromat_psf", C.c_int, [_fp, _fp, C.c_long, C.c_float, C.c_float, C.c_long, C.c_float, _fp]),
    ("atmwfs_psf_measure", C.c_int, [_fp, C.c_long, _dp, _dp, _dp, _dp]),
    ("atmwfs_gauss_filter", C.c_int, [_fp, C.c_long, C.c_long, C.c_float, C.c_int, _fp]),
    ("atmwfs_center_psf", C.c_int, [_fp, C.c_long, C.c_long, _dp, _dp]),
    ("atmwfs_measure_fwhm", C.c_int, [_fp, C.c_long, C.c_long, C.c_float, C.c_float, C.c_float, C.c_long, _fp]),
    ("atmwfs_measure_enc_nrj", C.c_int, [_fp, C.c_long, C.c_long, C.c_float, C.c_float, C.c_float, _fp]),
    ("atmwfs_expoframes", C.c_int, [C.c_char_p, C.c_float, C.c_char_p, _fp, C.c_long, C.c_int, _dp]),
    ("atmwfs_fno_pointwise_dev", C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_int, C.c_long,
                                           C.c_float, C.c_void_p, C.c_void_p, C.c_int, C.c_void_p]),
    ("atmwfs_fno_spectral_dev", C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_void_p, C.c_long, C.c_int,
                                          C.c_void_p]),
    ("atmwfs_fno_xspectral_dev", C.c_int, [C.c_void_p, C.c_int, C.c_int, C.c_void_p, C.c_long, C.c_long, C.c_long,
                                           C.c_int, C.c_long, C.c_void_p, C.c_long, C.c_long, C.c_long, C.c_int,
                                           C.c_long, C.c_long, C.c_int, C.c_void_p]),
    ("atmwfs_fno_umma_status", C.c_uint, [C.c_int]),
    ("atmwfs_gemm_bf16", C.c_int, [C.c_int, C.c_int, C.c_int, C.c_void_p, C.c_long, C.c_int, C.c_int, C.c_void_p,
                                   C.c_long, C.c_int, C.c_int, C.c_void_p, C.c_long, C.c_float, C.c_float, C.c_void_p,
                                   C.c_int, C.c_long, C.c_long, C.c_long, C.c_void_p]),
]

_lib = None


def load(path: str | os.PathLike | None = None) -> C.CDLL:
    """Load (once) and return the library with every signature declared."""
    global _lib
    if _lib is not None:
        return _lib
    p = Path(path) if path else LIB_PATH
    if not p.exists():
        raise ImportError(f"{p} is missing: build it with atmosphericturbulencesimul_gb300.build.build()")
    lib = C.CDLL(str(p))
    for name, res, args in SIGNATURES:
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    _lib = lib
    return lib


def check(status: int) -> None:
    if status != OK:
        raise AtmwfsError(status, load().atmwfs_last_error().decode(errors="replace"))
