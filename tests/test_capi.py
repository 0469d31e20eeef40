"""The C ABI library (no GPU needed): it builds for sm_103a, loads, exports
every entry point include/*.h declares, runs its host-only logic, and
reports errors as status codes."""
import ctypes as C
import re
import subprocess
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


def header_functions():
    names = set()
    for h in sorted((ROOT / "include").glob("*.h")):
        txt = re.sub(r"/\*.*?\*/", "", h.read_text(), flags=re.S)
        # declarations, not function-pointer typedefs such as (*atmwfs_refractivity_fn)
        names |= set(re.findall(r"\b(atmwfs_[a-z0-9_]+)\s*\(", txt))
    return sorted(names)


def test_exports_every_declared_symbol(lib):
    out = subprocess.run(["nm", "-D", "--defined-only", str(ROOT / "atmosphericturbulencesimul_gb300" / "libatmwfs.so")],
                         capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r" T (atmwfs_\w+)", out))
    declared = header_functions()
    assert len(declared) >= 38
    missing = [f for f in declared if f not in exported]
    assert not missing, missing
    for f in declared:
        assert hasattr(lib, f)


def test_binding_covers_header(lib):
    from atmosphericturbulencesimul_gb300 import _lib
    bound = {n for n, _, _ in _lib.SIGNATURES}
    assert set(header_functions()) <= bound


def test_layer_planes_match_oracle(lib, oracle64):
    from atmosphericturbulencesimul_gb300 import layer_planes
    rng = np.random.default_rng(0)
    for trial in range(200):
        L = int(rng.integers(1, 9))
        alt = np.sort(rng.uniform(0, 20000, L))
        if trial % 3 == 0:
            alt[rng.integers(0, L)] = alt[0]  # coincident altitudes
            alt.sort()
        cn2 = rng.uniform(0.01, 1, L)
        b = float(rng.choice([10.0, 100.0, 500.0, 2000.0, 1e5]))
        salt, sidx, planes, hz = layer_planes(alt, cn2, b)
        so, io = oracle64.superlayers(alt, cn2 / cn2.sum() * 1.0, b)
        assert np.allclose(salt, so, rtol=0, atol=1e-9) and list(sidx) == list(io)
        # planes: runs of equal super-layer index from the top layer down
        exp = []
        hi = L
        for l in range(L - 1, -1, -1):
            if l == 0 or io[l - 1] != io[l]:
                exp.append((l, hi))
                hi = l
        assert planes == exp
        assert len(hz) == len(planes) - 1
        for k in range(len(hz)):
            assert abs(hz[k] - (so[io[planes[k][0]]] - so[io[planes[k + 1][0]]])) < 1e-9
    # without amplitude or Fresnel propagation: one plane
    _, _, planes, hz = layer_planes([0.0, 1000.0], [1, 1], 10.0, amplitude=0)
    assert planes == [(0, 2)] and len(hz) == 0


def test_errors_are_status_codes(lib):
    from atmosphericturbulencesimul_gb300 import _lib, fresnel
    with pytest.raises(_lib.AtmwfsError) as e:
        fresnel(np.zeros((100, 100), np.complex64), 0.01, 100.0, 1e-6)
    assert e.value.status == 1 and "unsupported" in str(e.value)
    # a bad profile is rejected before any device work
    p = _lib.Params()
    p.nlayers = 0
    ctx = C.c_void_p()
    assert lib.atmwfs_create(C.byref(p), C.byref(ctx)) == 1
    assert lib.atmwfs_layer_planes(None, None, 0, 0.0, 1, 1, 0.0, None, None, None, None, None, None, None) == 1


@pytest.mark.parametrize("field,value,words", [
    ("wf_raw_size", 100, "power of two"),      # not a power of two
    ("wf_raw_size", 4096, "power of two"),     # above the largest propagation grid
    ("wf_size", 300, "wf_size"),               # crop larger than the grid
    ("wf_size", 0, "wf_size"),                 # empty crop
    ("mode", 3, "mode"),
    ("lambda_", 0.0, "lambda"),
])
def test_bad_instances_are_rejected_before_device_work(lib, field, value, words):
    """Instance geometry the engine cannot run is refused with
    ATMWFS_ERR_INVALID and a message (the reference would index out of its
    arrays or exit), before any CUDA call: this runs without a GPU."""
    from atmosphericturbulencesimul_gb300 import _lib
    alt = (C.c_double * 2)(0.0, 5000.0)
    cn2 = (C.c_double * 2)(0.5, 0.5)
    spd = (C.c_double * 2)(10.0, 20.0)
    drc = (C.c_double * 2)(0.1, 1.0)
    inst = (_lib.Instance * 1)()
    inst[0].lambda_ = 1.6e-6
    inst[0].mode = 1
    inst[0].wf_raw_size = 256
    inst[0].wf_size = 256
    setattr(inst[0], field, value)
    p = _lib.Params()
    p.nlayers, p.alt, p.cn2, p.speed, p.dir = 2, alt, cn2, spd, drc
    p.fresnel_bin, p.pupil_scale, p.time_step, p.master_size = 100.0, 0.01, 0.001, 512
    p.amplitude, p.fresnel, p.ninst, p.inst, p.ring = 1, 1, 1, inst, 1
    ctx = C.c_void_p()
    assert lib.atmwfs_create(C.byref(p), C.byref(ctx)) == 1
    assert words in lib.atmwfs_last_error().decode()
