"""The allocation-free Fresnel hop, called through the C ABI.

atmwfs_fresnel_noalloc serves callers that may not allocate device memory
while they run (a real-time loop feeding an adaptive-optics controller, a
host whose device memory is all handed to its own pool): it must give the
same field as the allocating atmwfs_fresnel_dev and as the FP64 oracle, call
after call, although every call reuses the same static scratch.  The calls go
small, large, then small again, so a call runs over scratch that a larger grid
left behind.  This file is collected last so that a run stopping at the first
failure has run every other test first.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# same bound as test_fresnel_matches_oracle (FP32 hop against FP64)
TOL = 2e-5

CALLS = [(256, 4000.0, 1.6e-6), (512, 800.0, 0.5e-6), (64, 12000.0, 2.2e-6)]


def _field(n, seed):
    rng = np.random.default_rng(seed)
    return np.exp(1j * rng.standard_normal((n, n)) * 3).astype(np.complex64)


def _dev(a):
    import torch
    return torch.from_numpy(a.view(np.float32).reshape(a.shape[0], 2 * a.shape[1]).copy()).cuda()


def test_noalloc_matches_allocating_path_and_oracle(lib, oracle64):
    import torch
    from atmosphericturbulencesimul_gb300 import _lib
    stream = torch.cuda.current_stream().cuda_stream
    dx = float(np.float32(0.01))
    for call, (n, z, lam) in enumerate(CALLS):
        host = _field(n, call)
        a = _dev(host)
        got = torch.empty_like(a)
        ref = torch.empty_like(a)
        _lib.check(lib.atmwfs_fresnel_noalloc(C.c_void_p(a.data_ptr()), C.c_void_p(got.data_ptr()), n, dx, z, lam,
                                              C.c_void_p(stream)))
        _lib.check(lib.atmwfs_fresnel_dev(C.c_void_p(a.data_ptr()), C.c_void_p(ref.data_ptr()), n, dx, z, lam,
                                          C.c_void_p(stream)))
        torch.cuda.synchronize()
        g = got.cpu().numpy().view(np.complex64)
        r = ref.cpu().numpy().view(np.complex64)
        err = np.abs(g - r).max() / np.abs(r).max()
        assert err < TOL, (call, n, "vs atmwfs_fresnel_dev", err)
        o = oracle64.fresnel(host.astype(np.complex128), dx, z, lam)
        err = np.abs(g - o).max() / np.abs(o).max()
        assert err < TOL, (call, n, "vs FP64 oracle", err)


def test_noalloc_rejects_sizes_above_its_scratch(lib):
    n = 1024
    a = _dev(_field(n, 9))
    out = a.clone()
    st = lib.atmwfs_fresnel_noalloc(C.c_void_p(a.data_ptr()), C.c_void_p(out.data_ptr()), n, 0.01, 100.0, 1e-6, None)
    assert st == 1
    assert b"512" in lib.atmwfs_last_error()
