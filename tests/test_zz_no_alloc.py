"""The allocation-free Fresnel hop, called through the C ABI.

atmwfs_fresnel_noalloc serves callers that may not allocate device memory
while they run (a real-time loop feeding an adaptive-optics controller, a
host whose device memory is all handed to its own pool): it must give the
same field as the allocating atmwfs_fresnel_dev, call after call, although
every call reuses the same static scratch.  This file is collected last so
that a run stopping at the first failure has run every other test first.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

# same bound as test_fresnel_matches_oracle
TOL = 2e-5


def _field(n, seed):
    import torch
    rng = np.random.default_rng(seed)
    a = np.exp(1j * rng.standard_normal((n, n)) * 3).astype(np.complex64)
    return torch.from_numpy(a.view(np.float32).reshape(n, 2 * n)).cuda()


def test_noalloc_matches_allocating_path_twice(lib):
    import torch
    from atmosphericturbulencesimul_gb300 import _lib
    stream = torch.cuda.current_stream().cuda_stream
    dx = float(np.float32(0.01))
    for call, (n, z, lam) in enumerate([(256, 4000.0, 1.6e-6), (512, 800.0, 0.5e-6)]):
        a = _field(n, call)
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
        assert err < TOL, (call, n, err)


def test_noalloc_rejects_sizes_above_its_scratch(lib):
    import torch
    n = 1024
    a = _field(n, 9)
    out = torch.empty_like(a)
    st = lib.atmwfs_fresnel_noalloc(C.c_void_p(a.data_ptr()), C.c_void_p(out.data_ptr()), n, 0.01, 100.0, 1e-6, None)
    assert st == 1
    assert b"512" in lib.atmwfs_last_error()
