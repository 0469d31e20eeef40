"""The surrogate's pointwise channel mixing on the tcgen05 tensor cores
(accumulator in tensor memory), called through the C ABI, against a plain
PyTorch FP32/FP64 product of the same BF16-rounded operands.

C[b] = W X[b] + bias + beta C[b] with W (o x c) BF16 and X[b] (c x P) FP32
rounded to BF16 on the way into shared memory; act = gelu(C) (tanh form).
Tolerance: products of BF16 values are exact in FP32 and c <= 128 of them
are summed, so the result matches to 1e-5 of the largest |C|; the GELU to
1e-5 absolute."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

torch = pytest.importorskip("torch")


def _run(lib, W, X, Cm, act, bias, beta, engine):
    B, c, P = X.shape
    o = W.shape[0]
    st = lib.atmwfs_fno_pointwise_dev(C.c_void_p(W.data_ptr()), o, c, C.c_void_p(X.data_ptr()),
                                      C.c_void_p(Cm.data_ptr()), B, P, beta, C.c_void_p(bias.data_ptr()),
                                      C.c_void_p(act.data_ptr() if act is not None else 0), engine,
                                      C.c_void_p(torch.cuda.current_stream().cuda_stream))
    torch.cuda.synchronize()
    return st


@pytest.mark.parametrize("o,c,P", [(64, 64, 65536), (128, 64, 4160), (64, 64, 200), (64, 8, 65536), (64, 8, 1000)])
def test_tcgen05_pointwise_matches_fp32(lib, o, c, P):
    from atmosphericturbulencesimul_gb300 import _lib
    g = torch.Generator(device="cuda").manual_seed(o * 1000 + P)
    B = 2
    W = (torch.randn((o, c), device="cuda", generator=g) / 8).to(torch.bfloat16)
    X = torch.randn((B, c, P), device="cuda", generator=g)
    bias = torch.randn((o,), device="cuda", generator=g)
    C0 = torch.randn((B, o, P), device="cuda", generator=g)
    ref = torch.einsum("oc,bcp->bop", W.double(), X.to(torch.bfloat16).double()) + bias.double()[None, :, None]
    ref = ref + 0.5 * C0.double()
    scale = float(ref.abs().max())
    lib.atmwfs_fno_umma_status(1)
    errs = {}
    for engine in (1, 2):
        Cm = C0.clone()
        # the lift shape (8 input planes, K padded to 16) has no activation
        act = torch.empty_like(C0) if c != 8 else None
        _lib.check(_run(lib, W, X, Cm, act, bias, 0.5, engine))
        errs[engine] = float((Cm.double() - ref).abs().max()) / scale
        if engine == 1 and act is not None:
            gelu = torch.nn.functional.gelu(Cm, approximate="tanh")
            assert float((act - gelu).abs().max()) < 1e-5
    print(f"\no={o} c={c} P={P}: relative error {errs[1]:.3g} (strides as laid out), {errs[2]:.3g} (exchanged)")
    assert lib.atmwfs_fno_umma_status(1) == 0
    assert errs[1] < 1e-5, errs
    assert errs[2] > 1e-2, errs


def test_tcgen05_pointwise_rejects_other_shapes(lib):
    W = torch.zeros((2, 128), device="cuda", dtype=torch.bfloat16)
    X = torch.zeros((1, 128, 256), device="cuda")
    Cm = torch.zeros((1, 2, 256), device="cuda")
    bias = torch.zeros((2,), device="cuda")
    assert _run(lib, W, X, Cm, None, bias, 0.0, 1) == 1


@pytest.mark.parametrize("o,c,P", [(64, 512, 32768), (512, 64, 32768), (64, 512, 1000), (512, 64, 1000)])
def test_tcgen05_spectral_product_matches_fp64(lib, o, c, P):
    """The Fourier layers' product along y (K = 512 in eight staged chunks of
    64 accumulated in tensor memory, or N = 512 as two MMAs of 256 per K
    step): C = W X against an FP64 product of the same BF16-rounded operands.
    Up to 512 exact BF16 products are summed in FP32, so the result matches
    to 1e-5 of the largest |C|; exchanging the descriptors' core-matrix
    strides (engine 2) must break it."""
    from atmosphericturbulencesimul_gb300 import _lib
    g = torch.Generator(device="cuda").manual_seed(o + c + P)
    W = (torch.randn((o, c), device="cuda", generator=g) / 16).to(torch.bfloat16)
    X = torch.randn((c, P), device="cuda", generator=g)
    ref = W.double() @ X.to(torch.bfloat16).double()
    scale = float(ref.abs().max())
    lib.atmwfs_fno_umma_status(1)
    errs = {}
    for engine in (1, 2):
        Cm = torch.full((o, P), float("nan"), device="cuda")
        _lib.check(lib.atmwfs_fno_spectral_dev(C.c_void_p(W.data_ptr()), o, c, C.c_void_p(X.data_ptr()),
                                               C.c_void_p(Cm.data_ptr()), P, engine,
                                               C.c_void_p(torch.cuda.current_stream().cuda_stream)))
        torch.cuda.synchronize()
        errs[engine] = float((Cm.double() - ref).abs().nan_to_num(float("inf")).max()) / scale
    print(f"\no={o} c={c} P={P}: relative error {errs[1]:.3g} (strides as laid out), {errs[2]:.3g} (exchanged)")
    assert lib.atmwfs_fno_umma_status(1) == 0
    assert errs[1] < 1e-5, errs
    assert errs[2] > 1e-2, errs


def _xspec(lib, Bt, A, maps, Cm, M, engine):
    n, k = Bt.shape
    return lib.atmwfs_fno_xspectral_dev(C.c_void_p(Bt.data_ptr()), n, k, C.c_void_p(A.data_ptr()), *maps[:5],
                                        C.c_void_p(Cm.data_ptr()), *maps[5:], M, engine,
                                        C.c_void_p(torch.cuda.current_stream().cuda_stream))


@pytest.mark.parametrize("direction", ["forward", "inverse"])
def test_tcgen05_x_spectral_products_match_fp64(lib, direction):
    """The Fourier layers' products along x through the network's planar
    layouts: the forward DFT reads lines of x values (K = 256 in four staged
    chunks) and writes the planar spectrum [2][G][B w][m]; the inverse reads
    that layout (two 32-value runs per row) and writes lines of 256 values.
    Against an FP64 product of the same BF16-rounded operands on the same
    index maps (1e-5 of the largest |C|); exchanged descriptor strides must
    break it."""
    from atmosphericturbulencesimul_gb300 import _lib
    G, m, BW = 256, 32, 6           # grid, modes, samples x width
    Nc = BW * m
    M = BW * G
    g = torch.Generator(device="cuda").manual_seed(11 if direction == "forward" else 12)
    if direction == "forward":
        n, k = 2 * m, G
        A = torch.randn((BW, G, G), device="cuda", generator=g)          # h[bc][y][x]
        Ad = A.reshape(M, G)
        maps = (0, G, 0, G, 0, G, Nc, m, m, G * Nc)
        Cm = torch.full((2, G, BW, m), float("nan"), device="cuda")      # a[p][y][bc][kx]
    else:
        n, k = G, 2 * m
        A = torch.randn((2, G, BW, m), device="cuda", generator=g)       # bb[p][y][bo][kx]
        Ad = A.permute(2, 1, 0, 3).reshape(M, 2 * m)                     # rows (bo, y), K (p, kx)
        maps = (G, Nc, m, m, G * Nc, 0, G, 0, G, 0)
        Cm = torch.full((BW, G, G), float("nan"), device="cuda")         # spec[bo][y][x]
    Bt = (torch.randn((n, k), device="cuda", generator=g) / 16).to(torch.bfloat16)
    ref = Ad.to(torch.bfloat16).double() @ Bt.double().t()              # (M, n)
    if direction == "forward":
        ref = ref.reshape(BW, G, 2, m).permute(2, 1, 0, 3)               # -> [p][y][bc][kx]
    else:
        ref = ref.reshape(BW, G, G)
    scale = float(ref.abs().max())
    lib.atmwfs_fno_umma_status(1)
    errs = {}
    for engine in (1, 2):
        Cm.fill_(float("nan"))
        _lib.check(_xspec(lib, Bt, A, maps, Cm, M, engine))
        torch.cuda.synchronize()
        errs[engine] = float((Cm.double() - ref).abs().nan_to_num(float("inf")).max()) / scale
    print(f"\nx {direction}: relative error {errs[1]:.3g} (strides as laid out), {errs[2]:.3g} (exchanged)")
    assert lib.atmwfs_fno_umma_status(1) == 0
    assert errs[1] < 1e-5, errs
    assert errs[2] > 1e-2, errs
