"""CPU emulation of the kernels' in-CTA building blocks (same template code):
Stockham FFT stages for every supported grid and radix plan, the transfer-table row
propagation, the TMA tile geometry of the bicubic screen gather, and the
FP32-only atan2 of the science unwrap."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent


@pytest.fixture(scope="module")
def emul_output(tmp_path_factory):
    exe = tmp_path_factory.mktemp("emul") / "pass_emul"
    cuda_inc = "/usr/local/cuda/include"
    if not Path(cuda_inc).exists() or shutil.which("g++") is None:
        pytest.skip("g++ or CUDA headers unavailable")
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", f"-I{cuda_inc}", f"-I{ROOT / 'atmosphericturbulencesimul_gb300' / 'csrc'}", f"-I{ROOT / 'include'}",
                    str(ROOT / "tests" / "emul" / "pass_emul.cpp"), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    return dict((l.split()[0], float(l.split()[1])) for l in out.strip().splitlines())


@pytest.mark.parametrize("n", [64, 128, 256, 512, 1024, "1024v1", 2048, 4096, 8192])
def test_fft_stages(emul_output, n):
    assert emul_output[f"fftfwd_{n}"] < 5e-7
    assert emul_output[f"fftinv_{n}"] < 5e-7
    assert emul_output[f"prop_{n}"] < 5e-7


def test_gather_geometry(emul_output):
    g = {k: v for k, v in emul_output.items() if k.startswith("gather_")}
    assert len(g) == 22
    for k, v in g.items():
        assert v < 1e-5, (k, v)


def test_atan2_fp32_only(emul_output):
    """The unwrap's float-float atan2 against (float)atan2 in double on about
    three million inputs (uniform, log-spread magnitudes, near the diagonal,
    on and beside the table points, signed zeros and the axes).  The
    float-float angle carries about 46 bits, so a result may differ by one
    unit in the last place only when the exact angle lies within 2^-46 of a
    midpoint between two floats: none occur in this set."""
    assert emul_output["atan2_count"] > 3_000_000
    assert emul_output["atan2_diff"] == 0
    assert emul_output["atan2_maxulp"] == 0


def test_atan2_output_epilogue(emul_output):
    """The last pass's FP32 atan2 (octant reduction and a degree-9 odd
    polynomial) against the double atan2 on about two million inputs: within
    3e-7 rad everywhere (one or two float roundings of pi near +-pi)."""
    assert emul_output["atan2out_count"] > 2_000_000
    assert emul_output["atan2out_maxerr"] < 3e-7
