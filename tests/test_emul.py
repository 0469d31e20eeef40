"""CPU emulation of the kernels' in-CTA building blocks (same template code):
Stockham FFT stages for every supported grid, the transfer-table row
propagation, and the TMA tile geometry of the bicubic screen gather."""
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
    subprocess.run(["g++", "-std=c++17", "-O2", f"-I{cuda_inc}", f"-I{ROOT / 'atmosphericturbulencesimul_gb300' / 'csrc'}", f"-I{ROOT / 'include'}",
                    str(ROOT / "tests" / "emul" / "pass_emul.cpp"), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout
    return dict((l.split()[0], float(l.split()[1])) for l in out.strip().splitlines())


@pytest.mark.parametrize("n", [64, 128, 256, 512, 1024, 2048, 4096, 8192])
def test_fft_stages(emul_output, n):
    assert emul_output[f"fftfwd_{n}"] < 5e-7
    assert emul_output[f"fftinv_{n}"] < 5e-7
    assert emul_output[f"prop_{n}"] < 5e-7


def test_gather_geometry(emul_output):
    g = {k: v for k, v in emul_output.items() if k.startswith("gather_")}
    assert len(g) == 22
    for k, v in g.items():
        assert v < 1e-5, (k, v)
