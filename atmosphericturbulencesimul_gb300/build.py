"""In-tree build of libatmwfs.so (CUDA kernels + C ABI) for sm_103a.

Every translation unit is compiled by its own nvcc process (in parallel) and
linked with the static CUDA runtime, so the library needs only the driver at
run time.  Re-running is cheap: objects newer than their sources are kept.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / "csrc"
BUILD = PKG / "_build"
LIB = PKG / "libatmwfs.so"
INCLUDE = ROOT / "include"

ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
# Host code is compiled without floating-point contraction so that the
# frozen-flow position updates round like the reference's x86 build (an FMA
# in `pos += v * dt` changes the last bit on Arm hosts).
NVCC_FLAGS = ["-std=c++17", "--expt-relaxed-constexpr", "-O3", "-lineinfo", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-ffp-contract=off",
              "-I", str(INCLUDE), "-I", str(CSRC)]
CC_FLAGS = ["-std=c11", "-O2", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-result", "-I", str(INCLUDE), "-I", str(CSRC)]
# host-only C++ (configuration, profile, FITS, shared memory, series driver)
CXX_FLAGS = ["-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-Wall", "-Wno-unused-result", "-I", str(INCLUDE),
             "-I", str(CSRC)]


def _cuda_include() -> list[str]:
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    inc = Path(nvcc).resolve().parent.parent / "include"
    return ["-I", str(inc)] if inc.exists() else []


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libatmwfs.so")
    return cand


def _headers() -> list[Path]:
    return sorted(CSRC.glob("*.cuh")) + sorted(CSRC.glob("*.h")) + sorted(INCLUDE.glob("*.h"))


def _stale(obj: Path, src: Path, deps: list[Path]) -> bool:
    if not obj.exists():
        return True
    t = obj.stat().st_mtime
    return src.stat().st_mtime > t or any(d.stat().st_mtime > t for d in deps)


def _run(cmd: list[str]) -> None:
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build step failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)


def build(verbose: bool = False, jobs: int | None = None) -> Path:
    """Compile every source under csrc/ and link libatmwfs.so; return its path."""
    BUILD.mkdir(exist_ok=True)
    nvcc = _nvcc()
    deps = _headers()
    cu = sorted(CSRC.glob("*.cu"))
    cc = sorted(CSRC.glob("*.c"))
    cxx = sorted(CSRC.glob("*.cpp"))
    jobs_list = []
    objs = []
    for src in cu:
        obj = BUILD / (src.stem + ".o")
        objs.append(obj)
        if _stale(obj, src, deps):
            jobs_list.append([nvcc, *ARCH, *NVCC_FLAGS, "-c", str(src), "-o", str(obj)])
    for src in cc:
        obj = BUILD / (src.stem + ".c.o")
        objs.append(obj)
        if _stale(obj, src, deps):
            jobs_list.append(["gcc", *CC_FLAGS, "-c", str(src), "-o", str(obj)])
    for src in cxx:
        obj = BUILD / (src.stem + ".cpp.o")
        objs.append(obj)
        if _stale(obj, src, deps):
            jobs_list.append(["g++", *CXX_FLAGS, *_cuda_include(), "-c", str(src), "-o", str(obj)])
    n = jobs or max(1, min(len(jobs_list), os.cpu_count() or 4))
    if jobs_list:
        with cf.ThreadPoolExecutor(max_workers=n) as ex:
            for fut in [ex.submit(_run, c) for c in jobs_list]:
                fut.result()
    if jobs_list or not LIB.exists() or any(o.stat().st_mtime > LIB.stat().st_mtime for o in objs):
        tmp = LIB.with_suffix(".so.tmp")
        _run([nvcc, *ARCH, "-shared", "-cudart", "static", "-o", str(tmp), *map(str, objs), "-lpthread", "-lrt", "-lm"])
        os.replace(tmp, LIB)
    if verbose:
        print(f"built {LIB}")
    return LIB


if __name__ == "__main__":
    build(verbose=True)
    sys.exit(0)
