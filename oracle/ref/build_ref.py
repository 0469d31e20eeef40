#!/usr/bin/env python3
"""Build the checker binary oracle/_ref/atmref from the reference's own C
sources (read in place under <reference root>/src) and the shims of this
directory (FFTW, cfitsio, GSL/libc noise, ncurses stand-ins).

The reference root is the first argument, else $ATMWFS_REFERENCE_ROOT, else
/root/reference.

Reference functions that the hot path never calls but that the compiled
modules reference are linked to generated stubs that abort if called.
Nothing is written outside oracle/_ref/.
"""
from __future__ import annotations

import os
import re
import subprocess
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent


def reference_root() -> Path:
    """Where the reference checkout lies (argument, environment, default)."""
    if len(sys.argv) > 1 and __name__ == "__main__":
        return Path(sys.argv[1])
    return Path(os.environ.get("ATMWFS_REFERENCE_ROOT", "/root/reference"))


REF = reference_root() / "src"
OUT = HERE.parent / "_ref"

# modules on the mkwfs path, the PSF consumers and their direct dependencies
REF_SOURCES = [
    "AtmosphericTurbulence/AtmosphericTurbulence.c",
    "WFpropagate/WFpropagate.c",
    "fft/fft.c",
    "AtmosphereModel/AtmosphereModel.c",
    "OpticsMaterials/OpticsMaterials.c",
    "COREMOD_memory/COREMOD_memory.c",
    "COREMOD_arith/COREMOD_arith.c",
    "COREMOD_tools/COREMOD_tools.c",
    "COREMOD_iofits/COREMOD_iofits.c",
    "image_gen/image_gen.c",
    "statistic/statistic.c",
    "info/info.c",
    "00CORE/00CORE.c",
    # the PSF consumers after the path and their image measures
    "psf/psf.c",
    "image_filter/image_filter.c",
]
SHIMS = ["shim_fftw.c", "shim_fitsio.c", "shim_rng_stubs.c", "atmref_driver.c"]
CFLAGS = ["-std=gnu99", "-O2", "-U_FORTIFY_SOURCE", "-D_FORTIFY_SOURCE=0", "-fcommon", "-w", "-ffp-contract=off", "-fno-builtin-rand",
          f"-I{HERE / 'shim'}", f"-I{REF}", '-DFFTCONFIGDIR="/tmp"']


def sh(cmd, check=True):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if check and r.returncode != 0:
        raise RuntimeError(" ".join(map(str, cmd)) + "\n" + r.stdout + r.stderr)
    return r


def build() -> Path:
    if not REF.exists():
        raise FileNotFoundError(f"{REF} not found: the checker binary is built only where the reference is mounted")
    OUT.mkdir(exist_ok=True)
    objs = []
    for s in REF_SOURCES:
        o = OUT / (Path(s).stem + ".o")
        sh(["gcc", *CFLAGS, "-c", str(REF / s), "-o", str(o)])
        objs.append(o)
    for s in SHIMS:
        o = OUT / (Path(s).stem + ".o")
        sh(["gcc", *CFLAGS, "-c", str(HERE / s), "-o", str(o)])
        objs.append(o)
    exe = OUT / "atmref"
    link = ["gcc", "-o", str(exe), *map(str, objs), "-lm", "-lpthread", "-lrt"]
    r = sh(link, check=False)
    if r.returncode != 0:
        missing = sorted(set(re.findall(r"undefined reference to `([^']+)'", r.stderr)))
        stub = OUT / "stubs.c"
        lines = ["/* generated: functions outside the mkwfs path */", "#include <stdio.h>", "#include <stdlib.h>"]
        for m in missing:
            lines.append(f'long {m}() {{ fprintf(stderr, "atmref: {m} is not part of the checker build\\n"); abort(); }}')
        stub.write_text("\n".join(lines) + "\n")
        so = OUT / "stubs.o"
        sh(["gcc", "-w", "-c", str(stub), "-o", str(so)])
        sh(link[:-3] + [str(so)] + link[-3:])
    return exe


if __name__ == "__main__":
    try:
        print(build())
    except FileNotFoundError as e:
        print(e)
        sys.exit(0)
