"""GPU parity at the shapes the batched benchmark runs: the 7-layer profile
(0-16 km, the benchmark's seeded winds), 2048^2 master screens, propagation
grids of 256, 512, 1024 and 2048, off-axis sources on the benchmark's 10 arcsec
grid, science output with the bin unwrap and a lambda-ref instance, against the
FP64 oracle through the C ABI.

The layer loop and the hops follow AtmosphericTurbulence.c:2649-2692, the
window sampling :2806-2917 / :3133-3246, the outputs :3418-3476 and the
unwrap :3522-4260.  Bars (FP32 engine against the FP64 oracle): wrapped phase
error < 0.05 nm rms, amplitude error < 2e-3, relative OPD rms within 1e-4,
relative amplitude variance within 1e-3, a 2 pi jump of the unwrapped phase on
fewer than 0.2 % of the pixels.
"""
import json

import numpy as np
import pytest

from series_case import Case, compare, worst

pytestmark = pytest.mark.gpu

ARCSEC = np.pi / 180.0 / 3600.0
TEN = 10 * ARCSEC


def bench_case(**kw) -> Case:
    """The benchmark's profile (its own seeded winds and directions)."""
    from bench import workload
    wl = workload("batched")
    return Case(alt=wl["alt"], cn2=wl["cn2"], speed=[float(v) for v in wl["speed"]],
                direction=[float(v) for v in wl["direction"]], M=wl["M"], pupil=wl["pupil"], dt=wl["dt"],
                lam_ref=wl["lam_ref"], seeing=float(np.float32(wl["seeing"])), fresnel_bin=wl["fresnel_bin"], **kw)


def _report(name, ms):
    w = worst(ms)
    by_w = {}
    for m in ms:
        by_w.setdefault(m["W"], []).append(m["wrapped_rms_nm"])
    print(f"\n{name}: {len(ms)} frames, worst " + json.dumps({k: float(f"{v:.3g}") for k, v in w.items()})
          + ", worst wrapped nm by grid " + json.dumps({k: float(f"{max(v):.3g}") for k, v in sorted(by_w.items())}))


def test_one_context_mixing_grid_classes(lib, oracle64):
    """One context holding 256, 512 and 1024 instances (three grid classes,
    three graph branches writing one output ring), off-axis directions,
    several wavelengths, crops, a lambda-ref instance at 1024; the tile
    configuration of each class is the autotuner's pick."""
    case = bench_case(W=1024, Wout=1024, sci=[
        (0.5e-6, -TEN, -TEN, 256, 256),
        (2.2e-6, 0.0, -TEN, 256, 256),
        (0.8e-6, 0.0, TEN, 512, 512),
        (1.6e-6, TEN, TEN, 512, 400),
        (1.25e-6, TEN, 0.0, 1024, 1024),
        (2.4e-6, -TEN, TEN, 1024, 1000),
    ])
    ms = compare(case, oracle64, 3)
    assert {m["W"] for m in ms} == {256, 512, 1024}
    _report("mixed 256/512/1024", ms)


@pytest.mark.parametrize("cfg", [0, 1, 2])
def test_w1024_every_tile_configuration(lib, oracle64, monkeypatch, cfg):
    """The 1024^2 passes (gather, both propagations, epilogue, science bins on
    51 x 51 bins) in each compiled tile configuration."""
    monkeypatch.setenv("ATMWFS_TILE_CFG", str(cfg))
    case = bench_case(W=1024, Wout=1024, sci=[(0.5e-6, 0.0, 0.0), (1.6e-6, TEN, -TEN), (2.4e-6, -TEN, 0.0)])
    ms = compare(case, oracle64, 2)
    _report(f"W=1024 tile configuration {cfg}", ms)


def test_w2048_step(lib, oracle64):
    """One step at a 2048^2 propagation grid (the runtime three-stage plan)
    on 2048^2 screens, science and lambda-ref outputs."""
    case = bench_case(W=2048, Wout=2048, sci=[(1.6e-6, TEN, 0.0)])
    ms = compare(case, oracle64, 1)
    _report("W=2048", ms)


def test_window_group_of_mixed_grids(lib, oracle64):
    """One direction, wavelengths on 256, 512 and 1024 grids with crops: a
    single window group whose windows are 1024 x 1024; the smaller grids read
    its top-left corner, the crops their centre.  A second direction makes a
    second group."""
    case = bench_case(W=1024, Wout=1024, sci=[
        (0.6e-6, 0.0, 0.0, 256, 200),
        (0.9e-6, 0.0, 0.0, 512, 512),
        (1.3e-6, 0.0, 0.0, 1024, 800),
        (2.0e-6, 0.0, 0.0, 256, 256),
        (1.1e-6, TEN, TEN, 512, 300),
    ])
    ms = compare(case, oracle64, 2)
    _report("one window group, mixed grids", ms)
