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

from series_case import Case, compare, worst  # noqa: F401

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


@pytest.mark.parametrize("factor", ["1", "0"])
def test_phase_sum_factored_per_window_group(lib, oracle64, monkeypatch, factor):
    """Scoeff equal on all layers (a fixed gas mixture, the benchmark's
    case): the phase sum of every instance of a window group is its Scoeff
    times the group's compensated layer sum, formed once per step; the
    lambda-ref instance and the science instances of each direction read it
    in the last pass's epilogue and in the science apply.  A direction whose
    instances carry layer-dependent Scoeff keeps the per-instance sum in the
    same context; ATMWFS_GROUP_PHASE_SUM=0 turns the factoring off."""
    monkeypatch.setenv("ATMWFS_GROUP_PHASE_SUM", factor)
    case = bench_case(W=1024, Wout=1024, flat_scoeff=True, sci=[
        (0.5e-6, -TEN, -TEN, 256, 256),
        (2.2e-6, -TEN, -TEN, 512, 400),
        (1.25e-6, 0.0, 0.0, 1024, 1000),
        (2.4e-6, 0.0, 0.0, 512, 512),
        (0.9e-6, TEN, 0.0, 1024, 1024),
    ])
    ms = compare(case, oracle64, 2)
    _report(f"phase sum factored ({factor})", ms)


def test_phase_sum_factored_and_per_instance_groups(lib, oracle64, monkeypatch):
    """One group whose members' Scoeff factors beside groups whose members'
    does not (layer-dependent Scoeff): both kinds of phase sum in one step."""
    monkeypatch.delenv("ATMWFS_GROUP_PHASE_SUM", raising=False)
    case = bench_case(W=512, Wout=512, ref=False, sci=[
        (0.7e-6, TEN, TEN, 512, 512),
        (1.9e-6, TEN, TEN, 256, 200),
        (1.1e-6, 0.0, 0.0, 512, 500),
    ])
    from series_case import instances as inst_of, make_screens
    screens = make_screens(case, oracle64)
    flat = Case(**{**case.__dict__, "flat_scoeff": True})
    specs = inst_of(case)
    specs_flat = inst_of(flat)
    specs[2].scoeff = specs_flat[2].scoeff            # the on-axis direction factors
    assert np.all(specs[2].scoeff == specs[2].scoeff[0]) and not np.all(specs[0].scoeff == specs[0].scoeff[0])
    ms = compare(case, oracle64, 2, screens=screens, specs=specs)
    _report("factored and per-instance phase sums", ms)


@pytest.mark.parametrize("cfg", [0, 1, 2, 3, 4, 5])
def test_w1024_every_tile_configuration(lib, oracle64, monkeypatch, cfg):
    """The 1024^2 passes (gather, both propagations, epilogue, science bins on
    51 x 51 bins) in each compiled configuration: the 32 x 32 radix plan in
    three tile shapes (0-2), the 16 x 8 x 8 plan in two (3, 4), and the
    transfer tables staged in shared memory (5)."""
    monkeypatch.setenv("ATMWFS_TILE_CFG", str(cfg))
    case = bench_case(W=1024, Wout=1024, sci=[(0.5e-6, 0.0, 0.0), (1.6e-6, TEN, -TEN), (2.4e-6, -TEN, 0.0)])
    ms = compare(case, oracle64, 2)
    _report(f"W=1024 tile configuration {cfg}", ms)


@pytest.mark.parametrize("W,cfg", [(1024, 3), (1024, 4), (1024, 5), (512, 5)])
def test_alternative_configurations_grouped_layers(lib, oracle64, monkeypatch, W, cfg):
    """The 16 x 8 x 8 plan and the staged transfer tables on a plane of two
    layers (0 and 50 m share a super-layer: the second layer's window rows
    come from global memory), a crop and a lambda-ref instance."""
    monkeypatch.setenv("ATMWFS_TILE_CFG", str(cfg))
    case = Case(alt=[0.0, 50.0, 5000.0, 12000.0], cn2=[0.4, 0.2, 0.3, 0.1], speed=[8.0, 12.0, 25.0, 30.0],
                direction=[0.1, 1.0, 3.0, 5.5], M=2048, W=W, Wout=W - 24, fresnel_bin=100.0,
                sci=[(1.25e-6, 0.0, 0.0), (2.2e-6, TEN, -TEN)])
    ms = compare(case, oracle64, 2)
    _report(f"W={W} configuration {cfg}, grouped layers", ms)


def test_autotuner_reports_its_radix_plan(lib, oracle64, monkeypatch):
    """The autotuner times every configuration compiled for a grid size --
    at 1024 the 32 x 32 plan in three tile shapes and the 16 x 8 x 8 plan in
    two -- and reports the one it keeps; a forced configuration is taken as
    given, for every size or for the sizes listed as N:k."""
    from atmosphericturbulencesimul_gb300 import Series
    from series_case import instances, make_screens

    case = bench_case(W=1024, Wout=1024, sci=[(1.6e-6, 0.0, 0.0), (0.8e-6, 0.0, 0.0, 512, 512)])
    screens = make_screens(case, oracle64)

    def classes():
        s = Series(case.alt, case.cn2, case.speed, case.direction, master_size=case.M, instances=instances(case),
                   pupil_scale=case.pupil, time_step=case.dt, fresnel_bin=case.fresnel_bin, zangle=case.zangle,
                   amplitude=case.amplitude, fresnel=case.fresnel)
        for l, sc in enumerate(screens):
            s.load_screen(l, sc)
        s.run_frames(1)
        info = {ci["n"]: ci for ci in (s.class_info(c) for c in range(s.num_classes()))}
        # the step graph: the window kernel (one window group, side 1024), a
        # phase sum per class (the layer-dependent Scoeff does not factor),
        # 7 passes, the unwrap and the apply per class, the step counter
        assert s.step_kernels() == 1 + 2 + 2 * (7 + 2) + 1
        s.close()
        return info

    monkeypatch.delenv("ATMWFS_TILE_CFG", raising=False)
    info = classes()
    assert set(info) == {512, 1024}
    assert all(t > 0 for t in info[1024]["tuned_ms"])          # six configurations timed at 1024
    assert info[512]["tuned_ms"][3:5] == [0.0, 0.0]            # no alternative plan at 512
    assert info[512]["tuned_ms"][5] > 0                        # staged tables at 512
    for n, ci in info.items():
        assert int(np.prod(ci["radices"])) == n
        timed = [t for t in ci["tuned_ms"] if t > 0]
        assert ci["tuned_ms"][ci["cfg"]] == min(timed)
    print("\nautotuner:", json.dumps({n: {k: ci[k] for k in ("cfg", "radices", "rows_per_cta", "tuned_ms")}
                                      for n, ci in info.items()}))
    monkeypatch.setenv("ATMWFS_TILE_CFG", "3")
    info = classes()
    assert info[1024]["cfg"] == 3 and info[1024]["radices"] == [16, 8, 8] and info[1024]["rows_per_cta"] == 4
    assert info[512]["cfg"] == 0 and info[512]["radices"] == [32, 16]
    # per-size form: 512 forced to the staged tables, 1024 tuned
    monkeypatch.setenv("ATMWFS_TILE_CFG", "512:5")
    info = classes()
    assert info[512]["cfg"] == 5 and all(t == 0 for t in info[512]["tuned_ms"])
    assert all(t > 0 for t in info[1024]["tuned_ms"])
    assert info[1024]["tuned_ms"][info[1024]["cfg"]] == min(info[1024]["tuned_ms"])


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
