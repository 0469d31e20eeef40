"""Frames delivered through atmwfs_run into the three kinds of sink: pageable
host arrays (copy engine), pinned host memory and device memory (the copy
kernel).  The same seeded series gives bit-identical frames in all three,
with a host ring shorter than the run (frames reused round-robin).  Every
frame is a deterministic function of the inputs (the science bins are summed
in fixed point, so the order in which CTAs add their parts does not matter),
so the three runs, λref and science instances alike, agree bit for bit."""
import numpy as np
import pytest

from series_case import Case, instances, make_screens

pytestmark = pytest.mark.gpu


def _series(case, screens):
    from atmosphericturbulencesimul_gb300 import Series
    s = Series(case.alt, case.cn2, case.speed, case.direction, master_size=case.M, instances=instances(case),
               pupil_scale=case.pupil, time_step=case.dt, fresnel_bin=case.fresnel_bin, zangle=case.zangle,
               amplitude=case.amplitude, fresnel=case.fresnel, ring=2)
    for l, sc in enumerate(screens):
        s.load_screen(l, sc)
    return s


@pytest.fixture
def fixed_tiles(monkeypatch):
    """One tile configuration for every series of a test: the autotuner of
    each series could otherwise pick another shape, which groups the
    per-CTA parts of the science bins differently."""
    monkeypatch.setenv("ATMWFS_TILE_CFG", "2")


def test_sinks_give_identical_frames(lib, oracle64, fixed_tiles):
    torch = pytest.importorskip("torch")
    case = Case(alt=[0.0, 1000.0, 5000.0], cn2=[0.6, 0.3, 0.1], speed=[8.0, 12.0, 20.0], direction=[0.0, 1.0, 2.5],
                sci=[(1.6e-6, 0.0, 0.0), (2.2e-6, 1e-5, 0.0)])
    screens = make_screens(case, oracle64)
    nsteps, nslots = 5, 3
    out = {}
    for kind in ("pageable", "pinned", "device"):
        s = _series(case, screens)
        ff = s.frame_floats
        if kind == "pageable":
            pha = np.zeros(nslots * ff, np.float32)
            amp = np.zeros(nslots * ff, np.float32)
            s.run(nsteps, pha=pha, amp=amp, nslots=nslots)
        else:
            dev = "cuda" if kind == "device" else "cpu"
            tp = torch.zeros(nslots * ff, dtype=torch.float32, device=dev, pin_memory=(kind == "pinned"))
            ta = torch.zeros(nslots * ff, dtype=torch.float32, device=dev, pin_memory=(kind == "pinned"))
            s.run(nsteps, pha_ptr=tp.data_ptr(), amp_ptr=ta.data_ptr(), nslots=nslots)
            torch.cuda.synchronize()
            pha, amp = tp.cpu().numpy(), ta.cpu().numpy()
        out[kind] = (pha.copy(), amp.copy())
        s.close()
    ref_pha, ref_amp = out["pageable"]
    assert np.isfinite(ref_pha).all() and np.abs(ref_amp).max() > 0
    for kind in ("pinned", "device"):
        assert np.array_equal(out[kind][0], ref_pha), kind
        assert np.array_equal(out[kind][1], ref_amp), kind


def test_time_pass_leaves_the_series_unchanged(lib, oracle64, fixed_tiles):
    """Timing every pass of every grid class between two runs (the last pass
    included, which adds science bin sums) leaves the following frames equal
    to those of a series that was not timed."""
    case = Case(alt=[0.0, 1000.0, 5000.0], cn2=[0.6, 0.3, 0.1], speed=[8.0, 12.0, 20.0], direction=[0.0, 1.0, 2.5],
                sci=[(1.6e-6, 0.0, 0.0), (2.2e-6, 1e-5, 0.0)])
    screens = make_screens(case, oracle64)
    a, b = _series(case, screens), _series(case, screens)
    fa = a.run_frames(4)
    fb1 = b.run_frames(2)
    nplanes = len(b.planes()[0])
    for c in range(b.num_classes()):
        for k in range(nplanes + 1):
            b.time_pass(k, c, reps=2)
    fb2 = b.run_frames(2)
    a.close()
    b.close()
    for (pa, aa), (p1, a1), (p2, a2) in zip(fa, fb1, fb2):
        assert np.array_equal(pa[:2], p1) and np.array_equal(aa[:2], a1)
        assert np.array_equal(pa[2:], p2) and np.array_equal(aa[2:], a2)
