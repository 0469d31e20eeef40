"""Learned surrogate of the multi-layer Fresnel propagation (include/atmwfs_fno.h).

A Fourier neural operator maps the per-layer phase windows of an instance
(plus its wavelength) to the diffraction correction D of the propagated
field, U = exp(i phi) (1 + D) with phi the geometric phase.  Its forward and
backward passes and its optimiser are the project's CUDA kernels in
libatmwfs.so; PyTorch only provides device buffers.  Training pairs come
from the plain engine (`PairSource`), which also judges the surrogate.
"""
from __future__ import annotations

import ctypes as C
import math
import os
from dataclasses import asdict, dataclass

import numpy as np

from . import _lib
from ._lib import check

ARCSEC = math.pi / 180.0 / 3600.0


@dataclass
class FnoConfig:
    nin: int = 8        # 7 layers + the wavelength plane
    width: int = 64
    modes: int = 32
    layers: int = 4
    proj: int = 128
    nout: int = 2
    grid: int = 256


def _ptr(t) -> int:
    return t.data_ptr()


class Surrogate:
    """The network: parameters, forward, loss gradient, Adam, files."""

    def __init__(self, cfg: FnoConfig | None = None, seed: int = 0, path: str | None = None):
        self._lib = _lib.load()
        h = C.c_void_p()
        if path is not None:
            check(self._lib.atmwfs_fno_load(os.fsencode(path), C.byref(h)))
            c = _lib.FnoCfg()
            check(self._lib.atmwfs_fno_get_cfg(h, C.byref(c)))
            cfg = FnoConfig(**{k: getattr(c, k) for k, _ in c._fields_})
        else:
            cfg = cfg or FnoConfig()
            c = _lib.FnoCfg(**asdict(cfg))
            check(self._lib.atmwfs_fno_create(C.byref(c), seed, C.byref(h)))
        self.cfg = cfg
        self._h = h

    def close(self):
        if self._h:
            self._lib.atmwfs_fno_destroy(self._h)
            self._h = None

    __del__ = close

    @property
    def num_params(self) -> int:
        return int(self._lib.atmwfs_fno_num_params(self._h))

    def get_params(self) -> np.ndarray:
        a = np.empty(self.num_params, np.float32)
        check(self._lib.atmwfs_fno_get_params(self._h, a.ctypes.data_as(C.POINTER(C.c_float))))
        return a

    def set_params(self, p) -> None:
        a = np.ascontiguousarray(p, np.float32)
        assert a.size == self.num_params
        check(self._lib.atmwfs_fno_set_params(self._h, a.ctypes.data_as(C.POINTER(C.c_float))))

    def get_grads(self) -> np.ndarray:
        a = np.empty(self.num_params, np.float32)
        check(self._lib.atmwfs_fno_get_grads(self._h, a.ctypes.data_as(C.POINTER(C.c_float))))
        return a

    def zero_grads(self, stream: int = 0) -> None:
        check(self._lib.atmwfs_fno_zero_grads(self._h, stream))

    def forward(self, x, out=None, stream: int = 0):
        """x: CUDA float32 tensor [B][nin][G][G] -> [B][nout][G][G]."""
        import torch
        B = x.shape[0]
        if out is None:
            out = torch.empty((B, self.cfg.nout, self.cfg.grid, self.cfg.grid), device=x.device, dtype=torch.float32)
        check(self._lib.atmwfs_fno_forward(self._h, _ptr(x), _ptr(out), B, stream))
        return out

    def loss_grad(self, x, target, out=None, stream: int = 0) -> float:
        import torch
        B = x.shape[0]
        if out is None:
            out = torch.empty((B, self.cfg.nout, self.cfg.grid, self.cfg.grid), device=x.device, dtype=torch.float32)
        loss = C.c_double()
        check(self._lib.atmwfs_fno_loss_grad(self._h, _ptr(x), _ptr(target), _ptr(out), B, C.byref(loss), stream))
        return float(loss.value)

    def adam(self, lr: float, beta1: float = 0.9, beta2: float = 0.999, eps: float = 1e-8, stream: int = 0) -> None:
        check(self._lib.atmwfs_fno_adam(self._h, lr, beta1, beta2, eps, stream))

    def save(self, path) -> None:
        check(self._lib.atmwfs_fno_save(self._h, os.fsencode(path)))


def gemm(A, B, C_out=None, *, ta=False, tb=False, alpha=1.0, beta=0.0, batch=1, sA=0, sB=0, sC=0, M=None, N=None,
         K=None, lda=None, ldb=None, ldc=None):
    """The surrogate's BF16 tensor-core product on CUDA tensors (FP32 or BF16 operands)."""
    import torch
    lib = _lib.load()
    abf = int(A.dtype == torch.bfloat16)
    bbf = int(B.dtype == torch.bfloat16)
    check(lib.atmwfs_gemm_bf16(M, N, K, _ptr(A), lda, int(ta), abf, _ptr(B), ldb, int(tb), bbf, _ptr(C_out), ldc,
                               alpha, beta, None, batch, sA, sB, sC, 0))
    return C_out


def prepare(win, lam, stream: int = 0):
    """windows [B][L][G][G] and wavelengths [B] (CUDA) -> (input [B][L+1][G][G], phi [B][G][G])."""
    import torch
    B, L, G, _ = win.shape
    x = torch.empty((B, L + 1, G, G), device=win.device, dtype=torch.float32)
    phi = torch.empty((B, G, G), device=win.device, dtype=torch.float32)
    check(_lib.load().atmwfs_fno_prepare(_ptr(win), _ptr(lam), B, L, G, _ptr(x), _ptr(phi), stream))
    return x, phi


def target(amp, pha, phi, stream: int = 0):
    import torch
    B, G, _ = amp.shape
    t = torch.empty((B, 2, G, G), device=amp.device, dtype=torch.float32)
    check(_lib.load().atmwfs_fno_target(_ptr(amp), _ptr(pha), _ptr(phi), B, G, _ptr(t), stream))
    return t


def assemble(out, phi, stream: int = 0):
    import torch
    B, _, G, _ = out.shape
    amp = torch.empty((B, G, G), device=out.device, dtype=torch.float32)
    pha = torch.empty((B, G, G), device=out.device, dtype=torch.float32)
    check(_lib.load().atmwfs_fno_assemble(_ptr(out), _ptr(phi), B, G, _ptr(amp), _ptr(pha), stream))
    return amp, pha


class PairSource:
    """Training / test pairs from the plain engine: `count` instances at
    wavelengths drawn from [lam_lo, lam_hi] and source offsets drawn within
    +-spread arcsec, on the 7-layer profile; every step() moves the windows
    by the wind over `dt` and returns (input, target, phi, amp, pha, lam)."""

    def __init__(self, count: int = 64, grid: int = 256, seed: int = 0, master: int = 1024, dt: float = 0.02,
                 lam_lo: float = 0.5e-6, lam_hi: float = 2.2e-6, spread: float = 30.0, lam_ref: float = 0.5e-6):
        import torch
        from .engine import MODE_REF, InstanceSpec, Series, master_screen
        from .refractivity import scoeff
        rng = np.random.default_rng(seed)
        alt = [0.0, 500.0, 1000.0, 2000.0, 4000.0, 8000.0, 16000.0]
        cn2 = [0.45, 0.15, 0.10, 0.10, 0.08, 0.07, 0.05]
        speed = list(rng.uniform(5.0, 30.0, 7))
        direction = list(rng.uniform(0.0, 2 * np.pi, 7))
        self.L, self.G, self.count = len(alt), grid, count
        self.alt, self.cn2, self.fresnel_bin, self.pupil = alt, cn2, 100.0, 0.01
        self.lam = rng.uniform(lam_lo, lam_hi, count)
        specs = [InstanceSpec(lam=float(l), mode=MODE_REF, src_x=float(rng.uniform(-spread, spread) * ARCSEC),
                              src_y=float(rng.uniform(-spread, spread) * ARCSEC), wf_raw_size=grid, wf_size=grid,
                              scoeff=scoeff(lam_ref, float(l), self.L)) for l in self.lam]
        self.series = Series(alt, cn2, speed, direction, master_size=master, instances=specs, pupil_scale=0.01,
                             time_step=dt, fresnel_bin=100.0)
        for l in range(self.L):
            s1, _, _ = master_screen(int(seed) * 1000 + l, master, 20.0 / 0.01, 0.01 / 0.01)
            self.series.load_screen(l, s1)
        self.series.normalize(np.float32(lam_ref), np.float32(0.5e-6 / 0.15 / ARCSEC))
        ff = self.series.frame_floats
        assert ff == count * grid * grid
        for i in range(count):
            assert self.series.frame_offset(i) == i * grid * grid
        dev = torch.device("cuda")
        self.pha = torch.empty((count, grid, grid), device=dev)
        self.amp = torch.empty((count, grid, grid), device=dev)
        self.win = torch.empty((count, self.L, grid, grid), device=dev)
        self.lam_t = torch.tensor(self.lam, device=dev, dtype=torch.float32)

    def step(self):
        s = self.series
        s.run(1, pha_ptr=self.pha.data_ptr(), amp_ptr=self.amp.data_ptr(), nslots=1)
        for i in range(self.count):
            s.windows_dev(i, self.win[i].data_ptr())
        x, phi = prepare(self.win, self.lam_t, s.stream)
        t = target(self.amp, self.pha, phi, s.stream)
        import torch
        torch.cuda.current_stream().wait_stream(torch.cuda.ExternalStream(s.stream))
        return x, t, phi, self.amp, self.pha, self.lam_t

    def close(self):
        self.series.close()


def field_errors(amp_p, pha_p, amp_t, pha_t, lam) -> dict:
    """Errors of a predicted field against the plain path's, per frame
    averaged: OPD rms (nm) of the wrapped phase difference, the same weighted
    by the plain path's intensity (the phase of near-dark pixels is ill
    defined), amplitude rms, and the relative error of the amplitude
    variance (scintillation)."""
    import torch
    d = torch.remainder(pha_p - pha_t + math.pi, 2 * math.pi) - math.pi
    nm = (lam.view(-1, 1, 1) / (2 * math.pi) * 1e9)
    opd = torch.sqrt(torch.mean((d * nm) ** 2, dim=(1, 2)))
    wgt = amp_t ** 2
    opdw = torch.sqrt(torch.sum(wgt * (d * nm) ** 2, dim=(1, 2)) / torch.sum(wgt, dim=(1, 2)))
    arms = torch.sqrt(torch.mean((amp_p - amp_t) ** 2, dim=(1, 2)))
    vt = torch.var(amp_t, dim=(1, 2))
    vp = torch.var(amp_p, dim=(1, 2))
    return {"opd_rms_nm": float(opd.mean()), "opd_wrms_nm": float(opdw.mean()), "amp_rms": float(arms.mean()),
            "scint_rel_err": float((torch.abs(vp - vt) / vt.clamp_min(1e-12)).mean())}


def evaluate(model: Surrogate, src: PairSource, steps: int = 4, batch: int = 8) -> dict:
    """Surrogate vs the geometric field exp(i phi) (no diffraction), both
    against the plain Fresnel path, over steps x src.count held-out frames."""
    import torch
    acc = {"model": [], "geometric": []}
    for _ in range(steps):
        x, t, phi, amp, pha, lam = src.step()
        for b0 in range(0, src.count, batch):
            sl = slice(b0, min(src.count, b0 + batch))
            out = model.forward(x[sl].contiguous())
            a_m, p_m = assemble(out, phi[sl].contiguous())
            torch.cuda.synchronize()
            acc["model"].append(field_errors(a_m, p_m, amp[sl], pha[sl], lam[sl]))
            acc["geometric"].append(field_errors(torch.ones_like(amp[sl]), phi[sl], amp[sl], pha[sl], lam[sl]))
            with torch.no_grad():
                dm = torch.mean((out - t[sl]) ** 2).item()
                d0 = torch.mean(t[sl] ** 2).item()
            acc["model"][-1]["mse"] = dm
            acc["geometric"][-1]["mse"] = d0
    return {k: {m: float(np.mean([e[m] for e in v])) for m in v[0]} for k, v in acc.items()}


def train(model: Surrogate, src: PairSource, pairs: int, batch: int = 8, lr: float = 1e-3, log=None) -> list:
    """Adam on `pairs` fresh plain-path pairs (src.count per engine step)."""
    losses = []
    seen = 0
    step = 0
    total_steps = max(1, pairs // batch)
    while seen < pairs:
        x, t, *_ = src.step()
        for b0 in range(0, src.count, batch):
            if seen >= pairs:
                break
            sl = slice(b0, min(src.count, b0 + batch))
            # cosine decay of the learning rate
            rate = lr * 0.5 * (1.0 + math.cos(math.pi * min(1.0, step / total_steps)))
            loss = model.loss_grad(x[sl].contiguous(), t[sl].contiguous())
            model.adam(rate)
            losses.append(loss)
            seen += sl.stop - sl.start
            step += 1
            if log and step % 50 == 0:
                log(f"step {step}: pairs {seen}, loss {loss:.4e}")
    return losses


def frame_flops(cfg: FnoConfig) -> float:
    """Floating-point operations of one inference frame, as the products execute them."""
    G, m, w, P = cfg.grid, cfg.modes, cfg.width, cfg.grid * cfg.grid
    f = 2.0 * w * cfg.nin * P
    per_layer = (2.0 * w * G * 2 * m * G            # DFT along x
                 + 2 * 2.0 * 2 * m * m * G * w      # DFT along y (two real products)
                 + 8.0 * w * w * m * m              # complex mode mixing
                 + 4 * 2.0 * G * m * m * w          # inverse along y (four real products)
                 + 2.0 * w * G * 2 * m * G          # inverse along x
                 + 2.0 * w * w * P)                 # pointwise mixing
    f += cfg.layers * per_layer
    f += 2.0 * cfg.proj * w * P + 2.0 * cfg.nout * cfg.proj * P
    return f


def frame_bytes(cfg: FnoConfig, bf16_act: bool | None = None) -> float:
    """HBM bytes one inference frame moves in the library's dataflow: FP32
    spectral images and pre-activations, each product reading its operands
    and writing its result once, the residual add and the activation in the
    pointwise epilogue, pre-activations that only training reads not stored;
    with bf16_act (ATMWFS_FNO_BF16_ACT=1; off by default) the activations
    between Fourier layers (h[1..]) and of the projection (q) stored as BF16.
    The algorithmic figure of the surrogate's HBM roofline."""
    if bf16_act is None:
        bf16_act = os.environ.get("ATMWFS_FNO_BF16_ACT", "0") == "1"
    ea = 2.0 if bf16_act else 4.0
    G, m, w, P = cfg.grid, cfg.modes, cfg.width, cfg.grid * cfg.grid
    spec_rows = 4.0 * w * G * 2 * m           # one x-DFT image (2m columns per row)
    modes = 4.0 * w * 2 * m * m               # one mode image (complex m x m per channel)
    b = 4.0 * cfg.nin * P + 4.0 * w * P       # lift: x in, h[0] out (FP32)
    for l in range(cfg.layers):
        eh = 4.0 if l == 0 else ea            # bytes of one element of h[l]
        last = l == cfg.layers - 1
        b += (eh * w * P + spec_rows          # h -> a
              + spec_rows + modes             # a -> z
              + 2 * modes                     # z -> y (mode mixing)
              + modes + spec_rows             # y -> bb
              + spec_rows + 4.0 * w * P       # bb -> u
              + eh * w * P + 4.0 * w * P      # pointwise: read h, u
              + (4.0 if last else ea) * w * P)  # write u (last layer) or gelu(u)
    b += 4.0 * w * P + ea * cfg.proj * P       # projection 1: u in, gelu out
    b += ea * cfg.proj * P + 4.0 * cfg.nout * P  # projection 2
    return b


def main(argv=None) -> int:
    """Train the surrogate on plain-path pairs and report its error on held-out seeds.

    python -m atmosphericturbulencesimul_gb300.fno --pairs 50000 --test 5000 --out fno256.bin --report r.json
    """
    import argparse
    import json
    import time

    import torch
    ap = argparse.ArgumentParser()
    ap.add_argument("--pairs", type=int, default=50000)
    ap.add_argument("--test", type=int, default=5000)
    ap.add_argument("--grid", type=int, default=256)
    ap.add_argument("--width", type=int, default=64)
    ap.add_argument("--modes", type=int, default=32)
    ap.add_argument("--layers", type=int, default=4)
    ap.add_argument("--proj", type=int, default=128)
    ap.add_argument("--batch", type=int, default=8)
    ap.add_argument("--lr", type=float, default=1e-3)
    ap.add_argument("--count", type=int, default=64, help="plain-path instances per engine step")
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--out", default=None)
    ap.add_argument("--report", default=None)
    a = ap.parse_args(argv)
    cfg = FnoConfig(grid=a.grid, width=a.width, modes=a.modes, layers=a.layers, proj=a.proj)
    src = PairSource(count=a.count, grid=a.grid, seed=a.seed)
    test = PairSource(count=a.count, grid=a.grid, seed=a.seed + 1000)
    model = Surrogate(cfg, seed=a.seed)
    torch.cuda.synchronize()
    t0 = time.time()
    losses = train(model, src, a.pairs, batch=a.batch, lr=a.lr, log=print)
    torch.cuda.synchronize()
    t_train = time.time() - t0
    ev = evaluate(model, test, steps=max(1, a.test // a.count), batch=a.batch)
    rep = {"config": asdict(cfg), "params": model.num_params, "pairs": a.pairs, "test_pairs": a.test,
           "train_s": t_train, "pairs_per_s": a.pairs / t_train, "final_loss": float(np.mean(losses[-50:])),
           "held_out": ev}
    print(json.dumps(rep))
    if a.out:
        model.save(a.out)
    if a.report:
        with open(a.report, "w") as f:
            json.dump(rep, f, indent=1)
    return 0


if __name__ == "__main__":
    raise SystemExit(main())
