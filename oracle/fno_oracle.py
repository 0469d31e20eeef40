"""FP64 numpy restatement of the surrogate's Fourier neural operator
(atmosphericturbulencesimul_gb300/csrc/fno.cu): forward pass and a
hand-derived backward pass over the same flat parameter layout.

Test infrastructure only (the oracle): it checks the GPU kernels' outputs
and gradients; it is pinned itself against finite differences
(tests/test_fno_oracle.py).  The reference simulator has no learned path,
so there is no reference code to follow; the model is defined by fno.cu's
header comment:
    h0 = Wlift x + blift
    u_l = W_l h_l + b_l + S_l(h_l),  h_{l+1} = gelu(u_l) (identity after the last layer)
    out = P2 gelu(P1 h + c1) + c2
    S(h) = Re(Gx Gy R Fy Fx h) on the modes ky in [-m/2, m/2), kx in [0, m).
"""
from __future__ import annotations

from dataclasses import dataclass

import numpy as np


@dataclass
class Cfg:
    nin: int
    width: int
    modes: int
    layers: int
    proj: int
    nout: int
    grid: int


def layout(c: Cfg) -> dict:
    """Offsets of every tensor in the flat parameter vector (fno.cu FnoLayout)."""
    o = 0
    L = {}

    def take(name, n):
        nonlocal o
        L[name] = (o, n)
        o += n

    take("lift_W", c.width * c.nin)
    take("lift_b", c.width)
    for l in range(c.layers):
        take(f"R{l}", c.modes * c.modes * c.width * c.width * 2)
        take(f"W{l}", c.width * c.width)
        take(f"b{l}", c.width)
    take("proj1_W", c.proj * c.width)
    take("proj1_b", c.proj)
    take("proj2_W", c.nout * c.proj)
    take("proj2_b", c.nout)
    L["_total"] = (0, o)
    return L


def unpack(p: np.ndarray, c: Cfg) -> dict:
    L = layout(c)
    t = {}
    for k, (o, n) in L.items():
        if k == "_total":
            continue
        a = p[o:o + n]
        if k.startswith("R"):
            a = a.reshape(c.modes, c.modes, c.width, c.width, 2)
            a = a[..., 0] + 1j * a[..., 1]           # [ky][kx][o][c]
        elif k == "lift_W":
            a = a.reshape(c.width, c.nin)
        elif k.startswith("W"):
            a = a.reshape(c.width, c.width)
        elif k == "proj1_W":
            a = a.reshape(c.proj, c.width)
        elif k == "proj2_W":
            a = a.reshape(c.nout, c.proj)
        t[k] = a
    return t


def pack_grads(g: dict, c: Cfg) -> np.ndarray:
    L = layout(c)
    out = np.zeros(L["_total"][1])
    for k, (o, n) in L.items():
        if k == "_total":
            continue
        a = g[k]
        if k.startswith("R"):
            a = np.stack([a.real, a.imag], axis=-1)
        out[o:o + n] = np.asarray(a, np.float64).ravel()
    return out


def _gelu(x):
    c = np.sqrt(2.0 / np.pi)
    return 0.5 * x * (1.0 + np.tanh(c * (x + 0.044715 * x ** 3)))


def _gelu_d(x):
    c = np.sqrt(2.0 / np.pi)
    t = np.tanh(c * (x + 0.044715 * x ** 3))
    return 0.5 * (1.0 + t) + 0.5 * x * (1.0 - t * t) * c * (1.0 + 3.0 * 0.044715 * x * x)


def _mats(c: Cfg):
    G, m = c.grid, c.modes
    x = np.arange(G)
    kx = np.arange(m)
    ky = np.array([j if j < m // 2 else j - m for j in range(m)])
    Fx = np.exp(-2j * np.pi * np.outer(x, kx) / G)            # [x][kx]
    Fy = np.exp(-2j * np.pi * np.outer(ky, x) / G)            # [ky][y]
    Gy = np.exp(2j * np.pi * np.outer(x, ky) / G)             # [y][ky]
    ck = np.where(kx == 0, 1.0, 2.0) / (G * G)
    Gx = ck[:, None] * np.exp(2j * np.pi * np.outer(kx, x) / G)   # [kx][x]
    return Fx, Fy, Gy, Gx


def _spectral(h, R, M):
    Fx, Fy, Gy, Gx = M
    a = h @ Fx                                                # [B][c][y][kx]
    z = np.einsum("jy,bcyk->bcjk", Fy, a)                     # [B][c][ky][kx]
    y = np.einsum("jkoc,bcjk->bojk", R, z)
    bb = np.einsum("yj,bojk->boyk", Gy, y)
    s = np.real(bb @ Gx)                                      # [B][o][y][x]
    return s, (a, z, y, bb)


def _spectral_bwd(ds, h, R, saved, M):
    Fx, Fy, Gy, Gx = M
    a, z, y, bb = saved
    dbb = ds @ np.conj(Gx).T                                  # complex gradient of bb
    dy = np.einsum("yj,boyk->bojk", np.conj(Gy), dbb)
    dz = np.einsum("jkoc,bojk->bcjk", np.conj(R), dy)
    dR = np.einsum("bojk,bcjk->jkoc", dy, np.conj(z))
    da = np.einsum("jy,bcjk->bcyk", np.conj(Fy), dz)
    dh = np.real(da @ np.conj(Fx).T)
    return dh, dR


def forward(p: np.ndarray, x: np.ndarray, c: Cfg, keep: bool = False):
    """out [B][nout][G][G] for input x [B][nin][G][G]."""
    t = unpack(np.asarray(p, np.float64), c)
    M = _mats(c)
    x = np.asarray(x, np.float64)
    h = np.einsum("oc,bcyx->boyx", t["lift_W"], x) + t["lift_b"][None, :, None, None]
    hs, us, sp = [h], [], []
    for l in range(c.layers):
        s, saved = _spectral(h, t[f"R{l}"], M)
        u = np.einsum("oc,bcyx->boyx", t[f"W{l}"], h) + t[f"b{l}"][None, :, None, None] + s
        h = _gelu(u) if l + 1 < c.layers else u
        us.append(u)
        sp.append(saved)
        hs.append(h)
    qpre = np.einsum("oc,bcyx->boyx", t["proj1_W"], h) + t["proj1_b"][None, :, None, None]
    q = _gelu(qpre)
    out = np.einsum("oc,bcyx->boyx", t["proj2_W"], q) + t["proj2_b"][None, :, None, None]
    if keep:
        return out, dict(t=t, M=M, x=x, hs=hs, us=us, sp=sp, qpre=qpre, q=q)
    return out


def loss_grad(p: np.ndarray, x: np.ndarray, target: np.ndarray, c: Cfg):
    """(mean squared error, flat gradient) as atmwfs_fno_loss_grad computes them."""
    out, k = forward(p, x, c, keep=True)
    t, M = k["t"], k["M"]
    d = out - np.asarray(target, np.float64)
    loss = float(np.mean(d * d))
    dout = 2.0 * d / d.size
    g = {}
    g["proj2_W"] = np.einsum("boyx,bcyx->oc", dout, k["q"])
    g["proj2_b"] = dout.sum(axis=(0, 2, 3))
    dq = np.einsum("oc,boyx->bcyx", t["proj2_W"], dout) * _gelu_d(k["qpre"])
    h = k["hs"][-1]
    g["proj1_W"] = np.einsum("boyx,bcyx->oc", dq, h)
    g["proj1_b"] = dq.sum(axis=(0, 2, 3))
    dh = np.einsum("oc,boyx->bcyx", t["proj1_W"], dq)
    for l in range(c.layers - 1, -1, -1):
        u = k["us"][l]
        du = dh * _gelu_d(u) if l + 1 < c.layers else dh
        hl = k["hs"][l]
        g[f"W{l}"] = np.einsum("boyx,bcyx->oc", du, hl)
        g[f"b{l}"] = du.sum(axis=(0, 2, 3))
        dsp, dR = _spectral_bwd(du, hl, t[f"R{l}"], k["sp"][l], M)
        g[f"R{l}"] = dR
        dh = np.einsum("oc,boyx->bcyx", t[f"W{l}"], du) + dsp
    g["lift_W"] = np.einsum("boyx,bcyx->oc", dh, k["x"])
    g["lift_b"] = dh.sum(axis=(0, 2, 3))
    return loss, pack_grads(g, c)


def init_params(c: Cfg, seed: int) -> np.ndarray:
    """A random parameter vector for tests (not the GPU initialiser)."""
    rng = np.random.default_rng(seed)
    p = np.zeros(layout(c)["_total"][1])
    for k, (o, n) in layout(c).items():
        if k == "_total":
            continue
        s = 1.0 / np.sqrt(c.width) if not k.startswith("R") else 0.5 / c.width
        p[o:o + n] = rng.uniform(-s, s, n)
    return p
