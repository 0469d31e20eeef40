"""Primary-HDU FITS image read/write (BITPIX -32/-64/8/16/32), enough for the
files the reference's save_fl_fits / save_db_fits produce and for inputs it
reads with load_fits."""
from __future__ import annotations

from pathlib import Path

import numpy as np

_DTYPE = {8: ">u1", 16: ">i2", 32: ">i4", 64: ">i8", -32: ">f4", -64: ">f8"}


def _cards(hdr: bytes):
    for o in range(0, len(hdr), 80):
        c = hdr[o:o + 80].decode("ascii", "replace")
        key = c[:8].strip()
        if key == "END":
            return
        if c[8:10] == "= ":
            yield key, c[10:].split("/")[0].strip().strip("'").strip()


def read(path) -> np.ndarray:
    raw = Path(path).read_bytes()
    off, hdr = 0, b""
    while True:
        block = raw[off:off + 2880]
        if len(block) < 2880:
            raise ValueError(f"{path}: truncated header")
        hdr += block
        off += 2880
        if any(block[i:i + 8] == b"END     " for i in range(0, 2880, 80)):
            break
    kv = dict(_cards(hdr))
    bitpix, naxis = int(kv["BITPIX"]), int(kv["NAXIS"])
    shape = [int(kv[f"NAXIS{i}"]) for i in range(1, naxis + 1)]
    n = int(np.prod(shape)) if shape else 0
    dt = np.dtype(_DTYPE[bitpix])
    a = np.frombuffer(raw, dt, count=n, offset=off).astype(dt.newbyteorder("="))
    bscale, bzero = float(kv.get("BSCALE", 1.0)), float(kv.get("BZERO", 0.0))
    if bscale != 1.0 or bzero != 0.0:
        a = a * bscale + bzero
    return a.reshape(shape[::-1])


def write(path, a: np.ndarray) -> None:
    a = np.ascontiguousarray(a)
    bitpix = {np.dtype(np.float32): -32, np.dtype(np.float64): -64, np.dtype(np.uint8): 8,
              np.dtype(np.int16): 16, np.dtype(np.int32): 32}[a.dtype]
    cards = [f"{'SIMPLE':8s}= {'T':>20s}", f"{'BITPIX':8s}= {bitpix:>20d}", f"{'NAXIS':8s}= {a.ndim:>20d}"]
    cards += [f"{'NAXIS' + str(i + 1):8s}= {d:>20d}" for i, d in enumerate(a.shape[::-1])]
    cards.append("END")
    hdr = "".join(c.ljust(80) for c in cards)
    hdr += " " * (-len(hdr) % 2880)
    body = a.astype(_DTYPE[bitpix]).tobytes()
    body += b"\0" * (-len(body) % 2880)
    Path(path).write_bytes(hdr.encode("ascii") + body)
