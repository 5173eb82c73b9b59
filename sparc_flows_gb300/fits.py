"""Minimal FITS I/O for the ``sparc`` file contract (no astropy in this environment).

The reference writes one primary HDU with BITPIX = -64 (big-endian IEEE doubles), NAXIS = 3,
NAXIS1 = nx, NAXIS2 = ny, NAXIS3 = dim3 and a TIME keyword (all_modules.f90:296-378), and reads
the first nx*ny*dim3 values of the primary array (all_modules.f90:99-171).  Arrays here use the
NumPy order of such a file: shape (dim3, ny, nx).
"""
from __future__ import annotations

import numpy as np

BLOCK = 2880


def _card(key: str, value=None, comment: str = "") -> bytes:
    if value is None:
        s = f"{key:<8}"
    else:
        if isinstance(value, bool):
            v = "T" if value else "F"
        elif isinstance(value, (int, np.integer)):
            v = str(int(value))
        elif isinstance(value, float):
            v = repr(value).upper()
        else:
            v = f"'{value}'"
        s = f"{key:<8}= {v:>20}"
        if comment:
            s += f" / {comment}"
    return s[:80].ljust(80).encode("ascii")


def header(shape: tuple, time: int | None = None, bitpix: int = -64) -> bytes:
    """Primary header of an array of NumPy shape `shape`, padded to a 2880-byte block."""
    dims = tuple(shape)[::-1]  # FITS NAXIS1 is the fastest axis
    cards = [_card("SIMPLE", True), _card("BITPIX", bitpix), _card("NAXIS", len(dims))]
    for i, n in enumerate(dims, 1):
        cards.append(_card(f"NAXIS{i}", int(n)))
    cards.append(_card("EXTEND", False))
    if time is not None:
        cards.append(_card("TIME", int(time), "Also, init = time+1"))
    cards.append(_card("END"))
    hdr = b"".join(cards)
    return hdr + b" " * (-len(hdr) % BLOCK)


def write_raw(path: str, shape: tuple, payload, time: int | None = None, bitpix: int = -64) -> None:
    """Header plus an already encoded big-endian payload (bytes-like), zero-padded to a block."""
    body = memoryview(payload).cast("B")
    with open(path, "wb") as f:
        f.write(header(shape, time, bitpix))
        f.write(body)
        f.write(b"\0" * (-len(body) % BLOCK))


def write(path: str, data, time: int | None = None) -> None:
    """Write a 1..3-D array (NumPy order) as a BITPIX=-64 primary HDU."""
    a = np.ascontiguousarray(np.asarray(data, dtype=">f8"))
    write_raw(path, a.shape, a.tobytes(), time)


def parse_header(raw: bytes, path: str = "") -> dict:
    """Keywords of the primary header and the payload offset (key 'offset')."""
    hdr = {}
    pos = 0
    while True:
        if pos + BLOCK > len(raw):
            raise ValueError(f"{path}: truncated FITS header")
        block = raw[pos:pos + BLOCK]
        pos += BLOCK
        done = False
        for i in range(0, BLOCK, 80):
            card = block[i:i + 80].decode("ascii", "replace")
            key = card[:8].strip()
            if key == "END":
                done = True
                break
            if card[8:10] == "= ":
                hdr[key] = card[10:].split("/")[0].strip()
        if done:
            break
    bitpix = int(hdr["BITPIX"])
    naxis = int(hdr["NAXIS"])
    hdr["shape"] = tuple(int(hdr[f"NAXIS{i}"]) for i in range(naxis, 0, -1))
    hdr["bitpix"] = bitpix
    hdr["offset"] = pos
    return hdr


def read(path: str) -> np.ndarray:
    """Read the primary array of a FITS file (BITPIX -64, -32, 16, 32 or 64) in NumPy order."""
    with open(path, "rb") as f:
        raw = f.read()
    hdr = parse_header(raw, path)
    shape, pos = hdr["shape"], hdr["offset"]
    dt = {-64: ">f8", -32: ">f4", 16: ">i2", 32: ">i4", 64: ">i8"}[hdr["bitpix"]]
    n = int(np.prod(shape)) if shape else 0
    nbytes = n * np.dtype(dt).itemsize
    if pos + nbytes > len(raw):
        raise ValueError(f"{path}: truncated FITS data")
    a = np.frombuffer(raw[pos:pos + nbytes], dtype=dt).reshape(shape).astype(np.float64)
    bscale = float(hdr.get("BSCALE", "1").replace("D", "E"))
    bzero = float(hdr.get("BZERO", "0").replace("D", "E"))
    return a * bscale + bzero if (bscale != 1.0 or bzero != 0.0) else a
