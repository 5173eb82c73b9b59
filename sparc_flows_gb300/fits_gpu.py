"""FITS files of device arrays: payload byte order converted on the GPU (csrc/sparc_fits.cu),
headers and file I/O on the host (fits.py).

write_fields / read_fields move many same-shaped fields at once through one pinned staging
buffer: the partial states the reference's forward and adjoint runs write and its kernel stage
reads, one file per field and record (all_modules.f90:750-784, kernels.f90:221-280).
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import capi, fits


def _prec(t: torch.Tensor) -> int:
    if t.dtype == torch.float32:
        return 32
    if t.dtype == torch.float64:
        return 64
    raise TypeError(f"FITS fields are float32 or float64, not {t.dtype}")


def write_fields(paths: list[str], fields: torch.Tensor, shape: tuple | None = None, bitpix: int = -64,
                 time: int | None = None) -> None:
    """fields: (nfiles, ...) CUDA tensor; file i holds fields[i] with NumPy shape `shape`
    (default fields.shape[1:]) as a BITPIX -64 (or -32) primary array."""
    L = capi.lib()
    f = fields.contiguous()
    nfile = f.shape[0]
    if nfile != len(paths):
        raise ValueError("one path per field")
    per = int(np.prod(f.shape[1:]))
    shape = tuple(f.shape[1:]) if shape is None else tuple(shape)
    if int(np.prod(shape)) != per:
        raise ValueError("shape does not match the field size")
    esize = 8 if bitpix == -64 else 4
    dev = torch.empty(nfile * per * esize, dtype=torch.uint8, device=f.device)
    stream = torch.cuda.current_stream(f.device)
    capi.check(L.sparc_fits_encode(ctypes.c_void_p(f.data_ptr()), _prec(f), nfile * per, bitpix,
                                   ctypes.c_void_p(dev.data_ptr()), ctypes.c_void_p(stream.cuda_stream)),
               "sparc_fits_encode")
    host = torch.empty(dev.numel(), dtype=torch.uint8).pin_memory()
    host.copy_(dev)  # synchronous: waits for the encode
    buf = host.numpy()
    for i, p in enumerate(paths):
        fits.write_raw(p, shape, buf[i * per * esize:(i + 1) * per * esize], time, bitpix)


def read_fields(paths: list[str], device, precision: int = 64) -> torch.Tensor:
    """Primary arrays (BITPIX -64 or -32, all the same shape and type) of the files, stacked as a
    (nfiles, *shape) tensor of the given precision on `device`."""
    L = capi.lib()
    shape = bitpix = None
    chunks = []
    for p in paths:
        with open(p, "rb") as fh:
            raw = fh.read()
        h = fits.parse_header(raw, p)
        if h["bitpix"] not in (-64, -32) or "BSCALE" in h or "BZERO" in h:
            raise ValueError(f"{p}: only unscaled BITPIX -64 / -32 arrays")
        if shape is None:
            shape, bitpix = h["shape"], h["bitpix"]
        elif (h["shape"], h["bitpix"]) != (shape, bitpix):
            raise ValueError(f"{p}: shape or type differs from {paths[0]}")
        n = int(np.prod(shape)) * (8 if bitpix == -64 else 4)
        if h["offset"] + n > len(raw):
            raise ValueError(f"{p}: truncated FITS data")
        chunks.append(np.frombuffer(raw, dtype=np.uint8, count=n, offset=h["offset"]))
    per = int(np.prod(shape))
    host = torch.from_numpy(np.concatenate(chunks)).pin_memory()
    dev = host.to(device, non_blocking=True)
    out = torch.empty((len(paths),) + tuple(shape), dtype=torch.float32 if precision == 32 else torch.float64,
                      device=device)
    stream = torch.cuda.current_stream(torch.device(device))
    capi.check(L.sparc_fits_decode(ctypes.c_void_p(dev.data_ptr()), bitpix, len(paths) * per,
                                   ctypes.c_void_p(out.data_ptr()), precision, ctypes.c_void_p(stream.cuda_stream)),
               "sparc_fits_decode")
    stream.synchronize()
    return out
