"""FITS payloads encoded and decoded on the GPU (csrc/sparc_fits.cu, fits_gpu.py) against the
host FITS writer and reader (fits.py)."""
import os

import numpy as np
import pytest
import torch

from sparc_flows_gb300 import fits
from sparc_flows_gb300.fits_gpu import read_fields, write_fields

pytestmark = pytest.mark.gpu


def test_gpu_written_files_equal_host_written_files(tmp_path):
    rng = np.random.default_rng(0)
    a = rng.standard_normal((3, 7, 1, 9))
    paths = [str(tmp_path / f"g{i}.fits") for i in range(3)]
    write_fields(paths, torch.as_tensor(a, device="cuda"))
    for i, p in enumerate(paths):
        q = str(tmp_path / f"h{i}.fits")
        fits.write(q, a[i])
        assert open(p, "rb").read() == open(q, "rb").read()


@pytest.mark.parametrize("prec,bitpix", [(64, -64), (32, -64), (32, -32), (64, -32)])
def test_round_trip(tmp_path, prec, bitpix):
    dt = torch.float32 if prec == 32 else torch.float64
    x = torch.randn((4, 300, 1, 64), dtype=dt, device="cuda") * 1e-7
    paths = [str(tmp_path / f"r{i}.fits") for i in range(4)]
    write_fields(paths, x, bitpix=bitpix)
    back = read_fields(paths, "cuda", precision=prec)
    want = x.double().cpu().numpy()
    if bitpix == -32:
        want = want.astype(np.float32).astype(np.float64)
    assert np.array_equal(back.double().cpu().numpy(), want)
    assert np.array_equal(fits.read(paths[2]), want[2])
