"""The C-ABI library loads, exports every function include/*.h declares, and its FP64
compact-derivative tables reproduce dbyd2.f (checked on the host, no GPU needed)."""
import ctypes
import glob
import os
import re

import numpy as np
import pytest

from oracle import oracle as O
from sparc_flows_gb300 import capi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_functions():
    names = []
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = re.sub(r"/\*.*?\*/", "", open(h).read(), flags=re.S)
        names += re.findall(r"^\s*(?:const\s+)?(?:\w+\s+)*\w+\s*\*?\s*(sparc_\w+)\s*\(", text, flags=re.M)
    return sorted(set(names))


def test_library_exports_every_declared_symbol():
    L = capi.lib()
    names = header_functions()
    assert "sparc_forward" in names and "sparc_plan_create" in names
    for n in names:
        assert hasattr(L, n), n
        assert n in capi.SIGNATURES, n


def test_plan_create_rejects_bad_config_without_gpu_work():
    L = capi.lib()
    cfg = capi.SparcConfig()
    cfg.nx, cfg.nz, cfg.nbatch, cfg.precision = 500, 300, 1, 32  # 500 is not in the FFT table
    cfg.npmlbot = cfg.npmltop = 10
    cfg.npmlhor = 9
    cfg.steps_out, cfg.k_inj, cfg.k_obs = 15, 100, 120
    h = ctypes.c_void_p()
    rc = L.sparc_plan_create(ctypes.byref(cfg), ctypes.byref(h))
    assert rc == -2 and not h.value
    assert b"nx" in L.sparc_last_error()
    assert L.sparc_plan_create(None, ctypes.byref(h)) == -1


def test_column_operator_rejects_bad_arguments_without_gpu_work():
    """sparc_colmat_apply (the discrete adjoint's transposed column operators) validates before any
    CUDA call: null or aliased buffers are SPARC_ERR_ARG with a message."""
    L = capi.lib()
    assert L.sparc_colmat_apply(None, 300, None, None, 1, 128, 0, 127, 0, None) == -1
    assert b"sparc_colmat_apply" in L.sparc_last_error()
    p = ctypes.c_void_p(4096)
    assert L.sparc_colmat_apply(p, 300, p, p, 1, 128, 0, 127, 0, None) == -1  # in == out
    assert b"aliased" in L.sparc_last_error()


@pytest.mark.parametrize("ibc", [0, 1, 2, 3])
@pytest.mark.parametrize("lmax", [16, 32])
def test_partitioned_tables_match_dbyd2(ibc, lmax):
    rng = np.random.default_rng(10 * ibc + lmax)
    nz, n1 = 300, 7
    b = rng.standard_normal((nz, n1))
    preset = rng.standard_normal(n1)
    pre_full = np.zeros((nz, n1))
    if ibc == 2:
        pre_full[0] = preset
    if ibc == 3:
        pre_full[nz - 1] = preset
    ref = O.dbyd2(b, ibc, preset=pre_full)
    out = np.zeros((nz, n1))
    dp = ctypes.POINTER(ctypes.c_double)
    rc = capi.lib().sparc_zsolve_host(nz, ibc, lmax, b.ctypes.data_as(dp), out.ctypes.data_as(dp),
                                      preset.ctypes.data_as(dp), n1)
    assert rc == 0
    assert np.abs(out - ref).max() <= 1e-12 * np.abs(ref).max()


@pytest.mark.parametrize("nz", [64, 100, 301, 384])
def test_partitioned_tables_other_depths(nz):
    rng = np.random.default_rng(nz)
    b = rng.standard_normal((nz, 3))
    ref = O.dbyd2(b, 1)
    out = np.zeros_like(b)
    dp = ctypes.POINTER(ctypes.c_double)
    rc = capi.lib().sparc_zsolve_host(nz, 1, 32, b.ctypes.data_as(dp), out.ctypes.data_as(dp), None, 3)
    assert rc == 0
    assert np.abs(out - ref).max() <= 1e-12 * np.abs(ref).max()


@pytest.mark.parametrize("ibc", [1, 2, 3])
@pytest.mark.parametrize("nz", [100, 300, 384])
def test_banded_form_matches_dbyd2(ibc, nz):
    """The banded inverse used by FP32 column passes: right-hand side as dbyd2 forms it, then a
    Toeplitz band of T^{-1} plus rank-2 corners; agrees with dbyd2 to 2e-9 of the result."""
    rng = np.random.default_rng(100 * ibc + nz)
    n1 = 5
    z = np.linspace(0.0, 1.0, nz)[:, None]
    b = np.sin(9.0 * z + rng.uniform(0, 6, n1)) + 0.05 * rng.standard_normal((nz, n1))
    preset = rng.standard_normal(n1)
    pre_full = np.zeros((nz, n1))
    if ibc == 2:
        pre_full[0] = preset
    if ibc == 3:
        pre_full[nz - 1] = preset
    ref = O.dbyd2(b, ibc, preset=pre_full)
    out = np.zeros((nz, n1))
    err = ctypes.c_double()
    dp = ctypes.POINTER(ctypes.c_double)
    rc = capi.lib().sparc_zband_host(nz, ibc, b.ctypes.data_as(dp), out.ctypes.data_as(dp),
                                     preset.ctypes.data_as(dp), n1, ctypes.byref(err))
    assert rc == 0
    assert err.value < 1e-9
    assert np.abs(out - ref).max() <= 2e-9 * np.abs(ref).max()
