"""ctypes binding of the C ABI in include/sparc_gb300.h (libsparc_gb300.so).

The library is the only compute path: if it cannot be loaded the import of the solver
fails loudly (there is no CPU fallback).
"""
from __future__ import annotations

import ctypes
import os

from . import _build

_LIB = None
_dp = ctypes.POINTER(ctypes.c_double)
_ip = ctypes.POINTER(ctypes.c_int)
_vp = ctypes.c_void_p

SPARC_OK = 0
ERRORS = {-1: "bad argument", -2: "unsupported size", -3: "non-finite state", -4: "device wait timed out",
          -5: "CUDA error", -6: "call out of order"}

# Every function declared in include/sparc_gb300.h, with its ctypes signature.
SIGNATURES = {
    "sparc_plan_create": (ctypes.c_int, [_vp, ctypes.POINTER(_vp)]),
    "sparc_plan_destroy": (ctypes.c_int, [_vp]),
    "sparc_last_error": (ctypes.c_char_p, []),
    "sparc_ddz": (ctypes.c_int, [_vp, _vp, _vp, ctypes.c_int, ctypes.c_int, _vp, _vp, _vp]),
    "sparc_ddzkern": (ctypes.c_int, [_vp, _vp, _vp, ctypes.c_int, ctypes.c_int, _vp, _vp]),
    "sparc_ddx": (ctypes.c_int, [_vp, _vp, _vp, ctypes.c_int, ctypes.c_double, _vp]),
    "sparc_set_background": (ctypes.c_int, [_vp, _vp, _vp]),
    "sparc_set_source": (ctypes.c_int, [_vp, _vp, _vp, ctypes.c_int, _dp, _ip, ctypes.c_int, _vp]),
    "sparc_reset_state": (ctypes.c_int, [_vp, ctypes.c_int, _vp]),
    "sparc_forward": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_double, _vp, _vp, ctypes.c_int, ctypes.c_int, _vp]),
    "sparc_forward_window": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_double, _vp, _vp, ctypes.c_int, ctypes.c_int,
                                            ctypes.c_int, _vp]),
    "sparc_checkpoint_bytes": (ctypes.c_size_t, [_vp]),
    "sparc_colmat_apply": (ctypes.c_int, [_vp, ctypes.c_int, _vp, _vp, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                          ctypes.c_int, ctypes.c_int, _vp]),
    "sparc_checkpoint_save": (ctypes.c_int, [_vp, _vp, _vp]),
    "sparc_checkpoint_load": (ctypes.c_int, [_vp, _vp, _vp]),
    "sparc_get_state": (ctypes.c_int, [_vp, _vp, _vp]),
    "sparc_set_state": (ctypes.c_int, [_vp, _vp, _vp]),
    "sparc_profile_passes": (ctypes.c_int, [_vp, ctypes.c_int, _dp, _vp]),
    "sparc_check_state": (ctypes.c_int, [_vp, _dp, _vp]),
    "sparc_get_time": (ctypes.c_int, [_vp, _ip, _vp]),
    "sparc_plan_describe": (ctypes.c_int, [_vp, ctypes.c_char_p, ctypes.c_int]),
    "sparc_kernels": (ctypes.c_int, [_vp, _vp, ctypes.c_int, _vp, ctypes.c_int, ctypes.c_int, _vp, _vp]),
    "sparc_kernels_accumulate": (ctypes.c_int, [_vp, _vp, ctypes.c_int, ctypes.c_int, _vp, _vp]),
    "sparc_kernels_accumulate_static": (ctypes.c_int, [_vp, _vp, ctypes.c_int, ctypes.c_int, _vp, _vp]),
    "sparc_adjoint": (ctypes.c_int, [_vp, _vp, ctypes.c_int, ctypes.c_int, _vp, _vp]),
    "sparc_zband_host": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, _dp, _dp, _dp, ctypes.c_int, _dp]),
    "sparc_zsolve_host": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, _dp, _dp, _dp, ctypes.c_int]),
    "sparc3d_plan_create": (ctypes.c_int, [_vp, ctypes.POINTER(_vp)]),
    "sparc3d_plan_destroy": (ctypes.c_int, [_vp]),
    "sparc3d_set_background": (ctypes.c_int, [_vp, _vp, _vp]),
    "sparc3d_set_source": (ctypes.c_int, [_vp, _vp, _dp, ctypes.c_int, _vp]),
    "sparc3d_reset_state": (ctypes.c_int, [_vp, ctypes.c_int, _vp]),
    "sparc3d_forward": (ctypes.c_int, [_vp, ctypes.c_int, _vp, ctypes.c_int, _ip, _vp]),
    "sparc3d_get_state": (ctypes.c_int, [_vp, _vp, _vp]),
    "sparc3d_set_state": (ctypes.c_int, [_vp, _vp, _vp]),
    "sparc3d_set_adjoint_source": (ctypes.c_int, [_vp, _vp, ctypes.c_int, _dp, _ip, ctypes.c_int, ctypes.c_double,
                                                  _vp]),
    "sparc3d_forward_records": (ctypes.c_int, [_vp, ctypes.c_int, _vp, ctypes.c_int, _ip, _vp, ctypes.c_int,
                                               ctypes.c_int, _vp]),
    "sparc3d_kernels_accumulate": (ctypes.c_int, [_vp, _vp, ctypes.c_int, _vp, _vp]),
    "sparc3d_checkpoint_bytes": (ctypes.c_size_t, [_vp]),
    "sparc3d_checkpoint_save": (ctypes.c_int, [_vp, _vp, _ip, _vp]),
    "sparc3d_checkpoint_load": (ctypes.c_int, [_vp, _vp, ctypes.c_int, _vp]),
    "sparc5_plan_create": (ctypes.c_int, [_vp, ctypes.POINTER(_vp)]),
    "sparc5_plan_destroy": (ctypes.c_int, [_vp]),
    "sparc5_set_background": (ctypes.c_int, [_vp, _vp, _vp]),
    "sparc5_set_source": (ctypes.c_int, [_vp, _vp, _dp, ctypes.c_int, _vp]),
    "sparc5_reset_state": (ctypes.c_int, [_vp, ctypes.c_int, _vp]),
    "sparc5_forward": (ctypes.c_int, [_vp, ctypes.c_int, _vp, ctypes.c_int, _ip, _vp]),
    "sparc5_get_state": (ctypes.c_int, [_vp, _vp, _vp]),
    "sparc_tt_plan_create": (ctypes.c_int, [ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                            ctypes.POINTER(_vp)]),
    "sparc_tt_plan_destroy": (ctypes.c_int, [_vp]),
    "sparc_tt_set_records": (ctypes.c_int, [_vp, _vp, _vp, _vp]),
    "sparc_tt_mode": (ctypes.c_int, [_vp, _vp, ctypes.c_int, _ip, ctypes.c_int, ctypes.c_int, ctypes.c_double, _dp,
                                     _vp]),
    "sparc_tt_misfit_mode": (ctypes.c_int, [_vp, _vp, ctypes.c_int, _ip, ctypes.c_int, ctypes.c_int,
                                            ctypes.c_double, _dp, _vp]),
    "sparc_tt_adjoint": (ctypes.c_int, [_vp, _vp, _vp]),
    "sparc_fits_encode": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_longlong, ctypes.c_int, _vp, _vp]),
    "sparc_fits_decode": (ctypes.c_int, [_vp, ctypes.c_int, ctypes.c_longlong, _vp, ctypes.c_int, _vp]),
    "sparc_grad_workspace_bytes": (ctypes.c_ulonglong, [ctypes.c_int, ctypes.c_int]),
    "sparc_gradient": (ctypes.c_int, [_vp, _vp, _vp, _vp, _vp, _vp, _vp]),
    "sparc_vec_dot": (ctypes.c_int, [ctypes.c_longlong, _vp, _vp, _vp, _dp, _vp, _vp]),
    "sparc_vec_axpby": (ctypes.c_int, [ctypes.c_longlong, ctypes.c_double, _vp, ctypes.c_double, _vp, _vp, _vp]),
    "sparc_update_direction": (ctypes.c_int, [ctypes.c_int, ctypes.c_longlong, _vp, _vp, _vp, _vp, _dp, _vp, _vp]),
    "sparc_lbfgs_direction": (ctypes.c_int, [ctypes.c_longlong, ctypes.c_int, _vp, _vp, _vp, _vp, _vp, _vp]),
    "sparc_linesearch_models": (ctypes.c_int, [ctypes.c_longlong, _vp, _vp, ctypes.c_int, _dp, _vp, _vp, _vp]),
}


class Sparc3DConfig(ctypes.Structure):
    """sparc3d_config_t."""

    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int), ("nbatch", ctypes.c_int),
                ("precision", ctypes.c_int), ("npmlbot", ctypes.c_int), ("npmltop", ctypes.c_int),
                ("deltat", ctypes.c_double), ("stretchx", ctypes.c_double), ("stretchy", ctypes.c_double),
                ("betas", ctypes.c_double * 5), ("flows", ctypes.c_int), ("steps_out", ctypes.c_int),
                ("k_src", ctypes.c_int), ("k_obs", ctypes.c_int), ("filter_every", ctypes.c_int)]


class Sparc5Config(ctypes.Structure):
    """sparc5_config_t."""

    _fields_ = [("nx", ctypes.c_int), ("nz", ctypes.c_int), ("nbatch", ctypes.c_int), ("precision", ctypes.c_int),
                ("npmlhor", ctypes.c_int), ("filter_all_x", ctypes.c_int), ("deltat", ctypes.c_double),
                ("stretchx", ctypes.c_double), ("betas", ctypes.c_double * 5), ("steps_out", ctypes.c_int),
                ("k_src", ctypes.c_int), ("k_obs", ctypes.c_int), ("option", ctypes.c_int),
                ("npmlbot", ctypes.c_int), ("npmltop", ctypes.c_int)]


class Sparc5Background(ctypes.Structure):
    """sparc5_background_t (device pointers)."""

    _fields_ = [(n, _vp) for n in ("stretch", "rhoinv", "rho0", "c2rho0", "gradp0_z", "gradrho0_z", "g",
                                    "source_dep", "sponge", "az", "bz", "box", "boz")]


class Sparc3DBackground(ctypes.Structure):
    """sparc3d_background_t (device pointers)."""

    _fields_ = [(n, _vp) for n in ("stretch", "rhoinv", "rho0", "c2rho0", "gradp0_z", "gradrho0_z", "g",
                                    "source_dep", "az", "bz", "v0x", "v0y", "v0z")]


class SparcGradConfig(ctypes.Structure):
    """sparc_grad_config_t."""

    _fields_ = [("nx", ctypes.c_int), ("nz", ctypes.c_int), ("nsrc", ctypes.c_int), ("nk", ctypes.c_double),
                ("sym", ctypes.c_int), ("zfilt", ctypes.c_int), ("zsigma", ctypes.c_double),
                ("hess_floor", ctypes.c_double), ("precondition", ctypes.c_int)]


class SparcConfig(ctypes.Structure):
    """sparc_config_t."""

    _fields_ = [
        ("nx", ctypes.c_int), ("nz", ctypes.c_int), ("nbatch", ctypes.c_int), ("precision", ctypes.c_int),
        ("npmlbot", ctypes.c_int), ("npmltop", ctypes.c_int), ("npmlhor", ctypes.c_int),
        ("deltat", ctypes.c_double), ("stretchx", ctypes.c_double), ("betas", ctypes.c_double * 5),
        ("flows", ctypes.c_int), ("c2d", ctypes.c_int), ("bg_per_solve", ctypes.c_int),
        ("steps_out", ctypes.c_int), ("k_inj", ctypes.c_int), ("k_obs", ctypes.c_int), ("src_until", ctypes.c_int),
        ("filter_k0", ctypes.c_int), ("filter_all_x", ctypes.c_int), ("compensated", ctypes.c_int),
        ("column_block", ctypes.c_int), ("column_impl", ctypes.c_int),
    ]


class SparcBackground(ctypes.Structure):
    """sparc_background_t (device pointers)."""

    _fields_ = [(n, _vp) for n in ("stretch", "unstretch", "rhoinv", "rho0", "gradp0_z", "gradrho0_z", "g", "fdz",
                                    "az", "bz", "ax", "bx", "c2rho0", "v0x", "v0z")]


class SparcError(RuntimeError):
    pass


def lib(build: bool = True):
    """Load (building first if sources changed) libsparc_gb300.so."""
    global _LIB
    if _LIB is None:
        path = _build.build() if build else _build.LIB_PATH
        if not os.path.exists(path):
            raise SparcError(f"CUDA extension missing: {path}")
        L = ctypes.CDLL(path)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(L, name)
            fn.restype = res
            fn.argtypes = args
        _LIB = L
    return _LIB


def check(rc: int, what: str):
    if rc != SPARC_OK:
        msg = lib().sparc_last_error()
        raise SparcError(f"{what} failed ({ERRORS.get(rc, rc)}): {msg.decode() if msg else ''}")
