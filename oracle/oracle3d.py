"""ctypes wrapper of the 3-D CPU FP64 oracle (sparc_oracle3d.c).  TEST INFRASTRUCTURE ONLY:
imported by tests/ and __graft_entry__.smoke(); the product never imports it."""
import ctypes

import numpy as np

from . import oracle as _o

_dp = ctypes.POINTER(ctypes.c_double)


class Orc3Params(ctypes.Structure):
    """Mirror of orc3_params."""

    _fields_ = [("nx", ctypes.c_int), ("ny", ctypes.c_int), ("nz", ctypes.c_int),
                ("npmlbot", ctypes.c_int), ("npmltop", ctypes.c_int),
                ("xlength", ctypes.c_double), ("ylength", ctypes.c_double), ("timestep", ctypes.c_double),
                ("excitdep", ctypes.c_double), ("obsheight", ctypes.c_double),
                ("steps_out", ctypes.c_int), ("filter_every", ctypes.c_int)]


_bound = False


def _lib():
    global _bound
    L = _o.lib()
    if not _bound:
        L.orc3_create.restype = ctypes.c_void_p
        L.orc3_create.argtypes = [ctypes.POINTER(Orc3Params), _dp]
        L.orc3_destroy.argtypes = [ctypes.c_void_p]
        L.orc3_set_flow.argtypes = [ctypes.c_void_p, _dp, _dp, _dp]
        L.orc3_set_source.argtypes = [ctypes.c_void_p, _dp, _dp, ctypes.c_int]
        L.orc3_step.argtypes = [ctypes.c_void_p]
        L.orc3_run.argtypes = [ctypes.c_void_p, ctypes.c_int, _dp]
        L.orc3_run.restype = ctypes.c_int
        L.orc3_get_state.argtypes = [ctypes.c_void_p, _dp, _dp]
        L.orc3_get_int.argtypes = [ctypes.c_void_p, ctypes.c_char_p]
        L.orc3_get_profile.argtypes = [ctypes.c_void_p, ctypes.c_char_p, _dp]
        L.orc3_get_profile.restype = ctypes.c_long
        L.orc3_get_double.argtypes = [ctypes.c_void_p, ctypes.c_char_p]
        L.orc3_get_double.restype = ctypes.c_double
        for f in ("orc3_ddx", "orc3_ddy"):
            getattr(L, f).argtypes = [ctypes.c_void_p, _dp, _dp]
        L.orc3_ddz.argtypes = [ctypes.c_void_p, _dp, _dp, ctypes.c_int]
        _bound = True
    return L


def _p(a):
    return a.ctypes.data_as(_dp)


class Sim3D:
    """One 3-D solve on the CPU (fields (nz, ny, nx))."""

    def __init__(self, nx, ny, nz, model, xlength_cm, ylength_cm, timestep=2.0, excitdep_cm=-150e5,
                 obsheight_cm=200e5, npmlbot=10, npmltop=10, steps_out=15, filter_every=2):
        self.L = _lib()
        p = Orc3Params(nx, ny, nz, npmlbot, npmltop, xlength_cm, ylength_cm, timestep, excitdep_cm,
                       obsheight_cm, steps_out, filter_every)
        self.nx, self.ny, self.nz = nx, ny, nz
        m = np.ascontiguousarray(model, dtype=np.float64)
        self.h = self.L.orc3_create(ctypes.byref(p), _p(m))
        if not self.h:
            raise ValueError("orc3_create failed (FFT size?)")

    def set_flow(self, v0x, v0y, v0z):
        a = [np.ascontiguousarray(v, dtype=np.float64) for v in (v0x, v0y, v0z)]
        self.L.orc3_set_flow(self.h, *[_p(v) for v in a])

    def set_source(self, pattern, amp):
        pt = np.ascontiguousarray(pattern, dtype=np.float64)
        am = np.ascontiguousarray(amp, dtype=np.float64)
        self.L.orc3_set_source(self.h, _p(pt), _p(am), len(am))

    def run(self, nsteps, max_records=None):
        nrec = max_records if max_records is not None else nsteps
        seis = np.zeros((max(nrec, 1), self.ny, self.nx))
        n = self.L.orc3_run(self.h, nsteps, _p(seis))
        return seis[:n]

    def state(self):
        a = np.zeros((6, self.nz, self.ny, self.nx))
        self.L.orc3_get_state(self.h, _p(a), None)
        return a

    def profile(self, name):
        out = np.zeros(self.nz)
        if self.L.orc3_get_profile(self.h, name.encode(), _p(out)) < 0:
            raise KeyError(name)
        return out

    def get_int(self, name):
        return self.L.orc3_get_int(self.h, name.encode())

    def get_double(self, name):
        return self.L.orc3_get_double(self.h, name.encode())

    def ddx(self, f):
        f = np.ascontiguousarray(f, dtype=np.float64)
        out = np.empty_like(f)
        self.L.orc3_ddx(self.h, _p(f), _p(out))
        return out

    def ddy(self, f):
        f = np.ascontiguousarray(f, dtype=np.float64)
        out = np.empty_like(f)
        self.L.orc3_ddy(self.h, _p(f), _p(out))
        return out

    def ddz(self, f, bc):
        f = np.ascontiguousarray(f, dtype=np.float64)
        out = np.empty_like(f)
        self.L.orc3_ddz(self.h, _p(f), _p(out), bc)
        return out

    def close(self):
        if self.h:
            self.L.orc3_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
