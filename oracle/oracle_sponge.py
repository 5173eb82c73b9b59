"""ctypes wrapper of the 2-D sponge-step oracle (sparc_oracle_sponge.c).  TEST INFRASTRUCTURE
ONLY: imported by tests/ and __graft_entry__.smoke(); the product never imports it."""
import ctypes

import numpy as np

from . import oracle as _o

_dp = ctypes.POINTER(ctypes.c_double)


class Orc5Params(ctypes.Structure):
    _fields_ = [("nx", ctypes.c_int), ("nz", ctypes.c_int), ("npmlhor", ctypes.c_int),
                ("xlength", ctypes.c_double), ("timestep", ctypes.c_double), ("excitdep", ctypes.c_double),
                ("obsheight", ctypes.c_double), ("steps_out", ctypes.c_int), ("filter_all_x", ctypes.c_int),
                ("option", ctypes.c_int), ("npmlbot", ctypes.c_int), ("npmltop", ctypes.c_int)]


_bound = False


def _lib():
    global _bound
    L = _o.lib()
    if not _bound:
        L.orc5_create.restype = ctypes.c_void_p
        L.orc5_create.argtypes = [ctypes.POINTER(Orc5Params), _dp]
        L.orc5_destroy.argtypes = [ctypes.c_void_p]
        L.orc5_set_source.argtypes = [ctypes.c_void_p, _dp, _dp, ctypes.c_int]
        L.orc5_run.argtypes = [ctypes.c_void_p, ctypes.c_int, _dp]
        L.orc5_run.restype = ctypes.c_int
        L.orc5_get_state.argtypes = [ctypes.c_void_p, _dp]
        L.orc5_get_int.argtypes = [ctypes.c_void_p, ctypes.c_char_p]
        L.orc5_get_profile.argtypes = [ctypes.c_void_p, ctypes.c_char_p, _dp]
        L.orc5_get_profile.restype = ctypes.c_long
        L.orc5_set_magnetic.argtypes = [ctypes.c_void_p, _dp, _dp]
        _bound = True
    return L


def _p(a):
    return a.ctypes.data_as(_dp)


class SimSponge:
    """One 2-D option-5 (sponge), option-6 (PML) or option-12 (MHD with PML) solve on the CPU;
    state (5, nz, nx): rho, v_x, v_y, v_z, p, and for option 12 (8, nz, nx) with b_x, b_y, b_z."""

    def __init__(self, nx, model, xlength_cm, timestep=2.0, excitdep_cm=-150e5, obsheight_cm=200e5, npmlhor=9,
                 steps_out=15, filter_all_x=False, option=5, npmlbot=10, npmltop=10):
        self.L = _lib()
        self.nx, self.nz = nx, model.shape[0]
        p = Orc5Params(nx, self.nz, npmlhor, xlength_cm, timestep, excitdep_cm, obsheight_cm, steps_out,
                       int(filter_all_x), option, npmlbot, npmltop)
        m = np.ascontiguousarray(model, dtype=np.float64)
        self.h = self.L.orc5_create(ctypes.byref(p), _p(m))
        if not self.h:
            raise ValueError("orc5_create failed")
        self.nf = self.L.orc5_get_int(self.h, b"nf")

    def set_magnetic(self, box, boz):
        """Background field (nz, nx), nondimensional (B / dimb); option 12 only."""
        bx = np.ascontiguousarray(box, dtype=np.float64)
        bz = np.ascontiguousarray(boz, dtype=np.float64)
        if self.L.orc5_set_magnetic(self.h, _p(bx), _p(bz)) != 0:
            raise ValueError("set_magnetic needs option 12")

    def set_source(self, pattern, amp):
        pt = np.ascontiguousarray(pattern, dtype=np.float64)
        am = np.ascontiguousarray(amp, dtype=np.float64)
        self.L.orc5_set_source(self.h, _p(pt), _p(am), len(am))

    def run(self, nsteps):
        seis = np.zeros((max(nsteps, 1), self.nx))
        n = self.L.orc5_run(self.h, nsteps, _p(seis))
        return seis[:n]

    def state(self):
        a = np.zeros((self.nf, self.nz, self.nx))
        self.L.orc5_get_state(self.h, _p(a))
        return a

    def profile(self, name):
        out = np.zeros(self.nz)
        if self.L.orc5_get_profile(self.h, name.encode(), _p(out)) < 0:
            raise KeyError(name)
        return out

    def get_int(self, name):
        return self.L.orc5_get_int(self.h, name.encode())

    def close(self):
        if self.h:
            self.L.orc5_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
