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
        L.orc3_set_adjoint_source.argtypes = [ctypes.c_void_p, _dp, ctypes.c_int, _dp, ctypes.POINTER(ctypes.c_int),
                                              ctypes.c_int, ctypes.c_double]
        L.orc3_advance.argtypes = [ctypes.c_void_p]
        L.orc3_advance.restype = ctypes.c_int
        L.orc3_get_scr.argtypes = [ctypes.c_void_p, _dp]
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

    def set_adjoint_source(self, rows, w, idx, scale):
        """Kernel-mode adjoint source (displacement.f90:615-627): rows (nrows, ny, nx), LAGRANGE_INTERP
        table w (ntab, 7), idx (ntab,), scale = delta_width / rho0(o_rad)."""
        self._adj = (np.ascontiguousarray(rows, dtype=np.float64), np.ascontiguousarray(w, dtype=np.float64),
                     np.ascontiguousarray(idx, dtype=np.int32))
        r, ww, ii = self._adj
        self.L.orc3_set_adjoint_source(self.h, _p(r), r.shape[0], _p(ww), ii.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                       len(ii), float(scale))

    def advance(self):
        """One step; returns the index of the step made."""
        return self.L.orc3_advance(self.h)

    def scr(self):
        out = np.zeros((6, self.nz, self.ny, self.nx))
        self.L.orc3_get_scr(self.h, _p(out))
        return out

    def ddzkern(self, f):
        """d/dz with ibc 1, then FILTER_VAR_Z (kernels.f90:891-928) as the GPU kernel stage applies it."""
        return filter_var_z(self.ddz(f, 1))

    def kernel_record(self):
        """The kernel-stage record of the current state: div xi, v_x, v_y, v_z, |acc|^2."""
        a, sc = self.state(), self.scr()
        div = self.ddx(a[0]) + self.ddy(a[1]) + self.ddzkern(a[2])
        acc2 = sc[3] * sc[3] + sc[4] * sc[4] + sc[5] * sc[5]
        return np.stack([div, a[3], a[4], a[5], acc2])

    def kernels_accumulate(self, rec, out):
        """Add the integrands of forward record rec against this solve's current v (the adjoint) to
        out (5, nz, ny, nx): div xi_f div v_a, sum_j d_i(v_f,j) v_a,j for i = x, y, z, |acc_f|^2."""
        a = self.state()
        diva = self.ddx(a[3]) + self.ddy(a[4]) + self.ddzkern(a[5])
        out[0] += rec[0] * diva
        out[4] += rec[4]
        for j in range(3):
            vf, va = rec[1 + j], a[3 + j]
            out[1] += self.ddx(vf) * va
            out[2] += self.ddy(vf) * va
            out[3] += self.ddzkern(vf) * va

    def close(self):
        if self.h:
            self.L.orc3_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def filter_var_z(d):
    """FILTER_VAR_Z along axis 0 (kernels.f90:891-928): rows 1-4 and nz-5 .. nz-2 the average of
    their two neighbours, rows 5 .. nz-6 the 11-point filter, the end rows unchanged."""
    nz = d.shape[0]
    c0, h = 0.75390625, [0.5 * 0.41015625, 0.5 * -0.234375, 0.5 * 0.087890625, 0.5 * -0.01953125, 0.5 * 0.001953125]
    out = d.copy()
    for k in list(range(1, 5)) + list(range(nz - 5, nz - 1)):
        out[k] = 0.5 * (d[k + 1] + d[k - 1])
    for k in range(5, nz - 5):
        v = c0 * d[k]
        for j in range(1, 6):
            v = v + h[j - 1] * (d[k - j] + d[k + j])
        out[k] = v
    return out
