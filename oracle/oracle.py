"""ctypes loader for the C FP64 oracle plus an independent NumPy restatement of single
operators.  TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and the
cpu_baseline / reference arm of bench.py; the product never imports it.

Parity against a run of the reference is unpinned (no Fortran/MPI/FFTW toolchain exists
here and the reference ships no tests); the restatement is pinned by known-answer tests
(analytic derivatives, polynomial exactness, numpy.fft) and by agreement between the C
code and the NumPy operators below.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libsparc_oracle.so")

_c_double_p = ctypes.POINTER(ctypes.c_double)


class OrcParams(ctypes.Structure):
    """Mirror of orc_params in sparc_oracle.c."""

    _fields_ = [
        ("nx", ctypes.c_int), ("nz", ctypes.c_int),
        ("npmlbot", ctypes.c_int), ("npmltop", ctypes.c_int), ("npmlhor", ctypes.c_int),
        ("xlength", ctypes.c_double), ("timestep", ctypes.c_double),
        ("excitdep", ctypes.c_double), ("obsheight", ctypes.c_double),
        ("flows", ctypes.c_int), ("adjoint", ctypes.c_int), ("steps_out", ctypes.c_int),
        ("src_until", ctypes.c_int), ("cadforcing", ctypes.c_double),
        ("filter_kst", ctypes.c_int), ("filter_all_x", ctypes.c_int),
    ]


def build(force=False):
    """Compile the oracle with its Makefile (gcc)."""
    if force or not os.path.exists(LIB_PATH) or any(
        os.path.getmtime(LIB_PATH) < os.path.getmtime(os.path.join(HERE, f))
        for f in ("sparc_oracle.c", "sparc_oracle3d.c", "sparc_oracle_sponge.c", "Makefile")
    ):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


_lib = None


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(LIB_PATH)
        L.orc_create.restype = ctypes.c_void_p
        L.orc_create.argtypes = [ctypes.POINTER(OrcParams), _c_double_p, _c_double_p]
        L.orc_destroy.argtypes = [ctypes.c_void_p]
        L.orc_set_psi.argtypes = [ctypes.c_void_p, _c_double_p]
        L.orc_set_flow.argtypes = [ctypes.c_void_p, _c_double_p, _c_double_p]
        L.orc_set_magnetic.argtypes = [ctypes.c_void_p, _c_double_p, _c_double_p]
        L.orc_set_forward_source.argtypes = [ctypes.c_void_p, ctypes.c_double, ctypes.c_int,
                                             ctypes.c_double, ctypes.c_int, ctypes.c_double, ctypes.c_int]
        L.orc_set_adjoint_source.argtypes = [ctypes.c_void_p, _c_double_p, ctypes.c_int, ctypes.c_int]
        L.orc_step.argtypes = [ctypes.c_void_p]
        L.orc_apply_filter.argtypes = [ctypes.c_void_p]
        L.orc_run.argtypes = [ctypes.c_void_p, ctypes.c_int, _c_double_p, _c_double_p]
        L.orc_run.restype = ctypes.c_int
        L.orc_get_int.argtypes = [ctypes.c_void_p, ctypes.c_char_p]
        L.orc_get_double.argtypes = [ctypes.c_void_p, ctypes.c_char_p]
        L.orc_get_double.restype = ctypes.c_double
        L.orc_get_array.argtypes = [ctypes.c_void_p, ctypes.c_char_p, _c_double_p]
        L.orc_get_array.restype = ctypes.c_long
        L.orc_set_array.argtypes = [ctypes.c_void_p, ctypes.c_char_p, _c_double_p]
        L.orc_dbyd2.argtypes = [_c_double_p, _c_double_p, ctypes.c_int, ctypes.c_int, ctypes.c_int]
        L.orc_fft_c2c.argtypes = [ctypes.c_int, _c_double_p, _c_double_p, ctypes.c_int]
        L.orc_sim_ddx.argtypes = [ctypes.c_void_p, _c_double_p, _c_double_p]
        L.orc_sim_ddz.argtypes = [ctypes.c_void_p, _c_double_p, _c_double_p, ctypes.c_int]
        L.orc_kernels.argtypes = [ctypes.c_void_p, _c_double_p, ctypes.c_int, _c_double_p, ctypes.c_int,
                                  ctypes.c_int] + [_c_double_p] * 5
        L.orc_run_batch.argtypes = [ctypes.POINTER(OrcParams), _c_double_p, ctypes.c_int, _c_double_p,
                                    _c_double_p, ctypes.c_int, ctypes.c_int, _c_double_p]
        _lib = L
    return _lib


def _p(a):
    return a.ctypes.data_as(_c_double_p) if a is not None else None


def params_from(run):
    """Build OrcParams from a sparc_flows_gb300.config.RunConfig-like object."""
    return OrcParams(run.nx, run.nz, run.npmlbot, run.npmltop, run.npmlhor, run.xlength_cm,
                     run.timestep, run.excitdep_cm, run.obsheight_cm, int(run.flows),
                     int(run.adjoint), run.steps_out, run.src_until, run.cadforcing,
                     getattr(run, "filter_kst", 6), int(getattr(run, "filter_all_x", False)))


class OracleSim:
    """One FP64 CPU solve (forward or reference-style adjoint)."""

    def __init__(self, run, model, cmul=None):
        self.L = lib()
        self.run = run
        self.nx, self.nz = run.nx, run.nz
        self._model = np.ascontiguousarray(model, dtype=np.float64)
        self._cmul = None if cmul is None else np.ascontiguousarray(cmul, dtype=np.float64)
        prm = params_from(run)
        self.h = self.L.orc_create(ctypes.byref(prm), _p(self._model), _p(self._cmul))
        if not self.h:
            raise RuntimeError("orc_create failed (unsupported nx?)")

    def close(self):
        if self.h:
            self.L.orc_destroy(self.h)
            self.h = None

    def __del__(self):
        self.close()

    def set_psi(self, psi):
        psi = np.ascontiguousarray(psi, dtype=np.float64)
        self.L.orc_set_psi(self.h, _p(psi))

    def set_flow(self, v0x, v0z):
        a = np.ascontiguousarray(v0x, dtype=np.float64)
        b = np.ascontiguousarray(v0z, dtype=np.float64)
        self.L.orc_set_flow(self.h, _p(a), _p(b))

    def set_magnetic(self, box, boz):
        """Option 18 (MP_MHD_PML_2D_DISPL): background field (nz, nx) in units of dimb; the run must
        have no flow."""
        a = np.ascontiguousarray(box, dtype=np.float64)
        b = np.ascontiguousarray(boz, dtype=np.float64)
        if self.L.orc_set_magnetic(self.h, _p(a), _p(b)) != 0:
            raise ValueError("orc_set_magnetic: the run has flows")

    def set_forward_source(self, xloc, spatial_kind=0, sigma=0.5, temporal_kind=0, nu0=0.003, nt=None):
        nt = nt if nt is not None else self.run.nsteps + 8
        self.L.orc_set_forward_source(self.h, xloc, spatial_kind, sigma, temporal_kind, nu0, nt)

    def set_adjoint_source(self, src, num_steps):
        src = np.ascontiguousarray(src, dtype=np.float64)
        self.L.orc_set_adjoint_source(self.h, _p(src), src.shape[0], num_steps)

    def step(self):
        self.L.orc_step(self.h)

    def apply_filter(self):
        self.L.orc_apply_filter(self.h)

    def run_steps(self, nsteps, snapshots=False):
        nrec_max = nsteps // self.run.steps_out + 2
        seis = np.zeros((nrec_max, self.nx))
        snaps = np.zeros((nrec_max, 6, self.nz, self.nx)) if snapshots else None
        nrec = self.L.orc_run(self.h, nsteps, _p(seis), _p(snaps))
        if snapshots:
            return seis[:nrec], snaps[:nrec]
        return seis[:nrec]

    def get(self, name):
        n = self.L.orc_get_array(self.h, name.encode(), None)
        if n < 0:
            raise KeyError(name)
        out = np.zeros(n)
        self.L.orc_get_array(self.h, name.encode(), _p(out))
        return out

    def set_state(self, a6):
        a6 = np.ascontiguousarray(a6, dtype=np.float64)
        self.L.orc_set_array(self.h, b"a", _p(a6))

    def set_time(self, t):
        v = np.array([float(t)])
        self.L.orc_set_array(self.h, b"time", _p(v))

    def geti(self, name):
        return self.L.orc_get_int(self.h, name.encode())

    def getd(self, name):
        return self.L.orc_get_double(self.h, name.encode())

    def ddx(self, f):
        f = np.ascontiguousarray(f, dtype=np.float64)
        out = np.zeros_like(f)
        self.L.orc_sim_ddx(self.h, _p(f), _p(out))
        return out

    def ddz(self, f, bc, preset=None):
        f = np.ascontiguousarray(f, dtype=np.float64)
        out = np.zeros_like(f) if preset is None else np.ascontiguousarray(preset, dtype=np.float64).copy()
        self.L.orc_sim_ddz(self.h, _p(f), _p(out), bc)
        return out

    def kernels(self, fsnaps, asnaps, nt_kern=None):
        fs = np.ascontiguousarray(fsnaps, dtype=np.float64)
        as_ = np.ascontiguousarray(asnaps, dtype=np.float64)
        nt_kern = nt_kern if nt_kern is not None else min(fs.shape[0], as_.shape[0])
        outs = [np.zeros((self.nz, self.nx)) for _ in range(5)]
        self.L.orc_kernels(self.h, _p(fs), fs.shape[0], _p(as_), as_.shape[0], nt_kern, *[_p(o) for o in outs])
        return dict(zip(["kernel_c", "kernel_vx", "kernel_vz", "kernel_psi", "hessian"], outs))


def dbyd2(B, ibc, preset=None):
    """C oracle compact derivative along axis 0 of B (n2, n1) (dbyd2.f layout: 2nd index)."""
    B = np.ascontiguousarray(B, dtype=np.float64)
    n2 = B.shape[0]
    n1 = int(np.prod(B.shape[1:])) if B.ndim > 1 else 1
    A = np.zeros_like(B) if preset is None else np.ascontiguousarray(preset, dtype=np.float64).copy()
    rc = lib().orc_dbyd2(_p(A), _p(B), n1, n2, ibc)
    if rc:
        raise ValueError("ibc out of range")
    return A


def fft(re, im, sign=-1):
    re = np.ascontiguousarray(re, dtype=np.float64).copy()
    im = np.ascontiguousarray(im, dtype=np.float64).copy()
    lib().orc_fft_c2c(len(re), _p(re), _p(im), sign)
    return re + 1j * im


def run_batch(run, model, xlocs, psi, nsteps, nthreads):
    """Run len(xlocs) independent forward solves on nthreads host threads."""
    prm = params_from(run)
    model = np.ascontiguousarray(model, dtype=np.float64)
    xl = np.ascontiguousarray(xlocs, dtype=np.float64)
    psi = None if psi is None else np.ascontiguousarray(psi, dtype=np.float64)
    nrec = (nsteps - 1) // run.steps_out + 1
    seis = np.zeros((len(xl), nrec, run.nx))
    lib().orc_run_batch(ctypes.byref(prm), _p(model), len(xl), _p(xl), _p(psi), nsteps, nthreads, _p(seis))
    return seis


# --------------------------------------------------------------------------------------
# Independent NumPy restatement of single operators (used to cross-check the C code).
# --------------------------------------------------------------------------------------
def np_dbyd2(B, ibc, preset=None):
    """dbyd2.f:8-235 + mtridag.f:96-112, vectorised over the first index (axis 1 here)."""
    f32 = np.float32
    B = np.asarray(B, dtype=np.float64)
    n2 = B.shape[0]
    A = np.zeros_like(B) if preset is None else np.array(preset, dtype=np.float64)
    d2i = f32(n2 - 1)
    C1 = f32(d2i * f32(7.0)) / f32(9.0)
    C2 = d2i / f32(36.0)
    A[2:n2 - 2] = np.float64(C1) * (B[3:n2 - 1] - B[1:n2 - 3]) + np.float64(C2) * (B[4:n2] - B[0:n2 - 4])
    C1 = -(f32(f32(43.0) / f32(96.0)) * d2i)
    C2 = -(f32(f32(5.0) / f32(6.0)) * d2i)
    C3 = f32(f32(9.0) / f32(8.0)) * d2i
    C4 = f32(f32(1.0) / f32(6.0)) * d2i
    C5 = -(f32(f32(1.0) / f32(96.0)) * d2i)
    c = [np.float64(v) for v in (C1, C2, C3, C4, C5)]
    A[1] = c[0] * B[0] + c[1] * B[1] + c[2] * B[2] + c[3] * B[3] + c[4] * B[4]
    A[n2 - 2] = -(c[0] * B[n2 - 1] + c[1] * B[n2 - 2] + c[2] * B[n2 - 3] + c[3] * B[n2 - 4] + c[4] * B[n2 - 5])
    C1 = -(f32(f32(10.0) / f32(3.0)) * d2i)
    C2 = -(f32(3.0) * d2i)
    C3 = f32(6.0) * d2i
    C4 = f32(f32(1.0) / f32(3.0)) * d2i
    c = [np.float64(v) for v in (C1, C2, C3, C4)]
    if ibc == 0:
        A[0] = 0.0
        A[n2 - 1] = 0.0
    if ibc in (1, 3):
        A[0] = c[0] * B[0] + c[1] * B[1] + c[2] * B[2] + c[3] * B[3]
    if ibc in (1, 2):
        A[n2 - 1] = -(c[0] * B[n2 - 1] + c[1] * B[n2 - 2] + c[2] * B[n2 - 3] + c[3] * B[n2 - 4])
    alpha = np.float64(f32(1.0) / f32(3.0))
    alpha2, gamma2, beta1 = f32(0.75), f32(0.125), f32(3.0)
    cnst = f32(1.0) / (alpha2 - beta1 * gamma2)
    up1 = (f32(6.0) * alpha2 - beta1) * cnst
    if ibc % 2:
        A[0] = (np.float64(alpha2) * A[0] - np.float64(beta1) * A[1]) * np.float64(cnst)
    if ibc in (1, 2):
        A[n2 - 1] = (np.float64(alpha2) * A[n2 - 1] - np.float64(beta1) * A[n2 - 2]) * np.float64(cnst)
    uppr = np.zeros(n2)
    uppr[2:n2 - 2] = alpha
    uppr[0] = 0.0 if ibc % 2 == 0 else np.float64(up1)
    uppr[1] = np.float64(alpha2)
    uppr[n2 - 2] = np.float64(gamma2)
    lowr = uppr[::-1].copy()
    lowr[n2 - 1] = np.float64(up1) if ibc in (1, 2) else 0.0
    gam = np.zeros(n2)
    bet = np.ones(n2)
    for j in range(1, n2):
        gam[j] = uppr[j - 1] / bet[j - 1]
        bet[j] = 1.0 - lowr[j] * gam[j]
    ud = np.zeros_like(A)
    ud[0] = A[0] / bet[0]
    for j in range(1, n2):
        ud[j] = (A[j] - lowr[j] * ud[j - 1]) / bet[j]
    for j in range(n2 - 2, -1, -1):
        ud[j] = ud[j] - gam[j + 1] * ud[j + 1]
    return ud


def np_ddx(f, stretchx):
    """derivatives.f90:28-58 with numpy's r2c/c2r in place of FFTW."""
    nx = f.shape[-1]
    F = np.fft.rfft(f, axis=-1)
    kap = np.arange(nx // 2 + 1) * (1.0 / nx) * 2.0 * np.pi
    F = F * (1j * kap)
    if nx % 2 == 0:
        F[..., -1] = 0.0
    # FFTW's c2r is unnormalised (the 1/nx sits in eyekx); numpy's irfft divides by nx
    return np.fft.irfft(F, n=nx, axis=-1) * nx * stretchx


FILTER_COEFFS = np.array([0.75390625, 0.41015625, -0.234375, 0.087890625, -0.01953125, 0.001953125])


def np_filter_z(a):
    """11-point z filter body of physics2d.f90:509-556 / kernels.f90:891-928 for k=6..nz-5."""
    c = FILTER_COEFFS
    nz = a.shape[0]
    t = np.array(a, copy=True)
    for k in range(5, nz - 5):
        t[k] = (c[0] * a[k] + 0.5 * c[1] * (a[k - 1] + a[k + 1]) + 0.5 * c[2] * (a[k - 2] + a[k + 2])
                + 0.5 * c[3] * (a[k - 3] + a[k + 3]) + 0.5 * c[4] * (a[k - 4] + a[k + 4])
                + 0.5 * c[5] * (a[k - 5] + a[k + 5]))
    return t
