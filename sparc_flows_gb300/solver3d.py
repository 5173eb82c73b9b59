"""3-D wave solver (option 16, MP_FLOWS_PML_3D_DISPL) for a batch of sources: the Python host of
the sparc3d_* C ABI (csrc/sparc_3d.cu, csrc/sparc_capi.cu).

Set-up follows the reference's 3-D initialisation: grid and stretch factors
(initialize.f90:195-226, 466-474), solar_data (initialize.f90:731-794, laterally uniform),
mp_Initialize_RHS (physics.f90:34-404: e_rad / o_rad, source_dep, rhoinv, c2 rho0, d rho0/dz,
d p0/dz, the vertical PML of physics.f90:255-295).  Fields on the device are
[nz][nbatch][ny][nx]; the state is (6, nz, nbatch, ny, nx): xi_x, xi_y, xi_z, v_x, v_y, v_z.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import capi
from .config import DIMC, DIMRHO, RSUN_CM
from .solver import PI, _F32, nearest_level, rk_betas


def _dbyd2_host(b: np.ndarray, ibc: int) -> np.ndarray:
    """dbyd2 of a profile in FP64 on the host (the plan's partitioned algebra, dbyd2.f:8-235)."""
    L = capi.lib()
    b = np.ascontiguousarray(b, dtype=np.float64)
    x = np.zeros_like(b)
    dp = ctypes.POINTER(ctypes.c_double)
    capi.check(L.sparc_zsolve_host(len(b), ibc, 16, b.ctypes.data_as(dp), x.ctypes.data_as(dp), None, 1),
               "sparc_zsolve_host")
    return x


class WaveSolver3D:
    """nbatch 3-D solves sharing a background (and flow) on one GPU."""

    def __init__(self, nx: int, ny: int, model: np.ndarray, xlength_cm: float, ylength_cm: float | None = None,
                 nbatch: int = 1, precision: int = 32, timestep: float = 2.0, excitdep_cm: float = -150e5,
                 obsheight_cm: float = 200e5, npmlbot: int = 10, npmltop: int = 10, steps_out: int = 15,
                 flows: bool = False, filter_every: int = 2, device="cuda"):
        self.L = capi.lib()
        self.nx, self.ny, self.nz, self.nb = nx, ny, model.shape[0], nbatch
        self.precision = precision
        self.dtype = torch.float32 if precision == 32 else torch.float64
        self.dev = torch.device(device)
        self.flows = bool(flows)
        ylength_cm = xlength_cm if ylength_cm is None else ylength_cm
        nz = self.nz
        diml = RSUN_CM
        z = model[:, 0].astype(np.float64)
        c = model[:, 1] / DIMC
        rho0 = model[:, 2] / DIMRHO
        p0 = model[:, 3] / (DIMRHO * DIMC * DIMC)
        g = model[:, 4] * diml / (DIMC * DIMC)
        self.z = z
        self.deltat = timestep * DIMC / diml
        self.betas = rk_betas(self.deltat)
        self.e_rad = nearest_level(z, 1.0 + excitdep_cm / RSUN_CM)
        self.o_rad = nearest_level(z, 1.0 + obsheight_cm / RSUN_CM)
        unstretch = _dbyd2_host(z, 1)
        stretch = 1.0 / unstretch
        gr0 = _dbyd2_host(rho0, 1) * stretch
        gp0 = _dbyd2_host(p0, 1) * stretch
        dz = z - z[self.e_rad]
        source_dep = np.exp(-1e7 * 4.0 * (dz * dz))                       # physics.f90:109
        # vertical PML, physics.f90:255-295 (0.005 a single-precision literal)
        l005 = float(_F32(0.005))
        az = np.zeros(npmlbot + npmltop)
        bz = np.zeros(npmlbot + npmltop)
        gmod = g.copy()
        for k in range(nz):
            if k < npmlbot:
                alk = PI * l005 * diml / DIMC * (z[k] - z[0]) / (z[npmlbot - 1] - z[0])
                rr = (z[npmlbot - 1] - z[k]) / (z[npmlbot - 1] - z[0])
                dampz = 2.0 * 3.0 * 3.0 * c[0] / (z[npmlbot - 1] - z[0]) * (rr * rr)
                pi_ = k
            elif k > nz - npmltop - 1:
                alk = PI * l005 * diml / DIMC * (z[nz - 1] - z[k]) / (z[nz - 1] - z[nz - npmltop])
                rr = (z[nz - npmltop] - z[k]) / (z[nz - 1] - z[nz - npmltop])
                dampz = 3.0 * 3.0 * c[nz - 1] / (z[nz - 1] - z[nz - npmltop]) * (rr * rr)
                pi_ = npmlbot + (k - (nz - npmltop))
            else:
                continue
            fd = alk / (dampz + alk)
            gp0[k] *= fd
            gr0[k] *= fd
            gmod[k] *= fd
            az[pi_] = -dampz
            bz[pi_] = -alk - dampz
        self.profiles = dict(stretch=stretch, rhoinv=1.0 / rho0, rho0=rho0, c2rho0=c * c * rho0, gradp0_z=gp0,
                             gradrho0_z=gr0, g=gmod, source_dep=source_dep, az=az, bz=bz)

        cfg = capi.Sparc3DConfig()
        cfg.nx, cfg.ny, cfg.nz, cfg.nbatch, cfg.precision = nx, ny, nz, nbatch, precision
        cfg.npmlbot, cfg.npmltop = npmlbot, npmltop
        cfg.deltat = self.deltat
        cfg.stretchx, cfg.stretchy = RSUN_CM / xlength_cm, RSUN_CM / ylength_cm
        for i in range(5):
            cfg.betas[i] = self.betas[i]
        cfg.flows, cfg.steps_out = int(self.flows), steps_out
        cfg.k_src, cfg.k_obs, cfg.filter_every = self.e_rad, self.o_rad, filter_every
        self.cfg = cfg
        h = ctypes.c_void_p()
        capi.check(self.L.sparc3d_plan_create(ctypes.byref(cfg), ctypes.byref(h)), "sparc3d_plan_create")
        self.plan = h
        self._dev_bg = {k: torch.as_tensor(v, dtype=torch.float64, device=self.dev) for k, v in self.profiles.items()}
        self._v0 = None
        if not self.flows:
            self._upload()

    def _stream(self):
        return ctypes.c_void_p(torch.cuda.current_stream(self.dev).cuda_stream)

    def _upload(self):
        bg = capi.Sparc3DBackground()
        for k, t in self._dev_bg.items():
            setattr(bg, k, t.data_ptr())
        if self.flows:
            for k, t in zip(("v0x", "v0y", "v0z"), self._v0):
                setattr(bg, k, t.data_ptr())
        capi.check(self.L.sparc3d_set_background(self.plan, ctypes.byref(bg), self._stream()), "sparc3d_set_background")
        torch.cuda.current_stream(self.dev).synchronize()

    def set_flow(self, v0x, v0y, v0z):
        """Flow fields (nz, ny, nx), nondimensional (cm/s / dimc)."""
        self._v0 = [torch.as_tensor(np.ascontiguousarray(v), dtype=torch.float64, device=self.dev).contiguous()
                    for v in (v0x, v0y, v0z)]
        self._upload()

    def set_source(self, pattern, amp):
        """forcing(x, y, step) = pattern[b] * amp[step]: pattern (nb, ny, nx), amp (nsteps,)."""
        pat = torch.as_tensor(np.ascontiguousarray(pattern), dtype=torch.float64, device=self.dev).contiguous()
        am = np.ascontiguousarray(amp, dtype=np.float64)
        capi.check(self.L.sparc3d_set_source(self.plan, pat.data_ptr(), am.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                             len(am), self._stream()), "sparc3d_set_source")
        torch.cuda.current_stream(self.dev).synchronize()

    def reset(self, time0: int = 0):
        capi.check(self.L.sparc3d_reset_state(self.plan, time0, self._stream()), "sparc3d_reset_state")

    def forward(self, nsteps: int, max_records: int | None = None) -> torch.Tensor:
        """Run nsteps; returns the v_z records (nrec, nb, ny, nx) made during the call."""
        cap = (nsteps // max(self.cfg.steps_out, 1) + 1) if max_records is None else max_records
        seis = torch.zeros((max(cap, 1), self.nb, self.ny, self.nx), dtype=self.dtype, device=self.dev)
        n = ctypes.c_int(0)
        capi.check(self.L.sparc3d_forward(self.plan, nsteps, seis.data_ptr(), cap, ctypes.byref(n), self._stream()),
                   "sparc3d_forward")
        return seis[:min(n.value, cap)]

    @property
    def adjoint_scale(self) -> float:
        """delta_width / rho0(o_rad): the factor of the kernel-mode adjoint forcing
        (displacement.f90:615-627), delta_width = 2 / (z(o_rad+1) - z(o_rad-1))."""
        k = self.o_rad
        return 2.0 / (self.z[k + 1] - self.z[k - 1]) / self.profiles["rho0"][k]

    def set_adjoint_source(self, rows: torch.Tensor, wts: np.ndarray, idx: np.ndarray, scale: float | None = None):
        """Kernel-mode adjoint source: slices rows (nb, nrows, ny, nx) FP64 on the device at the
        record cadence, LAGRANGE_INTERP table (wts (ntab, 7), idx (ntab,)) per step."""
        self._adj_rows = rows.to(device=self.dev, dtype=torch.float64).contiguous()  # the plan keeps the pointer
        self._adj_w = np.ascontiguousarray(wts, dtype=np.float64)
        self._adj_i = np.ascontiguousarray(idx, dtype=np.int32)
        capi.check(self.L.sparc3d_set_adjoint_source(
            self.plan, self._adj_rows.data_ptr(), self._adj_rows.shape[1],
            self._adj_w.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
            self._adj_i.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), len(self._adj_i),
            self.adjoint_scale if scale is None else float(scale), self._stream()), "sparc3d_set_adjoint_source")

    def forward_records(self, nsteps: int, snaps: torch.Tensor | None, rec0: int = 0,
                        seis: torch.Tensor | None = None) -> int:
        """nsteps steps; kernel-stage records rec0 .. rec0 + len(snaps) - 1 to snaps
        (nslot, 5, nz, nb, ny, nx); v_z records of the call to seis if given.  Returns the number of
        v_z records the call made."""
        n = ctypes.c_int(0)
        cap = 0 if seis is None else seis.shape[0]
        capi.check(self.L.sparc3d_forward_records(
            self.plan, nsteps, 0 if seis is None else seis.data_ptr(), cap, ctypes.byref(n),
            0 if snaps is None else snaps.data_ptr(), rec0, 0 if snaps is None else snaps.shape[0], self._stream()),
            "sparc3d_forward_records")
        return n.value

    def record_buffer(self, nslot: int) -> torch.Tensor:
        return torch.zeros((nslot, 5, self.nz, self.nb, self.ny, self.nx), dtype=self.dtype, device=self.dev)

    def kernels_accumulate(self, snaps: torch.Tensor, slot: int, out: torch.Tensor):
        """Add the kernel integrands of forward record slot of snaps against the current state
        (the adjoint fields) to out (5, nz, nb, ny, nx) FP64."""
        capi.check(self.L.sparc3d_kernels_accumulate(self.plan, snaps.data_ptr(), slot, out.data_ptr(), self._stream()),
                   "sparc3d_kernels_accumulate")

    def checkpoint_bytes(self) -> int:
        return int(self.L.sparc3d_checkpoint_bytes(self.plan))

    def checkpoint_save(self, buf: torch.Tensor) -> int:
        t = ctypes.c_int(0)
        capi.check(self.L.sparc3d_checkpoint_save(self.plan, buf.data_ptr(), ctypes.byref(t), self._stream()),
                   "sparc3d_checkpoint_save")
        return t.value

    def checkpoint_load(self, buf: torch.Tensor, time: int):
        capi.check(self.L.sparc3d_checkpoint_load(self.plan, buf.data_ptr(), int(time), self._stream()),
                   "sparc3d_checkpoint_load")

    def state(self) -> torch.Tensor:
        st = torch.empty((6, self.nz, self.nb, self.ny, self.nx), dtype=self.dtype, device=self.dev)
        capi.check(self.L.sparc3d_get_state(self.plan, st.data_ptr(), self._stream()), "sparc3d_get_state")
        return st

    def set_state(self, st: torch.Tensor):
        st = st.to(self.dtype).contiguous()
        capi.check(self.L.sparc3d_set_state(self.plan, st.data_ptr(), self._stream()), "sparc3d_set_state")

    def point_steps(self, nsteps: int) -> int:
        return self.nx * self.ny * self.nz * self.nb * nsteps

    def close(self):
        if getattr(self, "plan", None):
            self.L.sparc3d_plan_destroy(self.plan)
            self.plan = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
