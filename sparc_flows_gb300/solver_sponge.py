"""2-D velocity-pressure-density solver: option 5 (MP_QUIET_SPONGE_2D, a sponge absorber,
physics2d.f90:1099-1137), option 6 (MP_QUIET_PML_2D, the vertical PML, physics2d.f90:662-713) or
option 12 (MP_MHD_PML_2d, the same with a background magnetic field, physics2d.f90:411-474);
the Python host of the sparc5_* C ABI (csrc/sparc_sponge.cu, csrc/sparc_capi.cu).

Set-up as the reference's mp_Initialize_RHS_2d (physics2d.f90:23-332): e_rad, o_rad,
source_dep, rhoinv, c2 rho0, the background gradients d rho0/dz, d p0/dz, and either the sponge
profile spongez (physics2d.f90:62-69; spongexyz = spongez for a periodic box) or, with USE_PML,
no sponge (physics2d.f90:289-290) and the vertical PML coefficients with their decay of the
background gradients and g (physics2d.f90:288-332).  State (5, nz, nbatch, nx): rho, v_x, v_y,
v_z, p; for option 12 (8, nz, nbatch, nx) with b_x, b_y, b_z.  Option 12 takes the background
field (box, boz), (nz, nx) in units of dimb = (4 pi dimc^2 dimrho)^(1/2) (initialize.f90:759);
the stratification stays laterally uniform, as a current-free field leaves it.
"""
from __future__ import annotations

import ctypes

import numpy as np
import torch

from . import capi
from .config import DIMC, DIMRHO, RSUN_CM
from .solver import PI, _F32, nearest_level, rk_betas
from .solver3d import _dbyd2_host


class WaveSolverSponge:
    def __init__(self, nx: int, model: np.ndarray, xlength_cm: float, nbatch: int = 1, precision: int = 64,
                 timestep: float = 2.0, excitdep_cm: float = -150e5, obsheight_cm: float = 200e5, npmlhor: int = 9,
                 steps_out: int = 15, filter_all_x: bool = False, option: int = 5, npmlbot: int = 10,
                 npmltop: int = 10, box=None, boz=None, device="cuda"):
        self.L = capi.lib()
        self.nx, self.nz, self.nb = nx, model.shape[0], nbatch
        self.dtype = torch.float32 if precision == 32 else torch.float64
        self.dev = torch.device(device)
        z = model[:, 0].astype(np.float64)
        c = model[:, 1] / DIMC
        rho0 = model[:, 2] / DIMRHO
        p0 = model[:, 3] / (DIMRHO * DIMC * DIMC)
        g = model[:, 4] * RSUN_CM / (DIMC * DIMC)
        self.deltat = timestep * DIMC / RSUN_CM
        betas = rk_betas(self.deltat)
        self.e_rad = nearest_level(z, 1.0 + excitdep_cm / RSUN_CM)
        self.o_rad = nearest_level(z, 1.0 + obsheight_cm / RSUN_CM)
        stretch = 1.0 / _dbyd2_host(z, 1)
        f = lambda v: float(_F32(v))  # noqa: E731  single-precision literals of physics2d.f90:65-66
        sponge = (200.0 / (1.0 + np.exp((f(1.002) - z) / f(0.0001)))
                  + 300.0 / (1.0 + np.exp((z - (z[0] + f(0.005))) / f(0.0005))))
        dz = z - z[self.e_rad]
        gp0 = _dbyd2_host(p0, 1) * stretch
        gr0 = _dbyd2_host(rho0, 1) * stretch
        nz = self.nz
        az = np.zeros(npmlbot + npmltop)
        bz = np.zeros(npmlbot + npmltop)
        if option in (6, 12):
            sponge = np.zeros(nz)
            l005 = f(0.005)
            for k in range(nz):
                if k < npmlbot:
                    alk = PI * l005 * RSUN_CM / DIMC * (z[k] - z[0]) / (z[npmlbot - 1] - z[0])
                    rr = (z[npmlbot - 1] - z[k]) / (z[npmlbot - 1] - z[0])
                    dampz = 3.0 * 3.0 * c[0] / (z[npmlbot - 1] - z[0]) * (rr * rr)
                    pi_ = k
                elif k > nz - npmltop - 1:
                    alk = PI * l005 * RSUN_CM / DIMC * (z[nz - 1] - z[k]) / (z[nz - 1] - z[nz - npmltop])
                    rr = (z[nz - npmltop] - z[k]) / (z[nz - 1] - z[nz - npmltop])
                    dampz = 3.0 * 3.0 * c[nz - 6] / (z[nz - 1] - z[nz - npmltop]) * (rr * rr)
                    pi_ = npmlbot + (k - (nz - npmltop))
                else:
                    continue
                fd = alk / (dampz + alk)
                gp0[k] *= fd
                gr0[k] *= fd
                g[k] *= fd
                az[pi_] = -dampz
                bz[pi_] = -alk - dampz
        self.profiles = dict(stretch=stretch, rhoinv=1.0 / rho0, rho0=rho0, c2rho0=c * c * rho0,
                             gradp0_z=gp0, gradrho0_z=gr0, g=g, source_dep=np.exp(-1e7 * 4.0 * (dz * dz)),
                             sponge=sponge, az=az, bz=bz)
        cfg = capi.Sparc5Config()
        cfg.nx, cfg.nz, cfg.nbatch, cfg.precision = nx, self.nz, nbatch, precision
        cfg.npmlhor, cfg.filter_all_x = npmlhor, int(filter_all_x)
        cfg.deltat, cfg.stretchx = self.deltat, RSUN_CM / xlength_cm
        for i in range(5):
            cfg.betas[i] = betas[i]
        cfg.steps_out, cfg.k_src, cfg.k_obs = steps_out, self.e_rad, self.o_rad
        cfg.option, cfg.npmlbot, cfg.npmltop = option, npmlbot, npmltop
        self.cfg = cfg
        h = ctypes.c_void_p()
        capi.check(self.L.sparc5_plan_create(ctypes.byref(cfg), ctypes.byref(h)), "sparc5_plan_create")
        self.plan = h
        self.nf = 8 if option == 12 else 5
        if option == 12:
            if box is None or boz is None:
                raise ValueError("option 12 needs the background field box, boz (nz, nx)")
            self.profiles["box"] = np.ascontiguousarray(box, dtype=np.float64).reshape(nz, nx)
            self.profiles["boz"] = np.ascontiguousarray(boz, dtype=np.float64).reshape(nz, nx)
        self._bg = {k: torch.as_tensor(v, dtype=torch.float64, device=self.dev) for k, v in self.profiles.items()}
        bg = capi.Sparc5Background()
        for k, t in self._bg.items():
            setattr(bg, k, t.data_ptr())
        capi.check(self.L.sparc5_set_background(self.plan, ctypes.byref(bg), self._stream()), "sparc5_set_background")
        torch.cuda.current_stream(self.dev).synchronize()

    def _stream(self):
        return ctypes.c_void_p(torch.cuda.current_stream(self.dev).cuda_stream)

    def set_source(self, pattern, amp):
        """forcing(x, step) = pattern[b] * amp[step]: pattern (nb, nx), amp (nsteps,)."""
        pat = torch.as_tensor(np.ascontiguousarray(pattern), dtype=torch.float64, device=self.dev).contiguous()
        am = np.ascontiguousarray(amp, dtype=np.float64)
        capi.check(self.L.sparc5_set_source(self.plan, pat.data_ptr(), am.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                            len(am), self._stream()), "sparc5_set_source")
        torch.cuda.current_stream(self.dev).synchronize()

    def reset(self, time0: int = 0):
        capi.check(self.L.sparc5_reset_state(self.plan, time0, self._stream()), "sparc5_reset_state")

    def forward(self, nsteps: int) -> torch.Tensor:
        """nsteps steps; v_z records (nrec, nb, nx) of the call."""
        cap = nsteps // max(self.cfg.steps_out, 1) + 1
        seis = torch.zeros((cap, self.nb, self.nx), dtype=self.dtype, device=self.dev)
        n = ctypes.c_int(0)
        capi.check(self.L.sparc5_forward(self.plan, nsteps, seis.data_ptr(), cap, ctypes.byref(n), self._stream()),
                   "sparc5_forward")
        return seis[:n.value]

    def state(self) -> torch.Tensor:
        st = torch.empty((self.nf, self.nz, self.nb, self.nx), dtype=self.dtype, device=self.dev)
        capi.check(self.L.sparc5_get_state(self.plan, st.data_ptr(), self._stream()), "sparc5_get_state")
        return st

    def close(self):
        if getattr(self, "plan", None):
            self.L.sparc5_plan_destroy(self.plan)
            self.plan = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
