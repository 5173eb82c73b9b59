"""Host side of the GB300 wave solver: the set-up of mp_Initialize_RHS_2d and the run control of
TIMESTEPPING, driving the CUDA library through its C ABI.

``WaveSolver`` mirrors what one reference ``sparc`` process holds (initialize.f90:26-159), for
a batch of independent solves sharing a grid: background, PML coefficients, flows, sources,
and the state advanced by ``run``.  Pointwise set-up formulas are evaluated here in FP64 NumPy;
every derivative (stretch factors, background gradients, flows from the stream function) is
taken on the GPU by the library's FP64 derivative kernels, as the reference takes them with
its own ddz/ddx (initialize.f90:466-470, physics2d.f90:229-230, driver.f90:105-115).
"""
from __future__ import annotations

import ctypes
import math
import os

import numpy as np
import torch

from . import capi
from .config import DIMC, DIMRHO, RSUN_CM, RunConfig
from .model import SourceSpec, lagrange_weights, source_profile, source_time_series

PI = 3.141592653589793
_F32 = np.float32
# optimals of INITIALIZE_STEP (step.f90:28-32); entries 3..5 are single-precision literals
OPTIMALS = (1.0, 0.5, float(_F32(0.1665579725791151184)), float(_F32(0.03950410250586729987)),
            float(_F32(0.007810706393337838236)))


def rk_betas(deltat: float):
    """betas of INITIALIZE_STEP (step.f90:34-40), times deltat; betas[0] = 0."""
    b = [0.0] * 5
    b[4] = OPTIMALS[1]
    b[3] = OPTIMALS[2] / b[4]
    b[2] = OPTIMALS[3] / (b[4] * b[3])
    b[1] = OPTIMALS[4] / (b[4] * b[3] * b[2])
    return [v * deltat for v in b]


def nearest_level(z: np.ndarray, target: float) -> int:
    """Last k with |z(k) - target| <= the running minimum (physics2d.f90:35-50)."""
    best, idx = 1.0, 0
    for k, zk in enumerate(z):
        if abs(zk - target) <= best:
            best = abs(zk - target)
            idx = k
    return idx


def _ptr(t: torch.Tensor | None):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


class WaveSolver:
    """A batch of 2-D displacement-formulation solves (option 17, physics2d.f90:943-1094).

    run:        grid/timing parameters (``RunConfig``); run.adjoint selects the injection row
                (o_rad) and the reference's time-reversed adjoint convention.
    model:      (nz, 6) background table in the reference model format.
    nbatch:     number of solves (sources / line-search variants) advanced together.
    precision:  64 (FP64 state and arithmetic) or 32.
    cmul:       optional (nz, nx) multiplier on c (sound-speed perturbation), or a list of nbatch.
    psi:        optional (nz, nx) stream function in Mm (driver.f90:94-147), or a list of nbatch.
    """

    def __init__(self, run: RunConfig, model: np.ndarray, nbatch: int = 1, precision: int = 64, cmul=None,
                 psi=None, device: str = "cuda:0", column_impl: int | None = None, column_block: int | None = None):
        if not torch.cuda.is_available():
            raise capi.SparcError("WaveSolver needs a CUDA device")
        self.run, self.nb, self.precision = run, nbatch, precision
        self._column = (column_impl, column_block)
        self.dev = torch.device(device)
        self.dtype = torch.float32 if precision == 32 else torch.float64
        nx, nz = run.nx, run.nz
        self.L = capi.lib()
        per_solve = isinstance(cmul, (list, tuple)) or isinstance(psi, (list, tuple))
        self.nbg = nbatch if per_solve else 1
        cm = self._per_solve(cmul, np.ones((nz, nx)))
        ps = self._per_solve(psi, None)
        self.flows = bool(run.flows)
        c2d = cmul is not None
        with torch.cuda.device(self.dev):
            self._setup(model, cm, ps, c2d, per_solve)

    # ------------------------------------------------------------------------------------------
    def _per_solve(self, v, default):
        if isinstance(v, (list, tuple)):
            return [None if a is None else np.asarray(a, dtype=np.float64) for a in v]
        return [default if v is None else np.asarray(v, dtype=np.float64)] * self.nbg

    def _t(self, a, dtype=torch.float64):
        return torch.as_tensor(np.ascontiguousarray(a), dtype=dtype, device=self.dev)

    def _setup(self, model, cmuls, psis, c2d, per_solve):
        run, nx, nz, nb = self.run, self.run.nx, self.run.nz, self.nb
        nh, nzpml = run.npmlhor, run.npmlbot + run.npmltop
        diml = RSUN_CM
        # solar_data (initialize.f90:731-794)
        z = model[:, 0].astype(np.float64)
        rho0 = model[:, 2] / DIMRHO
        p0 = model[:, 3] / (DIMRHO * DIMC * DIMC)
        g = model[:, 4] * diml / (DIMC * DIMC)
        c_speed = [(model[:, 1] / DIMC)[:, None] * cm for cm in cmuls]          # (nz, nx) each
        c2 = [c * c for c in c_speed]
        self.deltat = run.timestep * DIMC / diml                                # initialize.f90:474
        self.stretchx = RSUN_CM / run.xlength_cm                                # initialize.f90:225
        self.betas = rk_betas(self.deltat)
        self.e_rad = nearest_level(z, 1.0 + run.excitdep_cm / RSUN_CM)
        self.o_rad = nearest_level(z, 1.0 + run.obsheight_cm / RSUN_CM)
        k_inj = self.o_rad if run.adjoint else self.e_rad
        self.k_inj = k_inj
        self.delta_width = 2.0 / (z[k_inj + 1] - z[k_inj - 1])

        cfg = capi.SparcConfig()
        cfg.nx, cfg.nz, cfg.nbatch, cfg.precision = nx, nz, nb, self.precision
        cfg.npmlbot, cfg.npmltop, cfg.npmlhor = run.npmlbot, run.npmltop, nh
        cfg.deltat, cfg.stretchx = self.deltat, self.stretchx
        for i in range(5):
            cfg.betas[i] = self.betas[i]
        cfg.flows, cfg.c2d, cfg.bg_per_solve = int(self.flows), int(c2d), int(per_solve)
        cfg.steps_out, cfg.k_inj, cfg.k_obs, cfg.src_until = run.steps_out, k_inj, self.o_rad, run.src_until
        cfg.filter_k0, cfg.filter_all_x = run.filter_kst - 1, int(run.filter_all_x)
        cfg.compensated = int(os.environ.get("SPARC_COMPENSATED", "0"))
        impl, block = self._column
        cfg.column_impl = int(os.environ.get("SPARC_COLUMN_IMPL", "2")) if impl is None else int(impl)
        cfg.column_block = int(os.environ.get("SPARC_COLUMN_BLOCK", "0")) if block is None else int(block)
        self.cfg = cfg
        h = ctypes.c_void_p()
        capi.check(self.L.sparc_plan_create(ctypes.byref(cfg), ctypes.byref(h)), "sparc_plan_create")
        self.plan = h

        # stretch factors: unstretch = dbyd2(z, ibc=1) (initialize.f90:466-470)
        zt = self._t(z)
        unstr = torch.empty_like(zt)
        self.ddz(zt, unstr, n1=1, ibc=1, stretch=None)
        stretch = 1.0 / unstr
        self.stretch_t, self.unstretch_t = stretch, unstr
        # background gradients (physics2d.f90:226-230)
        rho0_t, p0_t = self._t(rho0), self._t(p0)
        gr0 = torch.empty_like(rho0_t)
        gp0 = torch.empty_like(p0_t)
        self.ddz(rho0_t, gr0, n1=1, ibc=1, stretch=stretch)
        self.ddz(p0_t, gp0, n1=1, ibc=1, stretch=stretch)
        gr0_np, gp0_np = gr0.cpu().numpy(), gp0.cpu().numpy()

        # vertical PML (physics2d.f90:288-332); 0.005 is a single-precision literal
        l005 = float(_F32(0.005))
        nbt, ntp = run.npmlbot, run.npmltop
        fdz = np.ones((self.nbg, nzpml, nx))
        az = np.zeros((self.nbg, nzpml, nx))
        bz = np.zeros((self.nbg, nzpml, nx))
        gmod = g.copy()
        ax = np.zeros((self.nbg, nz, 2 * nh))
        bx = np.zeros((self.nbg, nz, 2 * nh))
        x = np.arange(nx, dtype=np.float64) / nx
        for bi in range(self.nbg):
            tempin = np.sqrt(c2[bi])
            for k in range(nz):
                if k < nbt:
                    pi_ = k
                    alk = PI * l005 * diml / DIMC * (z[k] - z[0]) / (z[nbt - 1] - z[0])
                    rr = (z[nbt - 1] - z[k]) / (z[nbt - 1] - z[0])
                    dampz = 3.0 * 3.0 * tempin[0] / (z[nbt - 1] - z[0]) * (rr * rr)
                elif k > nz - ntp - 1:
                    pi_ = nbt + (k - (nz - ntp))
                    alk = PI * l005 * diml / DIMC * (z[nz - 1] - z[k]) / (z[nz - 1] - z[nz - ntp])
                    rr = (z[nz - ntp] - z[k]) / (z[nz - 1] - z[nz - ntp])
                    dampz = 3.0 * 3.0 * tempin[nz - 6] / (z[nz - 1] - z[nz - ntp]) * (rr * rr)
                else:
                    continue
                fd = alk / (dampz + alk)
                fdz[bi, pi_] = fd
                az[bi, pi_] = -dampz
                bz[bi, pi_] = -alk - dampz
                if bi == 0:
                    gmod[k] = g[k] * fd[0]
            # horizontal PML (physics2d.f90:335-357)
            c1 = np.sqrt(c2[bi][:, 0])
            for i in range(nh):
                rr = (x[i] - x[nh - 1]) / (x[nh - 1] - x[0])
                a_ = -0.25 * 3.0 * 3.0 * c1 / (x[nh - 1] - x[0]) * (rr * rr)
                ax[bi, :, i] = a_
                bx[bi, :, i] = a_ - l005 * diml / DIMC * PI * (x[i] - x[0]) / (x[nh - 1] - x[0])
            for cnt, i in enumerate(range(nx - nh, nx)):
                rr = (x[nx - nh] - x[i]) / (x[nx - nh] - x[nx - 1])
                a_ = -0.25 * 3.0 * 3.0 * c1 / (x[nx - 1] - x[nx - nh]) * (rr * rr)
                ax[bi, :, nh + cnt] = a_
                bx[bi, :, nh + cnt] = a_ - l005 * diml / DIMC * PI * (x[nx - 1] - x[i]) / (x[nx - 1] - x[nx - nh])

        rhoinv = 1.0 / rho0
        if c2d:
            c2rho0 = np.stack([c * rho0[:, None] for c in c2])
        else:
            c2rho0 = c2[0][:, 0] * rho0
        self.rho0 = rho0
        self.c2 = c2
        self.z = z
        # flows from the stream function (driver.f90:94-115)
        v0x = v0z = None
        if self.flows:
            v0x = torch.zeros((self.nbg, nz, nx), dtype=torch.float64, device=self.dev)
            v0z = torch.zeros_like(v0x)
            for bi in range(self.nbg):
                if psis[bi] is None:
                    continue
                pv = self._t(rho0[:, None] * np.sqrt(c2[bi]) * (psis[bi] / (diml / 1.0e8)))
                self.ddz(pv, v0x[bi], n1=nx, ibc=1, stretch=stretch)
                self.ddx(pv, v0z[bi], nrows=nz, stretchx=self.stretchx)
            r0 = self._t(rho0)[None, :, None]
            v0x = -v0x / r0
            v0z = v0z / r0
        self.v0x, self.v0z = v0x, v0z
        self.bg = dict(stretch=stretch, unstretch=unstr, rhoinv=self._t(rhoinv), rho0=rho0_t,
                       gradp0_z=gp0, gradrho0_z=gr0, g=self._t(gmod), fdz=self._t(fdz), az=self._t(az),
                       bz=self._t(bz), ax=self._t(ax), bx=self._t(bx), c2rho0=self._t(c2rho0),
                       v0x=v0x, v0z=v0z)
        self.gradp0_z, self.gradrho0_z, self.g = gp0_np, gr0_np, gmod
        bgs = capi.SparcBackground()
        for name, t in self.bg.items():
            setattr(bgs, name, t.data_ptr() if t is not None else None)
        capi.check(self.L.sparc_set_background(self.plan, ctypes.byref(bgs), _stream()), "sparc_set_background")
        torch.cuda.synchronize(self.dev)

    # ------------------------------------------------------------------------------------------
    def ddz(self, var: torch.Tensor, dvar: torch.Tensor, n1: int, ibc: int, stretch=None, preset=None):
        """FP64 compact z-derivative of n1 columns (ddz, derivatives.f90:10-24)."""
        capi.check(self.L.sparc_ddz(self.plan, _ptr(var), _ptr(dvar), n1, ibc, _ptr(preset), _ptr(stretch),
                                    _stream()), "sparc_ddz")

    def ddzkern(self, var: torch.Tensor, dvar: torch.Tensor, n1: int, ibc: int, stretch=None):
        """FP64 kernel-stage z-derivative with FILTER_VAR_Z (ddzkern, kernels.f90:648-661)."""
        capi.check(self.L.sparc_ddzkern(self.plan, _ptr(var), _ptr(dvar), n1, ibc, _ptr(stretch), _stream()),
                   "sparc_ddzkern")

    def ddx(self, var: torch.Tensor, dvar: torch.Tensor, nrows: int, stretchx: float):
        """FP64 spectral x-derivative of nrows rows (ddx, derivatives.f90:28-58)."""
        capi.check(self.L.sparc_ddx(self.plan, _ptr(var), _ptr(dvar), nrows, stretchx, _stream()), "sparc_ddx")

    # ------------------------------------------------------------------------------------------
    def set_forward_sources(self, specs: list[SourceSpec], ntab: int | None = None):
        """Forward sources (DETERMINE_STATUS / FORWARD_SOURCE, driver.f90:536-553, 1120-1145)."""
        if len(specs) != self.nb:
            raise ValueError("one SourceSpec per solve")
        run = self.run
        ntab = ntab if ntab is not None else run.nsteps + 8
        rows = np.stack([source_profile(run, s) for s in specs])[:, None, :]
        ts = source_time_series(run, specs[0], ntab)
        for s in specs[1:]:
            if (s.temporal, s.nu0) != (specs[0].temporal, specs[0].nu0):
                raise ValueError("all sources of a batch share one time function")
        wts = np.zeros((ntab, 7))
        wts[:, 0] = ts
        idx = np.zeros(ntab, dtype=np.int32)
        self._set_source(rows, wts, idx)
        self.src_rows, self.src_wts = rows, wts

    def set_adjoint_sources(self, src: np.ndarray, ntab: int | None = None):
        """Adjoint sources: (nbatch, forcing_length, nx) at cadforcing cadence (driver.f90:584-594),
        interpolated in time by LAGRANGE_INTERP (physics.f90:678-737)."""
        src = np.asarray(src, dtype=np.float64)
        if src.ndim != 3 or src.shape[0] != self.nb or src.shape[2] != self.run.nx:
            raise ValueError("adjoint source must be (nbatch, nt, nx)")
        ntab = ntab if ntab is not None else self.run.nsteps
        idx, w = lagrange_weights(self.run, ntab, self.run.num_steps, src.shape[1])
        self._set_source(src, w, idx)

    def set_adjoint_sources_device(self, src: torch.Tensor):
        """As set_adjoint_sources, with the slices already on the device (FP64)."""
        if src.dim() != 3 or src.shape[0] != self.nb or src.shape[2] != self.run.nx:
            raise ValueError("adjoint source must be (nbatch, nt, nx)")
        if getattr(self, "_lagr", None) is None or self._lagr[0] != src.shape[1]:
            idx, w = lagrange_weights(self.run, self.run.nsteps, self.run.num_steps, src.shape[1])
            self._lagr = (src.shape[1], idx, w)
        _, idx, w = self._lagr
        self._set_source(src, w, idx)

    def _set_source(self, rows, wts, idx):
        inj = np.broadcast_to(self.delta_width / self.rho0[self.k_inj], (self.nb, self.run.nx))
        inj_t = self._t(inj)
        rows_t = rows.to(torch.float64).contiguous() if isinstance(rows, torch.Tensor) else self._t(rows)
        w = np.ascontiguousarray(wts, dtype=np.float64)
        ix = np.ascontiguousarray(idx, dtype=np.int32)
        capi.check(self.L.sparc_set_source(self.plan, _ptr(inj_t), _ptr(rows_t), rows.shape[1],
                                           w.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                           ix.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), len(ix), _stream()),
                   "sparc_set_source")
        torch.cuda.current_stream(self.dev).synchronize()  # host tables outlive the copies

    def update_flow(self, psi: torch.Tensor):
        """New stream function (nz, nx) in Mm, a device tensor: recompute v0 on the GPU
        (driver.f90:94-115) and upload it; the rest of the background is kept."""
        run, nx, nz = self.run, self.run.nx, self.run.nz
        if not self.flows or self.nbg != 1:
            raise ValueError("update_flow needs a flow-enabled solver with one shared background")
        psi = psi.to(device=self.dev, dtype=torch.float64).reshape(nz, nx)
        r0 = self.bg["rho0"][:, None]
        c = torch.sqrt(torch.as_tensor(self.c2[0], device=self.dev))
        pv = (r0 * c * (psi / (RSUN_CM / 1.0e8))).contiguous()
        v0x = torch.empty((1, nz, nx), dtype=torch.float64, device=self.dev)
        v0z = torch.empty_like(v0x)
        self.ddz(pv, v0x[0], n1=nx, ibc=1, stretch=self.stretch_t)
        self.ddx(pv, v0z[0], nrows=nz, stretchx=self.stretchx)
        self.bg["v0x"] = (-v0x / r0[None]).contiguous()
        self.bg["v0z"] = (v0z / r0[None]).contiguous()
        self.v0x, self.v0z = self.bg["v0x"], self.bg["v0z"]
        self._upload_background()

    def set_flow_direct(self, v0x, v0z):
        """Flow given directly (nondimensional, (nz, nx)), as the data run reads true_vx/true_vz
        (driver.f90:63-76)."""
        if not self.flows or self.nbg != 1:
            raise ValueError("set_flow_direct needs a flow-enabled solver with one shared background")
        nz, nx = self.run.nz, self.run.nx
        self.bg["v0x"] = torch.as_tensor(v0x, dtype=torch.float64, device=self.dev).reshape(1, nz, nx).contiguous()
        self.bg["v0z"] = torch.as_tensor(v0z, dtype=torch.float64, device=self.dev).reshape(1, nz, nx).contiguous()
        self.v0x, self.v0z = self.bg["v0x"], self.bg["v0z"]
        self._upload_background()

    def _upload_background(self):
        bgs = capi.SparcBackground()
        for name, t in self.bg.items():
            setattr(bgs, name, t.data_ptr() if t is not None else None)
        capi.check(self.L.sparc_set_background(self.plan, ctypes.byref(bgs), _stream()), "sparc_set_background")

    def kernels_accumulate(self, fsnaps: torch.Tensor, jf: int, out: torch.Tensor):
        """Accumulate the kernel integrand of forward record jf against this solver's current
        state (the adjoint fields) into out (nb, 4, nz, nx) FP64."""
        capi.check(self.L.sparc_kernels_accumulate(self.plan, _ptr(fsnaps), fsnaps.shape[1], jf, _ptr(out),
                                                   _stream()), "sparc_kernels_accumulate")

    def adjoint_with_kernels(self, fsnaps: torch.Tensor, out: torch.Tensor, nsteps: int | None = None):
        """The whole adjoint run with the kernel integral (sparc_adjoint): from rest, nsteps steps
        with the flow negated; after each adjoint record, its v_x, v_z against the matching forward
        record of fsnaps (nb, nfwd, 6, nz, nx) accumulated into out (nb, 4, nz, nx) FP64 (zeroed
        first).  The adjoint source must be set."""
        nsteps = self.run.nsteps if nsteps is None else nsteps
        capi.check(self.L.sparc_adjoint(self.plan, _ptr(fsnaps), fsnaps.shape[1], nsteps, _ptr(out), _stream()),
                   "sparc_adjoint")

    def reset(self, time0: int = 0):
        capi.check(self.L.sparc_reset_state(self.plan, time0, _stream()), "sparc_reset_state")

    def run_steps(self, nsteps: int, seis: torch.Tensor | None = None, snaps: torch.Tensor | None = None,
                  nrec_cap: int | None = None, flow_sign: float | None = None, use_graph: bool = True,
                  rec0: int = 0):
        """Advance nsteps steps; records rec0 .. rec0 + nrec_cap - 1 go to the given device tensors
        (slots 0 .. nrec_cap - 1)."""
        if flow_sign is None:
            flow_sign = -1.0 if self.run.adjoint else 1.0
        cap = nrec_cap if nrec_cap is not None else (seis.shape[1] if seis is not None else
                                                     (snaps.shape[1] if snaps is not None else 0))
        if rec0:
            capi.check(self.L.sparc_forward_window(self.plan, nsteps, flow_sign, _ptr(seis), _ptr(snaps), rec0, cap,
                                                   int(use_graph), _stream()), "sparc_forward_window")
        else:
            capi.check(self.L.sparc_forward(self.plan, nsteps, flow_sign, _ptr(seis), _ptr(snaps), cap,
                                            int(use_graph), _stream()), "sparc_forward")

    def checkpoint_bytes(self) -> int:
        """Bytes of one checkpoint (step counter, state, PML auxiliaries of the batch)."""
        return int(self.L.sparc_checkpoint_bytes(self.plan))

    def checkpoint_save(self, buf: torch.Tensor):
        """Copy everything the next step depends on into the device byte buffer buf (16-byte aligned)."""
        capi.check(self.L.sparc_checkpoint_save(self.plan, _ptr(buf), _stream()), "sparc_checkpoint_save")

    def checkpoint_load(self, buf: torch.Tensor):
        capi.check(self.L.sparc_checkpoint_load(self.plan, _ptr(buf), _stream()), "sparc_checkpoint_load")

    def forward(self, nsteps: int | None = None, snapshots: bool = False, use_graph: bool = True):
        """Run from rest: returns seismograms (nb, nrec, nx) and optionally snapshots
        (nb, nrec, 6, nz, nx), as device tensors of the plan precision."""
        run = self.run
        nsteps = nsteps if nsteps is not None else run.nsteps
        nrec = (nsteps - 1) // run.steps_out + 1
        with torch.cuda.device(self.dev):
            seis = torch.zeros((self.nb, nrec, run.nx), dtype=self.dtype, device=self.dev)
            snaps = (torch.zeros((self.nb, nrec, 6, run.nz, run.nx), dtype=self.dtype, device=self.dev)
                     if snapshots else None)
            self.reset(0)
            self.run_steps(nsteps, seis, snaps, nrec, use_graph=use_graph)
        return (seis, snaps) if snapshots else seis

    def state(self) -> torch.Tensor:
        """The state (nb, 4, nz, nx): xi_x, xi_z, v_x, v_z."""
        out = torch.empty((self.nb, 4, self.run.nz, self.run.nx), dtype=self.dtype, device=self.dev)
        capi.check(self.L.sparc_get_state(self.plan, _ptr(out), _stream()), "sparc_get_state")
        return out

    def set_state(self, st: torch.Tensor):
        st = st.to(device=self.dev, dtype=self.dtype).contiguous()
        capi.check(self.L.sparc_set_state(self.plan, _ptr(st), _stream()), "sparc_set_state")

    def profile_passes(self, nsteps: int = 20) -> dict:
        """Event-timed passes of nsteps steps (no graph): milliseconds per step by pass class.
        Advances the state; call reset() before a real run."""
        ms = (ctypes.c_double * 4)()
        capi.check(self.L.sparc_profile_passes(self.plan, nsteps, ms, _stream()), "sparc_profile_passes")
        per = {"row": ms[0] / nsteps, "column": ms[1] / nsteps, "end": ms[2] / nsteps}
        tot = sum(per.values())
        return {"per_class_ms": per, "share": {k: v / tot for k, v in per.items()} if tot > 0 else {},
                "wall_ms_per_step": ms[3] / nsteps}

    LAUNCHES_PER_STEP = 12  # 6 row passes, 5 column passes, 1 end-of-step pass

    def describe(self) -> dict:
        """Kernels of the column and end-of-step passes of this plan and whether the row pass
        overlaps the column pass's last wave (sparc_plan_describe)."""
        buf = ctypes.create_string_buffer(256)
        capi.check(self.L.sparc_plan_describe(self.plan, buf, 256), "sparc_plan_describe")
        return dict(kv.split("=", 1) for kv in buf.value.decode().split())

    def column_kernel_name(self) -> str:
        return self.describe()["column"]

    def check(self) -> np.ndarray:
        """L2 norm of v_z per solve (rms_hist, driver.f90:364-383); raises SparcError with code
        'non-finite state' if any solve diverged."""
        out = np.zeros(self.nb)
        capi.check(self.L.sparc_check_state(self.plan, out.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                            _stream()), "sparc_check_state")
        return out

    def time(self) -> int:
        t = ctypes.c_int()
        capi.check(self.L.sparc_get_time(self.plan, ctypes.byref(t), _stream()), "sparc_get_time")
        return t.value

    def close(self):
        if getattr(self, "plan", None):
            self.L.sparc_plan_destroy(self.plan)
            self.plan = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
