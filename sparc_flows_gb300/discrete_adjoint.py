"""Exact discrete adjoint of the option-17 time step (FP64): the transpose of every operator of
STEP (step.f90:43-119) with MP_QUIET_PML_2D_DISPL's right-hand side (physics2d.f90:943-1094) and
FILTER_VARS_2D (physics2d.f90:509-583), run backwards over a forward solve to give the exact
gradient of a seismogram misfit with respect to the flow stream function.

The reference has no discrete adjoint: its adjoint run is a time-reversed forward solve with the
flow negated (driver.f90:144-147) whose kernels match finite differences only to discretisation
accuracy.  Here the forward solve is the device step of the plan (fused kernels, sparc_forward);
the backward pass replays it segment by segment from HBM checkpoints (sparc_checkpoint_save /
load), recomputes the five stage inputs of each step with the same operators applied one at a
time, and applies the transposed stages in reverse order:

  x-derivative  D_x (spectral, Nyquist bin dropped) is real antisymmetric: D_x^T = -D_x, applied
                with the device ddx;
  z-derivative  dbyd2 with its boundary closures times stretch (ibc 1, 2, 3; the ibc-3 top row
                preset -dxi_x/dx * unstretch, physics2d.f90:954-955) and the z filter are linear
                maps of each column: tabulated once as dense nz x nz FP64 matrices by applying the
                device ddz to the identity, their transposes applied by sparc_colmat_apply;
  PML           the auxiliary equations of psi_vz, psi_p (z) and psi_vx, psi_gradp_x (x) are
                pointwise; their transposes scatter into the derivative adjoints;
  RK            temp_s = a + beta_s R_{s-1}; a' = F(a + dt R_4): reversed stage by stage;
  boundaries    the zeroed RHS rows and columns are a symmetric projection;
  records       the seismogram v_z(k_obs) after steps at multiples of steps_out: its adjoint is
                added to the state adjoint before the step that produced it is transposed.

The flow enters through the advection terms -2 v0x d_x v - 2 v0z d_z v of each stage; their
derivative with respect to v0 is accumulated from the recomputed stage inputs, and v0 =
curl(rho0 c psi) / rho0 (driver.f90:94-115) is linear in psi, so its transpose gives dL/dpsi.
The sound speed enters through p = -c^2 rho0 div - ...: dL/d(c^2 rho0) = -sum lambda_p div over
stages and steps (the exact counterpart of kernel_c, with the PML profiles held fixed).
Pointwise algebra runs as device tensor arithmetic; every derivative, transposed derivative and
transposed filter is one of the plan's kernels.
"""
from __future__ import annotations

import numpy as np
import torch

from . import capi
from .config import RSUN_CM
from .solver import WaveSolver, _ptr, _stream

F64 = torch.float64
# FILTER_VARS_2D coefficients (physics2d.f90:509-583): c0 and the half-weights of neighbours 1..5
FILTER_C = (0.75390625, 0.41015625, -0.234375, 0.087890625, -0.01953125, 0.001953125)


def filter_matrix(nz: int, k0: int) -> np.ndarray:
    """FILTER_VARS_2D's z filter of one column as an nz x nz matrix: rows k0 .. nz-2 are replaced
    (the 11-point filter for 5 <= k <= nz-6, the two-point mean elsewhere), others kept."""
    Fm = np.eye(nz)
    for k in range(k0, nz - 1):
        row = np.zeros(nz)
        if 5 <= k <= nz - 6:
            row[k] = FILTER_C[0]
            for j in range(1, 6):
                row[k - j] += 0.5 * FILTER_C[j]
                row[k + j] += 0.5 * FILTER_C[j]
        else:
            row[k - 1] += 0.5
            row[k + 1] += 0.5
        Fm[k] = row
    return Fm


class StepOperators:
    """The linear operators of one option-17 step of an FP64 plan with one shared background,
    applied one at a time on the device, and their transposes."""

    def __init__(self, ws: WaveSolver):
        if ws.precision != 64 or ws.nbg != 1 or not ws.flows:
            raise ValueError("the discrete adjoint needs an FP64 flow plan with one shared background")
        self.ws, self.L = ws, ws.L
        run, dev = ws.run, ws.dev
        nx, nz = run.nx, run.nz
        self.nx, self.nz, self.nb = nx, nz, ws.nb
        nbt, ntp, nh = run.npmlbot, run.npmltop, run.npmlhor
        self.nzpml, self.nhx = nbt + ntp, 2 * nh
        self.prow = torch.as_tensor(list(range(nbt)) + list(range(nz - ntp, nz)), device=dev)
        self.xcol = torch.as_tensor(list(range(nh)) + list(range(nx - nh, nx)), device=dev)
        bg = ws.bg
        col = lambda t: t.reshape(nz, 1)  # noqa: E731
        fdz = torch.ones((nz, nx), dtype=F64, device=dev)
        fdz[self.prow] = bg["fdz"][0]
        self.gp0 = col(bg["gradp0_z"]) * fdz          # background gradients decayed in the PML
        self.gr0 = col(bg["gradrho0_z"]) * fdz
        c2r = bg["c2rho0"]
        self.c2rho0 = c2r[0] if c2r.dim() == 3 else col(c2r)
        self.rho0, self.rhoinv, self.g = col(bg["rho0"]), col(bg["rhoinv"]), col(bg["g"])
        self.az, self.bz = bg["az"][0], bg["bz"][0]
        self.ax, self.bx = bg["ax"][0], bg["bx"][0]
        self.ut = float(bg["unstretch"][nz - 1])
        self.stretch = bg["stretch"]
        self.dt, self.betas = ws.deltat, ws.betas
        self.k_inj, self.k_obs = ws.k_inj, ws.o_rad
        self.src_until = run.src_until
        # dense column operators: M[ibc][:, j] = ddz(e_j) (stretch included), the ibc-3 top preset
        # column, and the z filter; transposes kept contiguous for sparc_colmat_apply
        eye = torch.eye(nz, dtype=F64, device=dev).contiguous()
        self.M, self.MT = {}, {}
        for ibc in (1, 2, 3):
            m = torch.empty_like(eye)
            ws.ddz(eye, m, n1=nz, ibc=ibc, stretch=self.stretch)
            self.M[ibc] = m
            self.MT[ibc] = m.t().contiguous()
        one = torch.ones(1, dtype=F64, device=dev)
        m3p = torch.empty((nz, 1), dtype=F64, device=dev)
        ws.ddz(torch.zeros((nz, 1), dtype=F64, device=dev), m3p, n1=1, ibc=3, preset=one, stretch=self.stretch)
        self.m3p = m3p.reshape(1, nz, 1)
        Fm = filter_matrix(nz, run.filter_kst - 1)
        self.Fm = torch.as_tensor(Fm, device=dev).contiguous()
        self.FmT = torch.as_tensor(Fm.T.copy(), device=dev).contiguous()
        self.fi0, self.fi1 = (0, nx - 1) if run.filter_all_x else (nh - 1, nx - nh)
        torch.cuda.synchronize(dev)

    # ---- elementary operators -------------------------------------------------------------
    def dx(self, f: torch.Tensor) -> torch.Tensor:
        f = f.contiguous()
        out = torch.empty_like(f)
        self.ws.ddx(f, out, nrows=f.numel() // self.nx, stretchx=self.ws.stretchx)
        return out

    def dxT(self, f: torch.Tensor) -> torch.Tensor:
        return -self.dx(f)

    def colmat(self, W: torch.Tensor, f: torch.Tensor, i0: int = 0, i1: int | None = None) -> torch.Tensor:
        f = f.contiguous()
        out = torch.empty_like(f)
        nplanes = f.numel() // (self.nz * self.nx)
        capi.check(self.L.sparc_colmat_apply(_ptr(W), self.nz, _ptr(f), _ptr(out), nplanes, self.nx, i0,
                                             self.nx - 1 if i1 is None else i1, 0, _stream()), "sparc_colmat_apply")
        return out

    def dz(self, f, ibc):
        return self.colmat(self.M[ibc], f)

    def dzT(self, f, ibc):
        return self.colmat(self.MT[ibc], f)

    def _zero_boundaries(self, R: torch.Tensor) -> torch.Tensor:
        R[:, :, 0, :] = 0.0
        R[:, :, :, 0] = 0.0
        R[:, :, :, -1] = 0.0
        return R

    # ---- one stage ------------------------------------------------------------------------
    def rhs(self, X, Pz, Px, v0x, v0z, forcing=None):
        """Right-hand side of one stage (physics2d.f90:943-1094) for the stage input X (nb, 4, nz,
        nx) = (xi_x, xi_z, v_x, v_z) and PML auxiliaries Pz (nb, 2, nzpml, nx) = (psi_vz, psi_p),
        Px (nb, 2, nz, 2 npmlhor) = (psi_vx, psi_gradp_x).  forcing (nb, nx) is added to RHS v_z at
        the injection row.  Returns (R, RPz, RPx, the four velocity derivatives and div)."""
        xi_x, xi_z, v_x, v_z = X.unbind(1)
        pr, xc = self.prow, self.xcol
        dxx = self.dx(xi_x)
        preset = -dxx[:, -1, :] * self.ut
        dzz = self.dz(xi_z, 3) + self.m3p * preset[:, None, :]
        RPvz = self.az * dzz[:, pr, :] + self.bz * Pz[:, 0]
        dzz[:, pr, :] = dzz[:, pr, :] + Pz[:, 0]
        dxx[:, :, xc] = dxx[:, :, xc] + Px[:, 0]
        RPvx = self.ax * dxx[:, :, xc] + self.bx * Px[:, 0]
        div = dxx + dzz
        p = -self.c2rho0 * div - self.gp0 * xi_z
        gpx = self.dx(p)
        gpx[:, :, xc] = gpx[:, :, xc] + Px[:, 1]
        RPg = self.ax * gpx[:, :, xc] + self.bx * Px[:, 1]
        gpz = self.dz(p, 2)
        RPp = self.az * gpz[:, pr, :] + self.bz * Pz[:, 1]
        gpz[:, pr, :] = gpz[:, pr, :] + Pz[:, 1]
        rho = -self.rho0 * div - self.gr0 * xi_z
        Rvx = -self.rhoinv * gpx
        Rvz = -self.rhoinv * (gpz + rho * self.g)
        if forcing is not None:
            Rvz[:, self.k_inj, :] += forcing
        d = (self.dx(v_x), self.dz(v_x, 1), self.dx(v_z), self.dz(v_z, 1), div)
        Rvx = Rvx - 2.0 * v0x * d[0] - 2.0 * v0z * d[1]
        Rvz = Rvz - 2.0 * v0x * d[2] - 2.0 * v0z * d[3]
        R = self._zero_boundaries(torch.stack((v_x.clone(), v_z.clone(), Rvx, Rvz), 1))
        return R, torch.stack((RPvz, RPp), 1), torch.stack((RPvx, RPg), 1), d

    def rhs_T(self, lR, lRPz, lRPx, v0x, v0z, d):
        """Transpose of the linear part of rhs: adjoints of (R, RPz, RPx) -> adjoints of (X, Pz,
        Px), and the derivatives of <lR, R> with respect to v0x, v0z and c2rho0 (summed over the
        batch; d holds the stage's velocity derivatives and div, zeros for the operator alone)."""
        pr, xc = self.prow, self.xcol
        lR = self._zero_boundaries(lR.clone())
        lRxx, lRxz, lRvx, lRvz = lR.unbind(1)
        gv0x = (-2.0 * (lRvx * d[0] + lRvz * d[2])).sum(0)
        gv0z = (-2.0 * (lRvx * d[1] + lRvz * d[3])).sum(0)
        lvx = lRxx - 2.0 * self.dxT(v0x * lRvx) - 2.0 * self.dzT(v0z * lRvx, 1)
        lvz = lRxz - 2.0 * self.dxT(v0x * lRvz) - 2.0 * self.dzT(v0z * lRvz, 1)
        lgpz = -self.rhoinv * lRvz
        lrho = -self.rhoinv * self.g * lRvz
        ldiv = -self.rho0 * lrho
        lxiz = -self.gr0 * lrho
        lgpx = -self.rhoinv * lRvx
        # z-PML of dp/dz, dp/dz (ibc 2)
        lpsip = lgpz[:, pr, :] + self.bz * lRPz[:, 1]
        lgpz[:, pr, :] = lgpz[:, pr, :] + self.az * lRPz[:, 1]
        lp = self.dzT(lgpz, 2)
        # x-PML of dp/dx, dp/dx
        lgpx[:, :, xc] = lgpx[:, :, xc] + self.ax * lRPx[:, 1]
        lpsig = lgpx[:, :, xc] + self.bx * lRPx[:, 1]
        lp = lp + self.dxT(lgpx)
        # pressure p = -c2rho0 div - gradp0_z xi_z
        gc2 = (-(lp * d[4])).sum(0) if len(d) > 4 else torch.zeros_like(gv0x)
        ldiv = ldiv - self.c2rho0 * lp
        lxiz = lxiz - self.gp0 * lp
        # x-PML of dxi_x/dx
        ldxx = ldiv.clone()
        ldxx[:, :, xc] = ldxx[:, :, xc] + self.ax * lRPx[:, 0]
        lpsivx = ldxx[:, :, xc] + self.bx * lRPx[:, 0]
        # z-PML of dxi_z/dz, dxi_z/dz (ibc 3) with its top preset
        lpsivz = ldiv[:, pr, :] + self.bz * lRPz[:, 0]
        ldzz = ldiv.clone()
        ldzz[:, pr, :] = ldzz[:, pr, :] + self.az * lRPz[:, 0]
        lxiz = lxiz + self.dzT(ldzz, 3)
        lpre = (self.m3p * ldzz).sum(1)
        ldxx[:, -1, :] = ldxx[:, -1, :] - self.ut * lpre
        lxix = self.dxT(ldxx)
        lX = torch.stack((lxix, lxiz, lvx, lvz), 1)
        return lX, torch.stack((lpsivz, lpsip), 1), torch.stack((lpsivx, lpsig), 1), gv0x, gv0z, gc2

    # ---- one step -------------------------------------------------------------------------
    def filt(self, a):
        return self.colmat(self.Fm, a, self.fi0, self.fi1)

    def filtT(self, la):
        return self.colmat(self.FmT, la, self.fi0, self.fi1)

    def step(self, a, Pz, Px, v0x, v0z, forcing=None):
        """One step (STEP, step.f90:43-119) from (a, Pz, Px); returns the new state and the
        stage caches (velocity derivatives of the five stage inputs)."""
        caches = []
        X, Z, W = a, Pz, Px
        for s in range(5):
            if s > 0:
                b = self.betas[s]
                X, Z, W = a + b * R, Pz + b * RPz, Px + b * RPx
            R, RPz, RPx, d = self.rhs(X, Z, W, v0x, v0z, forcing)
            caches.append(d)
        a1 = self.filt(a + self.dt * R)
        return a1, Pz + self.dt * RPz, Px + self.dt * RPx, caches

    def step_T(self, la, lPz, lPx, v0x, v0z, caches):
        """Transpose of step (linear part) given the adjoints of its outputs; returns the adjoints
        of its inputs and the gradients with respect to v0x, v0z and c2rho0."""
        mu = self.filtT(la)
        lA, lZ0, lW0 = mu.clone(), lPz.clone(), lPx.clone()
        lR, lRPz, lRPx = self.dt * mu, self.dt * lPz, self.dt * lPx
        gx = torch.zeros((self.nz, self.nx), dtype=F64, device=la.device)
        gz = torch.zeros_like(gx)
        gc = torch.zeros_like(gx)
        for s in range(4, -1, -1):
            lX, lZ, lW, g1, g2, g3 = self.rhs_T(lR, lRPz, lRPx, v0x, v0z, caches[s])
            gx += g1
            gz += g2
            gc += g3
            lA += lX
            lZ0 += lZ
            lW0 += lW
            if s > 0:
                b = self.betas[s]
                lR, lRPz, lRPx = b * lX, b * lZ, b * lW
        return lA, lZ0, lW0, gx, gz, gc


class ExactGradient:
    """Seismograms at receiver columns as a function of the stream function, with the exact
    gradient of any loss of them by the discrete adjoint.  The forward solve is the plan's device
    step; states are checkpointed every `segment` steps in HBM and each segment is replayed once
    during the backward pass."""

    def __init__(self, ws: WaveSolver, receivers, segment: int = 25, use_graph: bool = True):
        self.ws, self.ops = ws, StepOperators(ws)
        self.use_graph, self._graph = use_graph, None
        self.run = ws.run
        self.rcv = torch.as_tensor(np.asarray(receivers), device=ws.dev)
        self.seg = int(segment)
        self.nrec = self.run.nrec
        n = self.run.nsteps
        self.nseg = -(-n // self.seg)
        ops = self.ops
        nb, nz, nx = ops.nb, ops.nz, ops.nx
        self._nA, self._nZ, self._nW = nb * 4 * nz * nx, nb * 2 * ops.nzpml * nx, nb * 2 * nz * ops.nhx
        nbytes = ws.checkpoint_bytes()
        if nbytes != 16 + 8 * (self._nA + self._nZ + self._nW):
            raise RuntimeError("unexpected checkpoint layout")
        self.row = -(-nbytes // 256) * 256
        self.ckpt = torch.empty((self.nseg, self.row), dtype=torch.uint8, device=ws.dev)
        self.segbuf = torch.empty((self.seg, self.row), dtype=torch.uint8, device=ws.dev)
        self.seis = torch.zeros((nb, self.nrec, nx), dtype=F64, device=ws.dev)
        ws_rows = getattr(ws, "src_rows", None)
        if ws_rows is None:
            raise ValueError("set the forward sources first")
        self.src_rows = torch.as_tensor(ws_rows[:, 0, :], device=ws.dev)
        self.src_ts = np.asarray(ws.src_wts[:, 0])
        self.inj = ws.delta_width / ws.rho0[ws.k_inj]

    def _views(self, blob):
        ops, o = self.ops, 16
        out = []
        for n, shape in ((self._nA, (ops.nb, 4, ops.nz, ops.nx)), (self._nZ, (ops.nb, 2, ops.nzpml, ops.nx)),
                         (self._nW, (ops.nb, 2, ops.nz, ops.nhx))):
            out.append(blob[o:o + 8 * n].view(F64).view(shape))
            o += 8 * n
        return out

    def _forcing(self, time: int):
        if 0 <= time <= self.ops.src_until and time < len(self.src_ts):
            return self.src_ts[time] * self.src_rows * self.inj
        return None

    def forward(self, psi: torch.Tensor) -> torch.Tensor:
        ws = self.ws
        ws.update_flow(psi)
        ws.reset(0)
        n = self.run.nsteps
        for m in range(self.nseg):
            ws.checkpoint_save(self.ckpt[m])
            ws.run_steps(min(self.seg, n - m * self.seg), self.seis, None, self.nrec)
        return self.seis[:, :, self.rcv]

    def _static(self):
        """Static device buffers of one reverse step: the state before the step, the adjoints,
        the gradient accumulators, the forcing row and the flow."""
        if getattr(self, "_s", None) is None:
            ops, dev = self.ops, self.ws.dev
            sa, sz, sw = ((ops.nb, 4, ops.nz, ops.nx), (ops.nb, 2, ops.nzpml, ops.nx), (ops.nb, 2, ops.nz, ops.nhx))
            z = lambda sh: torch.zeros(sh, dtype=F64, device=dev)  # noqa: E731
            self._s = dict(a=z(sa), Pz=z(sz), Px=z(sw), la=z(sa), lZ=z(sz), lW=z(sw), gx=z((ops.nz, ops.nx)),
                           gz=z((ops.nz, ops.nx)), gc=z((ops.nz, ops.nx)), f=z((ops.nb, ops.nx)),
                           v0x=z((ops.nz, ops.nx)),
                           v0z=z((ops.nz, ops.nx)))
        return self._s

    def _reverse_step(self):
        """Recompute the stages of one step from the static state and apply the transposed step
        to the static adjoints in place, accumulating the flow gradient."""
        S, ops = self._s, self.ops
        _, _, _, caches = ops.step(S["a"], S["Pz"], S["Px"], S["v0x"], S["v0z"], S["f"])
        la, lZ, lW, g1, g2, g3 = ops.step_T(S["la"], S["lZ"], S["lW"], S["v0x"], S["v0z"], caches)
        S["la"].copy_(la)
        S["lZ"].copy_(lZ)
        S["lW"].copy_(lW)
        S["gx"].add_(g1)
        S["gz"].add_(g2)
        S["gc"].add_(g3)

    def _run_reverse_step(self):
        """One reverse step, replayed from a CUDA graph when capture works (the same launches
        on the same buffers), eagerly otherwise."""
        if self.use_graph and self._graph is None:
            S = self._s
            keep = {k: v.clone() for k, v in S.items()}
            try:
                side = torch.cuda.Stream(device=self.ws.dev)
                side.wait_stream(torch.cuda.current_stream(self.ws.dev))
                with torch.cuda.stream(side):
                    for _ in range(2):
                        self._reverse_step()
                torch.cuda.current_stream(self.ws.dev).wait_stream(side)
                g = torch.cuda.CUDAGraph()
                with torch.cuda.graph(g):
                    self._reverse_step()
                self._graph = g
            except RuntimeError:
                self.use_graph = False
            for k, v in keep.items():  # the warm-up and capture ran on the live buffers
                S[k].copy_(v)
        if self._graph is not None:
            self._graph.replay()
        else:
            self._reverse_step()

    def gradient(self, psi: torch.Tensor, grad_rec: torch.Tensor) -> torch.Tensor:
        """dL/dpsi for dL/d(records at the receivers) = grad_rec (nb, nrec, nrcv), at the psi of
        the last forward call."""
        ws, ops, run = self.ws, self.ops, self.run
        so, n = run.steps_out, run.nsteps
        S = self._static()
        for k in ("la", "lZ", "lW", "gx", "gz", "gc"):
            S[k].zero_()
        S["v0x"].copy_(ws.bg["v0x"][0])
        S["v0z"].copy_(ws.bg["v0z"][0])
        grad_rec = grad_rec.to(device=ws.dev, dtype=F64)
        for m in range(self.nseg - 1, -1, -1):
            n0, n1 = m * self.seg, min((m + 1) * self.seg, n)
            ws.checkpoint_load(self.ckpt[m])
            for j in range(n1 - n0):  # replay the segment, keeping the state before each step
                ws.checkpoint_save(self.segbuf[j])
                ws.run_steps(1, None, None, 0)
            for step in range(n1 - 1, n0 - 1, -1):
                if step % so == 0 and step // so < self.nrec:  # record taken after this step
                    S["la"][:, 3, ops.k_obs, self.rcv] += grad_rec[:, step // so, :]
                for dst, src in zip((S["a"], S["Pz"], S["Px"]), self._views(self.segbuf[step - n0])):
                    dst.copy_(src)
                fc = self._forcing(step)
                if fc is None:
                    S["f"].zero_()
                else:
                    S["f"].copy_(fc)
                self._run_reverse_step()
        self.last = {"v0x": S["gx"].clone(), "v0z": S["gz"].clone(), "c2rho0": S["gc"].clone()}
        return self.psi_gradient(self.last["v0x"], self.last["v0z"])

    def set_c2rho0(self, c2rho0: torch.Tensor):
        """Replace the plan's c^2 rho0 field (nz, nx), the PML profiles kept: the parameter whose
        gradient ``last["c2rho0"]`` is (needs a plan built with a sound-speed field, cmul)."""
        ws = self.ws
        if ws.bg["c2rho0"].dim() != 3:
            raise ValueError("the plan has a depth-only c^2 rho0; build it with cmul")
        # in place: the operators (and a captured reverse-step graph) hold this buffer's address
        ws.bg["c2rho0"].copy_(c2rho0.to(device=ws.dev, dtype=F64).reshape(1, self.ops.nz, self.ops.nx))
        ws._upload_background()

    def psi_gradient(self, gx: torch.Tensor, gz: torch.Tensor) -> torch.Tensor:
        """Transpose of psi -> (v0x, v0z) = (-d_z(rho0 c psi / R) / rho0, d_x(rho0 c psi / R) / rho0)
        (driver.f90:94-115, solver.update_flow)."""
        ops, ws = self.ops, self.ws
        r0 = ops.rho0
        c = torch.sqrt(torch.as_tensor(ws.c2[0], device=ws.dev))
        gpv = ops.dzT((-gx / r0)[None], 1)[0] + ops.dxT((gz / r0)[None])[0]
        return r0 * c * gpv / (RSUN_CM / 1.0e8)


class RecordsFromPsi(torch.autograd.Function):
    """Records at the receivers as a differentiable function of psi; backward is the exact
    discrete adjoint of the device forward solve."""

    @staticmethod
    def forward(ctx, psi: torch.Tensor, eg: ExactGradient):
        out = eg.forward(psi.detach())
        ctx.eg = eg
        ctx.save_for_backward(psi.detach())
        return out.clone()

    @staticmethod
    def backward(ctx, grad):
        (psi,) = ctx.saved_tensors
        eg = ctx.eg
        eg.forward(psi)  # the checkpoints of this psi (another forward may have run since)
        return eg.gradient(psi, grad), None


def records(psi: torch.Tensor, eg: ExactGradient) -> torch.Tensor:
    return RecordsFromPsi.apply(psi, eg)
