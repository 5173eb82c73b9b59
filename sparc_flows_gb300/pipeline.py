"""Forward solve, reference-style adjoint solve and sensitivity kernels for a batch of sources:
the sequence full.py runs per source (full.py:18-59) -- ``sparc NN 00`` with the Spectral
instruction, with the Adjoint instruction, then without one (kernel stage) -- done in one process
with every wavefield resident in HBM instead of ~520 partial-state FITS dumps.

Forward partial states are kept in device memory at the reference cadence (every
steps_out steps, all_modules.f90:750-784): all of them, or with ``checkpoint_every=K`` only a
checkpoint of the forward solve every K records and a buffer of K records, each segment being
recomputed from its checkpoint when the adjoint run reaches it (one more forward solve for about
K/nrec of the memory).  The adjoint is the reference's continuous adjoint: a
forward-type solve with the flow negated (driver.f90:144-147) driven by the time-reversed
residual injected at o_rad (physics2d.f90:1052-1054).  After each adjoint step that produces a
record, its v_x, v_z are paired with the matching forward record (kernels.f90:215, 258) and the
kernel integrands are accumulated in FP64 on the device; the final scalings and the stream-function
kernel follow kernels.f90:495-581.
"""
from __future__ import annotations

import math

import numpy as np
import torch

from .config import DIMC, RSUN_CM, RunConfig
from .model import SourceSpec
from .solver import WaveSolver

L1E8 = float(np.float32(1e-8))   # 10.0**(-8.) in kernels.f90 is a single-precision constant
L1E5 = float(np.float32(1e-5))
DIMRHO_KERNEL = float(np.float32(1e-3))  # kernel_back uses dimrho = 10.0**(-3.0) (initialize.f90:962)


def receiver_columns(run: RunConfig, n: int = 128, x0: float = -127.0, dx: float = 2.0) -> np.ndarray:
    """Grid columns nearest to receivers at x0 + dx*j Mm (box-centred coordinates)."""
    x = (np.arange(run.nx) / run.nx - 0.5) * run.xlength_cm * 1e-8
    return np.array([int(np.argmin(np.abs(x - (x0 + dx * j)))) for j in range(n)])


class FwdAdjKernels:
    """Batched forward + adjoint + kernel computation for one model and many sources."""

    def __init__(self, run: RunConfig, model: np.ndarray, specs: list[SourceSpec], psi=None, cmul=None,
                 precision: int = 32, receivers: np.ndarray | None = None, device: str = "cuda:0",
                 column_impl: int | None = None, column_block: int | None = None,
                 checkpoint_every: int | None = None):
        self.run, self.nb = run, len(specs)
        self.ck = int(checkpoint_every) if checkpoint_every else 0
        if self.ck < 0 or self.ck >= run.nrec:
            raise ValueError(f"checkpoint_every must be in 1..{run.nrec - 1}")
        self.dev = torch.device(device)
        col = dict(column_impl=column_impl, column_block=column_block)
        self.fwd = WaveSolver(run, model, nbatch=self.nb, precision=precision, cmul=cmul, psi=psi, device=device, **col)
        self.fwd.set_forward_sources(specs)
        self.adj = WaveSolver(run.replace(adjoint=True), model, nbatch=self.nb, precision=precision, cmul=cmul,
                              psi=psi, device=device, **col)
        self.nrec = run.nrec
        self.rcv = receiver_columns(run) if receivers is None else np.asarray(receivers)
        dt = self.fwd.dtype
        nbuf = self.ck or self.nrec
        with torch.cuda.device(self.dev):
            self.seis = torch.zeros((self.nb, self.nrec, run.nx), dtype=dt, device=self.dev)
            self.snaps = torch.zeros((self.nb, nbuf, 6, run.nz, run.nx), dtype=dt, device=self.dev)
            if self.ck:
                nseg = -(-self.nrec // self.ck)
                row = -(-self.fwd.checkpoint_bytes() // 256) * 256  # each checkpoint 256-byte aligned
                self.ckpt = torch.empty((nseg, row), dtype=torch.uint8, device=self.dev)
            self.kacc = torch.zeros((self.nb, 4, run.nz, run.nx), dtype=torch.float64, device=self.dev)
            self.rcv_t = torch.as_tensor(self.rcv, device=self.dev)
        self._adj_src = None
        self._seg = None  # segment whose forward records are in the buffer (checkpointed runs)

    def adjoint_source(self, data: torch.Tensor | None) -> torch.Tensor:
        """Waveform residual (synthetic minus data) at the receiver columns, time reversed, as the
        adjoint source slices (nb, nrec, nx) at cadforcing cadence (the layout of source.fits)."""
        res = self.seis.to(torch.float64)
        if data is not None:
            res = res - data.to(device=self.dev, dtype=torch.float64)
        src = torch.zeros((self.nb, self.nrec, self.run.nx), dtype=torch.float64, device=self.dev)
        src[:, :, self.rcv_t] = torch.flip(res[:, :, self.rcv_t], dims=[1])
        return src

    def _segment_steps(self, m: int) -> int:
        """Steps of segment m: those from the step that writes record m*K up to the next segment's."""
        so = self.run.steps_out
        return min((m + 1) * self.ck * so, self.run.nsteps) - m * self.ck * so

    def forward(self):
        self.fwd.reset(0)
        self._seg = None
        if not self.ck:
            self.fwd.run_steps(self.run.nsteps, self.seis, self.snaps, self.nrec)
            return self.seis
        for m in range(self.ckpt.shape[0]):
            self.fwd.checkpoint_save(self.ckpt[m])
            self.fwd.run_steps(self._segment_steps(m), self.seis, None, self.nrec)
        return self.seis

    def _forward_records(self, jf: int):
        """(buffer, slot) holding forward record jf, recomputing its segment from the checkpoint."""
        if not self.ck:
            return self.snaps, jf
        m = jf // self.ck
        if self._seg != m:
            self.fwd.checkpoint_load(self.ckpt[m])
            self.fwd.run_steps(self._segment_steps(m), None, self.snaps, self.ck, rec0=m * self.ck)
            self._seg = m
        return self.snaps, jf - m * self.ck

    def adjoint(self, src: torch.Tensor):
        """Adjoint solve with kernel accumulation at each record (kernels.f90:209-358)."""
        run, so = self.run, self.run.steps_out
        self.adj.set_adjoint_sources_device(src)
        if not self.ck:  # every forward record is resident: the library runs the whole loop
            self.adj.adjoint_with_kernels(self.snaps, self.kacc, run.nsteps)
            return
        self.adj.reset(0)
        self.kacc.zero_()
        done = 0
        for ja in range(self.nrec):
            n = 1 if ja == 0 else so
            self.adj.run_steps(n, None, None, 0)
            done += n
            buf, slot = self._forward_records(self.nrec - 1 - ja)
            self.adj.kernels_accumulate(buf, slot, self.kacc)
        if run.nsteps > done:
            self.adj.run_steps(run.nsteps - done, None, None, 0)

    def run_all(self, data: torch.Tensor | None = None):
        self.forward()
        src = self.adjoint_source(data)
        self.adjoint(src)
        return self.seis, self.kacc

    def launch_count(self) -> int:
        """Kernels of ours launched by one run_all."""
        per = WaveSolver.LAUNCHES_PER_STEP
        solves = 3 if self.ck else 2  # the checkpointed run recomputes the forward solve once
        return solves * per * self.run.nsteps + 2 * self.nrec + 4

    def point_steps(self) -> int:
        """Grid-point steps of one run_all (forward and adjoint counted once each)."""
        return 2 * self.nb * self.run.nx * self.run.nz * self.run.nsteps

    def final_kernels(self, summed: bool = True) -> dict:
        """Scaled kernels (kernels.f90:495-581): kernel_c, kernel_vx, kernel_vz, kernel_psi, hessian."""
        acc = self.kacc.sum(0, keepdim=True) if summed else self.kacc
        return scale_kernels(self.fwd, acc)

    def close(self):
        self.fwd.close()
        self.adj.close()


def scale_kernels(ws: WaveSolver, acc: torch.Tensor) -> dict:
    """Final scalings of PRODUCE_KERNELS (kernels.f90:495-581) applied to accumulated integrands
    acc (n, 4, nz, nx) = (div f_xi div a_v, d_x f_v . a_v, d_z f_v . a_v, |f_acc|^2) summed over
    the records.  The stream-function kernel is the y-component of the curl of the flow kernel
    with the kernel-stage z-derivative at ibc 0 (CURL_KERN, kernels.f90:815-838, 510-513)."""
    run, dev = ws.run, ws.dev
    nz, nx = run.nz, run.nx
    rho0k = torch.as_tensor(ws.rho0 * 1e-3 / DIMRHO_KERNEL, device=dev)[None, :, None]
    c2k = torch.as_tensor(np.stack(ws.c2), device=dev)
    if c2k.shape[0] != acc.shape[0]:
        c2k = c2k[:1]
    stepskern = float(run.steps_out)
    dimen = 1.0 / (RSUN_CM * L1E8 * run.xlength_cm * L1E8 * DIMC * L1E5)
    kv1, kv3 = acc[:, 1], acc[:, 2]
    t2 = torch.empty((nz, nx), dtype=torch.float64, device=dev)
    t3 = torch.empty_like(t2)
    kpsi = torch.empty_like(kv1)
    for b in range(acc.shape[0]):
        ws.ddzkern(kv1[b].contiguous(), t2, n1=nx, ibc=0, stretch=ws.stretch_t)
        ws.ddx(kv3[b].contiguous(), t3, nrows=nz, stretchx=ws.stretchx)
        kpsi[b] = t2 - t3
    fac = stepskern * run.timestep
    kernel_psi = 2.0 * kpsi * dimen * (rho0k * torch.sqrt(c2k)) * fac * dimen
    kernel_vx = -2.0 * kv1 * rho0k * fac * dimen
    kernel_vz = -2.0 * kv3 * rho0k * fac * dimen
    dimc2 = 1.0 / (RSUN_CM * L1E8 * run.xlength_cm * L1E8)
    kernel_c = -acc[:, 0] * rho0k * c2k * fac * dimc2 * 2.0
    return dict(kernel_c=kernel_c, kernel_vx=kernel_vx, kernel_vz=kernel_vz, kernel_psi=kernel_psi,
                hessian=acc[:, 3])


def kernels_from_partial_states(ws: WaveSolver, fsn: np.ndarray, asn: np.ndarray) -> dict:
    """PRODUCE_KERNELS from stored partial states of one forward and one adjoint run
    ((nrec, 6, nz, nx) each): pairs forward record j with adjoint record n-1-j and returns the
    scaled kernels as (nz, nx) host arrays."""
    import ctypes
    from . import capi
    from .solver import _ptr, _stream

    dev, dt = ws.dev, ws.dtype
    f = torch.as_tensor(fsn, dtype=dt, device=dev)[None].contiguous()
    a = torch.as_tensor(asn, dtype=dt, device=dev)[None].contiguous()
    npair = min(f.shape[1], a.shape[1])
    acc = torch.zeros((1, 4, ws.run.nz, ws.run.nx), dtype=torch.float64, device=dev)
    capi.check(ws.L.sparc_kernels(ws.plan, _ptr(f), f.shape[1], _ptr(a), a.shape[1], npair, _ptr(acc), _stream()),
               "sparc_kernels")
    out = scale_kernels(ws, acc)
    return {k: v[0].cpu().numpy() for k, v in out.items()}
