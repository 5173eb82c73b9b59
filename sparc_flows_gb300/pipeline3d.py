"""3-D forward solve, reference-style adjoint solve and kernel integral for a batch of sources,
with the forward field checkpointed in HBM and recomputed per segment.

The 2-D pipeline (pipeline.py) keeps every forward record in HBM; a 3-D record of config 4
(256 x 256 x 300, 4 sources) is 1.6 GB in FP32, so here the forward run keeps its v_z records and
a checkpoint of the state and PML auxiliaries every ``checkpoint_every`` steps (the reference
instead dumps the full state every 200 steps and restarts from disk, driver.f90:418-456), and the
adjoint run, on reaching a segment, restores its checkpoint and recomputes that segment's
kernel-stage records into a buffer of one segment (sparc3d_forward_records).

The adjoint is the reference's kernel-mode adjoint (displacement.f90:615-627): the time-reversed
v_z residual at the observation level, LAGRANGE_INTERP-ed in time (physics.f90:678-737), injected
as forcing / rho0 * delta_width at o_rad of a solve with the flow negated (driver.f90:144-147).
After each adjoint step that produces a record, its v is paired with the matching forward record
(kernels.f90:215, 258) and the integrands of kernels.f90:293-358, extended by the y terms, are
accumulated in FP64 (sparc3d_kernels_accumulate): div xi_f div v_a, sum_j d_i(v_f,j) v_a,j
(i = x, y, z) and |acc_f|^2.
"""
from __future__ import annotations

import numpy as np
import torch

from .config import RunConfig
from .model import lagrange_weights
from .solver3d import WaveSolver3D


class FwdAdjKernels3D:
    """Forward + adjoint + kernel integrands of nb 3-D solves sharing a background and flow."""

    def __init__(self, nx: int, ny: int, model: np.ndarray, xlength_cm: float, patterns: np.ndarray,
                 amp: np.ndarray, nsteps: int, flow=None, precision: int = 32, steps_out: int = 15,
                 checkpoint_every: int = 100, timestep: float = 2.0, device: str = "cuda:0", **kw):
        self.nb, self.nsteps, self.so = patterns.shape[0], int(nsteps), int(steps_out)
        self.K = int(checkpoint_every)
        if self.K < 1:
            raise ValueError("checkpoint_every must be >= 1")
        self.dev = torch.device(device)
        common = dict(nbatch=self.nb, precision=precision, steps_out=steps_out, flows=flow is not None,
                      timestep=timestep, device=device, **kw)
        self.fwd = WaveSolver3D(nx, ny, model, xlength_cm, **common)
        self.adj = WaveSolver3D(nx, ny, model, xlength_cm, **common)
        if flow is not None:
            self.fwd.set_flow(*flow)
            self.adj.set_flow(*[-np.asarray(v) for v in flow])  # driver.f90:144-147
        self.fwd.set_source(patterns, amp)
        self.nrec = (self.nsteps - 1) // self.so + 1
        self.nseg = -(-self.nsteps // self.K)
        row = -(-self.fwd.checkpoint_bytes() // 256) * 256
        self.ckpt = torch.empty((self.nseg, row), dtype=torch.uint8, device=self.dev)
        self.ckpt_time = [0] * self.nseg
        self.seg_rec = max(len(self._records_of(m)) for m in range(self.nseg))
        self.snaps = self.fwd.record_buffer(self.seg_rec)
        self.seis = torch.zeros((self.nrec, self.nb, ny, nx), dtype=self.fwd.dtype, device=self.dev)
        self.kacc = torch.zeros((5, self.fwd.nz, self.nb, ny, nx), dtype=torch.float64, device=self.dev)
        self._seg = None
        self.run_cfg = RunConfig(nx=nx, nz=self.fwd.nz, nsteps=self.nsteps, timestep=timestep,
                                 outputcad=steps_out * timestep, cadforcing=steps_out * timestep)

    def _records_of(self, m: int) -> list[int]:
        """Record indices made by the steps of segment m (steps mK .. (m+1)K - 1)."""
        t0, t1 = m * self.K, min((m + 1) * self.K, self.nsteps)
        return [j for j in range(self.nrec) if t0 <= j * self.so < t1]

    def forward(self) -> torch.Tensor:
        """The forward run: v_z records (nrec, nb, ny, nx) and a checkpoint before every segment."""
        self.fwd.reset(0)
        self._seg = None
        done = 0
        for m in range(self.nseg):
            self.ckpt_time[m] = self.fwd.checkpoint_save(self.ckpt[m])
            n = min(self.K, self.nsteps - m * self.K)
            done += self.fwd.forward_records(n, None, 0, self.seis[done:])
        return self.seis

    def _forward_record(self, jf: int) -> int:
        """Slot of forward record jf in the segment buffer, recomputing its segment if needed."""
        m = (jf * self.so) // self.K
        recs = self._records_of(m)
        if self._seg != m:
            self.fwd.checkpoint_load(self.ckpt[m], self.ckpt_time[m])
            self.fwd.forward_records(min(self.K, self.nsteps - m * self.K), self.snaps, recs[0])
            self._seg = m
        return jf - recs[0]

    def adjoint_source(self, data: torch.Tensor | None = None) -> torch.Tensor:
        """The time-reversed v_z residual (synthetic minus data) at the observation level as adjoint
        source slices (nb, nrec, ny, nx), FP64."""
        res = self.seis.to(torch.float64)
        if data is not None:
            res = res - data.to(device=self.dev, dtype=torch.float64)
        return torch.flip(res, dims=[0]).permute(1, 0, 2, 3).contiguous()

    def adjoint(self, src: torch.Tensor):
        """The adjoint run with the kernel integrands accumulated at each record."""
        idx, w = lagrange_weights(self.run_cfg, self.nsteps + 1, self.run_cfg.num_steps, src.shape[1])
        # the 3-D step counter starts at 0 where the 2-D one has already advanced to 1
        self.adj.set_adjoint_source(src, w[1:], idx[1:])
        self.adj.reset(0)
        self.kacc.zero_()
        done = 0
        for ja in range(self.nrec):
            n = 1 if ja == 0 else self.so
            self.adj.forward_records(n, None)
            done += n
            slot = self._forward_record(self.nrec - 1 - ja)
            self.adj.kernels_accumulate(self.snaps, slot, self.kacc)
        if self.nsteps > done:
            self.adj.forward_records(self.nsteps - done, None)

    def run_all(self, data: torch.Tensor | None = None):
        self.forward()
        self.adjoint(self.adjoint_source(data))
        return self.seis, self.kacc

    def point_steps(self) -> int:
        """Forward + adjoint grid-point steps of one run_all (the segment recomputation not counted)."""
        return 2 * self.nb * self.fwd.nx * self.fwd.ny * self.fwd.nz * self.nsteps

    def close(self):
        self.fwd.close()
        self.adj.close()
