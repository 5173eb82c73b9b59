"""torch.autograd wrapper of the forward / adjoint pair: seismograms as a function of the flow
stream function psi.

forward  = the forward solve of every source of a ``FwdAdjKernels`` batch with v0 recomputed
           from psi on the GPU (driver.f90:94-147, TIMESTEPPING driver.f90:337-475), returning
           v_z at the receiver columns, (nb, nrec, nrcv);
backward = the reference's adjoint: the incoming gradient at the receivers, time reversed, is
           the adjoint source (driver.f90:584-594, LAGRANGE_INTERP physics.f90:678-737) of a
           solve with the flow negated (driver.f90:144-147); the kernel integral over the
           records (kernels.f90:209-358) and PRODUCE_KERNELS' scalings give kernel_psi
           (kernels.f90:495-513), summed over the batch, which is returned as the gradient.

For L = 1/2 |seis - data|^2 the incoming gradient is the waveform residual, so backward runs
exactly the reference's adjoint + kernel stage.  The reference's adjoint is a continuous
(time-reversal) adjoint and kernel_psi a density: kernel_psi times the cell height dz equals
dL/dpsi up to the reference's fixed normalisation (its units and sign) below the receiver layer,
but not in the top rows that hold the receiver / adjoint-source row and the top PML, where the
time-reversed solve is not the discrete adjoint (measured in tests/test_gpu_reference_kernel.py).
``fd_check`` measures it against central finite differences, with the dz pairing if given.

The exact gradient of the same seismograms is ``exact_records`` (discrete_adjoint.py): its
backward is the transpose of the device step itself, replayed from HBM checkpoints, and agrees
with central finite differences to rounding.
"""
from __future__ import annotations

import numpy as np
import torch

from .discrete_adjoint import ExactGradient, records as exact_records  # noqa: F401
from .pipeline import FwdAdjKernels


class SeismogramsFromPsi(torch.autograd.Function):
    @staticmethod
    def forward(ctx, psi: torch.Tensor, pipe: FwdAdjKernels):
        pipe.fwd.update_flow(psi)
        pipe.adj.update_flow(psi)
        seis = pipe.forward()
        ctx.pipe = pipe
        return seis[:, :, pipe.rcv_t].to(torch.float64).clone()

    @staticmethod
    def backward(ctx, grad_seis: torch.Tensor):
        pipe = ctx.pipe
        nb, nrec, nx = pipe.nb, pipe.nrec, pipe.run.nx
        src = torch.zeros((nb, nrec, nx), dtype=torch.float64, device=pipe.dev)
        src[:, :, pipe.rcv_t] = torch.flip(grad_seis.to(torch.float64), dims=[1])
        pipe.adjoint(src)
        kpsi = pipe.final_kernels(summed=True)["kernel_psi"][0]
        return kpsi.to(torch.float64), None


def seismograms(psi: torch.Tensor, pipe: FwdAdjKernels) -> torch.Tensor:
    """Differentiable seismograms at the receivers of ``pipe`` for stream function psi (nz, nx)."""
    return SeismogramsFromPsi.apply(psi, pipe)


def fd_check(pipe: FwdAdjKernels, psi: torch.Tensor, data: torch.Tensor, directions: list[torch.Tensor],
             eps: float, weight: torch.Tensor | None = None) -> dict:
    """Central finite differences of L(psi) = 1/2 |seis(psi) - data|^2 along each direction
    against <grad, direction> from backward (weighted by ``weight``, e.g. the cell height dz per
    row, if given).  Returns the per-direction ratios FD / <grad, d>: their spread measures the
    gradient's direction error, their mean the normalisation."""
    psi = psi.detach().clone().requires_grad_(True)
    loss = 0.5 * ((seismograms(psi, pipe) - data) ** 2).sum()
    loss.backward()
    g = psi.grad.detach().clone()
    ratios, fds, dots = [], [], []
    for d in directions:
        with torch.no_grad():
            lp = 0.5 * ((seismograms(psi.detach() + eps * d, pipe) - data) ** 2).sum().item()
            lm = 0.5 * ((seismograms(psi.detach() - eps * d, pipe) - data) ** 2).sum().item()
        fd = (lp - lm) / (2.0 * eps)
        dot = float((g * d * (weight if weight is not None else 1.0)).sum().item())
        fds.append(fd)
        dots.append(dot)
        ratios.append(fd / dot if dot != 0.0 else float("nan"))
    r = np.asarray(ratios)
    return {"fd": fds, "dot": dots, "ratio": ratios, "ratio_mean": float(r.mean()),
            "ratio_spread": float(r.std() / abs(r.mean())) if r.size > 1 else 0.0, "loss": float(loss.item())}
