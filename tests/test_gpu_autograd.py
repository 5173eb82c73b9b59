"""autograd wrapper of the forward / adjoint pair (forward = the forward solve, backward = the
reference's adjoint + kernel stage)."""
import numpy as np
import pytest
import torch

from sparc_flows_gb300 import model as M
from sparc_flows_gb300.config import RunConfig

pytestmark = pytest.mark.gpu


def test_backward_is_the_reference_kernel_of_the_residual():
    """For L = 1/2 |seis - data|^2, psi.grad is kernel_psi of the reference pipeline run with
    the same residual as adjoint source (summed over the batch)."""
    from sparc_flows_gb300.autograd import seismograms
    from sparc_flows_gb300.pipeline import FwdAdjKernels, receiver_columns
    run = RunConfig(nx=128, nz=300, xlength_cm=200e8, nsteps=91, flows=True)
    model = M.polytrope(300)
    A = M.psi_amplitude_for_peak(run, model, 240.0)
    psi_true = torch.as_tensor(M.gaussian_psi(run, model, A), device="cuda")
    rcv = receiver_columns(run, n=32, x0=-62.0, dx=4.0)
    specs = [M.SourceSpec(-20.0), M.SourceSpec(25.0)]
    pipe = FwdAdjKernels(run, model, specs, psi=np.zeros((300, 128)), precision=64, receivers=rcv)
    with torch.no_grad():
        data = seismograms(psi_true, pipe).clone()
    psi = (0.5 * psi_true).clone().requires_grad_(True)
    loss = 0.5 * ((seismograms(psi, pipe) - data) ** 2).sum()
    loss.backward()
    # the same through the pipeline: residual at the receivers as the data difference
    pipe.fwd.update_flow(psi.detach())
    pipe.adj.update_flow(psi.detach())
    full = torch.zeros((len(specs), run.nrec, run.nx), dtype=torch.float64, device="cuda")
    full[:, :, pipe.rcv_t] = data  # only the receiver columns enter the adjoint source
    pipe.forward()
    pipe.adjoint(pipe.adjoint_source(full))
    ref = pipe.final_kernels(summed=True)["kernel_psi"][0]
    pipe.close()
    g = psi.grad
    assert torch.isfinite(g).all() and g.abs().max() > 0
    assert (torch.linalg.vector_norm(g - ref) / torch.linalg.vector_norm(ref)).item() < 1e-12
