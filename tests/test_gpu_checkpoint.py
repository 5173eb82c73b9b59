"""Forward field checkpointed in HBM and recomputed per segment during the adjoint run: the
seismograms and the accumulated kernel integrands equal those of the run that keeps every
partial state (all_modules.f90:750-784, kernels.f90:209-358), bit for bit."""
import numpy as np
import pytest
import torch

from sparc_flows_gb300 import model as M
from sparc_flows_gb300.config import RunConfig
from sparc_flows_gb300.pipeline import FwdAdjKernels

pytestmark = pytest.mark.gpu


def _case():
    # 226 steps: records 0 .. 15 at steps_out = 15, the last segment shorter than the others
    run = RunConfig(nx=128, nz=300, xlength_cm=200e8, nsteps=226, flows=True)
    model = M.polytrope(300)
    psi = M.gaussian_psi(run, model, M.psi_amplitude_for_peak(run, model, 240.0))
    specs = [M.SourceSpec(-20.0), M.SourceSpec(15.0)]
    return run, model, psi, M.c_bump(run, model), specs


@pytest.mark.parametrize("precision,every", [(64, 4), (64, 5), (32, 3), (32, 15)])
def test_checkpointed_kernels_equal_stored(precision, every):
    run, model, psi, cmul, specs = _case()
    ref = FwdAdjKernels(run, model, specs, psi=psi, cmul=cmul, precision=precision)
    seis_r, kacc_r = (t.cpu().numpy() for t in ref.run_all())
    ref.close()
    ck = FwdAdjKernels(run, model, specs, psi=psi, cmul=cmul, precision=precision, checkpoint_every=every)
    assert ck.snaps.shape[1] == every
    seis_c, kacc_c = (t.cpu().numpy() for t in ck.run_all())
    ck.close()
    assert np.abs(kacc_r).max() > 0
    assert np.array_equal(seis_c, seis_r)
    assert np.array_equal(kacc_c, kacc_r)


def test_record_window_matches_full_records():
    """sparc_forward_window writes records rec0 .. rec0 + cap - 1 to slots 0 .. cap - 1."""
    from sparc_flows_gb300.solver import WaveSolver
    run, model, psi, cmul, specs = _case()
    ws = WaveSolver(run, model, nbatch=1, precision=64, psi=psi, cmul=cmul)
    ws.set_forward_sources(specs[:1])
    seis, snaps = ws.forward(snapshots=True)
    win = torch.zeros_like(snaps[:, :4])
    ws.reset(0)
    ws.run_steps(run.nsteps, None, win, 4, rec0=6)
    assert torch.equal(win, snaps[:, 6:10])
    ws.close()


def test_bad_checkpoint_interval():
    run, model, psi, cmul, specs = _case()
    with pytest.raises(ValueError):
        FwdAdjKernels(run, model, specs[:1], psi=psi, cmul=cmul, precision=64, checkpoint_every=16)
