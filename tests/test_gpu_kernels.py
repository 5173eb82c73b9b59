"""Sensitivity kernels: GPU forward + adjoint + in-HBM kernel integral against the oracle's
restatement of the reference's three sparc runs (forward, adjoint, PRODUCE_KERNELS)."""
import numpy as np
import pytest

from oracle import oracle as O
from sparc_flows_gb300 import model as M
from sparc_flows_gb300.config import RunConfig

pytestmark = pytest.mark.gpu


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


@pytest.fixture(scope="module")
def kernel_case():
    run = RunConfig(nx=128, nz=300, xlength_cm=200e8, nsteps=91, flows=True)
    model = M.polytrope(300)
    psi = M.gaussian_psi(run, model, M.psi_amplitude_for_peak(run, model, 240.0))
    cmul = M.c_bump(run, model)
    spec = M.SourceSpec(-20.0)
    # oracle: forward with partial states, adjoint driven by the time-reversed seismogram at receivers
    fw = O.OracleSim(run, model, cmul=cmul)
    fw.set_psi(psi)
    fw.set_forward_source(spec.xloc, spec.spatial, spec.sigma, spec.temporal, spec.nu0, run.nsteps + 8)
    seis_o, fsn = fw.run_steps(run.nsteps, snapshots=True)
    from sparc_flows_gb300.pipeline import receiver_columns
    rcv = receiver_columns(run, n=32, x0=-62.0, dx=4.0)
    src = np.zeros_like(seis_o)
    src[:, rcv] = seis_o[::-1][:, rcv]
    arun = run.replace(adjoint=True)
    ad = O.OracleSim(arun, model, cmul=cmul)
    ad.set_psi(psi)
    ad.set_adjoint_source(src, arun.num_steps)
    _, asn = ad.run_steps(run.nsteps, snapshots=True)
    ker = fw.kernels(fsn, asn)
    fw.close()
    ad.close()
    return run, model, psi, cmul, spec, rcv, seis_o, ker


# FP32: the metric's own bound, 1e-4 rel-L2 against the FP64 restatement
@pytest.mark.parametrize("precision,tol", [(64, 1e-9), (32, 1e-4)])
def test_kernels_match_oracle(kernel_case, precision, tol):
    from sparc_flows_gb300.pipeline import FwdAdjKernels
    run, model, psi, cmul, spec, rcv, seis_o, ker = kernel_case
    pipe = FwdAdjKernels(run, model, [spec], psi=psi, cmul=cmul, precision=precision, receivers=rcv)
    seis, _ = pipe.run_all()
    assert rel_l2(seis.cpu().numpy()[0], seis_o) < (1e-10 if precision == 64 else 1e-4)
    got = {k: v.cpu().numpy()[0] for k, v in pipe.final_kernels(summed=False).items()}
    pipe.close()
    errs = {name: rel_l2(got[name], ker[name]) for name in ("kernel_c", "kernel_vx", "kernel_vz", "kernel_psi", "hessian")}
    for name in errs:
        assert np.abs(ker[name]).max() > 0, name
        assert errs[name] < tol, (name, errs)
