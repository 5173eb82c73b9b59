"""sparc_kernels_accumulate_static: the kernel-integral accumulation for callers that must not
see the library call cudaMalloc mid-run (an embedding host whose allocator owns all device
memory, or a run with a device-memory budget fixed before it starts).  It
must give the same sums as sparc_kernels_accumulate, whose work buffer is allocated on first
use, call after call.  Runs alone in a fresh process or after the rest of the suite."""
import ctypes

import numpy as np
import pytest

from sparc_flows_gb300 import model as M
from sparc_flows_gb300.config import RunConfig

pytestmark = pytest.mark.gpu

TOL = 1e-12  # both paths run the same kernels; only the scratch location differs


def _accumulate(lib_fn, ws, snaps, jf, out):
    import torch
    from sparc_flows_gb300 import capi
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = lib_fn(ws.plan, ctypes.c_void_p(snaps.data_ptr()), snaps.shape[1], jf, ctypes.c_void_p(out.data_ptr()),
                stream)
    capi.check(rc, lib_fn.__name__)


@pytest.mark.parametrize("precision", [32, 64])
def test_static_scratch_matches_allocating_path(precision):
    import torch
    from sparc_flows_gb300 import capi
    from sparc_flows_gb300.solver import WaveSolver

    run = RunConfig(nx=128, nz=300, xlength_cm=200e8, nsteps=46, flows=True)
    model = M.polytrope(300)
    psi = M.gaussian_psi(run, model, M.psi_amplitude_for_peak(run, model, 240.0))
    ws = WaveSolver(run, model, nbatch=2, precision=precision, psi=psi, cmul=M.c_bump(run, model))
    ws.set_forward_sources([M.SourceSpec(-15.0), M.SourceSpec(25.0)])
    _, snaps = ws.forward(snapshots=True)          # the solver's final state plays the adjoint
    L = capi.lib()
    out_a = torch.zeros((2, 4, run.nz, run.nx), dtype=torch.float64, device="cuda")
    out_b = torch.zeros_like(out_a)
    for jf in (snaps.shape[1] - 1, 0):             # two calls in a row, accumulating
        _accumulate(L.sparc_kernels_accumulate, ws, snaps, jf, out_a)
        _accumulate(L.sparc_kernels_accumulate_static, ws, snaps, jf, out_b)
        torch.cuda.synchronize()
        a, b = out_a.cpu().numpy(), out_b.cpu().numpy()
        assert np.abs(a).max() > 0
        for f in range(4):
            assert np.linalg.norm(b[:, f] - a[:, f]) <= TOL * max(np.linalg.norm(a[:, f]), 1e-300), (jf, f)
    ws.close()


def test_static_scratch_rejects_oversize_batch():
    from sparc_flows_gb300 import capi
    from sparc_flows_gb300.solver import WaveSolver
    import torch

    # 4 * 300 * 1024 * 8 bytes * 2 solves = 19.7 MB > 8 MiB
    run = RunConfig(nx=1024, nz=300, xlength_cm=400e8, nsteps=16, flows=False)
    ws = WaveSolver(run, M.polytrope(300), nbatch=2, precision=64)
    ws.set_forward_sources([M.SourceSpec(0.0), M.SourceSpec(10.0)])
    _, snaps = ws.forward(nsteps=1, snapshots=True)
    out = torch.zeros((2, 4, run.nz, run.nx), dtype=torch.float64, device="cuda")
    with pytest.raises(capi.SparcError, match="8 MiB"):
        _accumulate(capi.lib().sparc_kernels_accumulate_static, ws, snaps, 0, out)
    ws.close()
