"""full_batched on two ranks (gloo, CPU), the GPU pipeline replaced by a stand-in: the sources of
master.pixels are split between the ranks with none lost or repeated, every source's files are
written by the rank that ran it, and the kernel sums over all sources (grad.py:188-196: kernel_psi
and |hessian|) reach every rank and rank 0's kernel/*_sum.fits."""
import os
import socket

import numpy as np
import torch.distributed as dist
import torch.multiprocessing as mp

from sparc_flows_gb300 import fits
from sparc_flows_gb300 import model as M

PARAMS = """\
integer nx, ny, nz
parameter (nx = 64, ny = 1, nz = 300)
real(kind=real64) xlength, ylength, timestep
parameter (xlength = 200.0 * 10**(8), ylength = xlength, timestep = 2.0)
character (LEN = *), PARAMETER :: file_data = 'polytrope_gen'
character (LEN = *), PARAMETER :: directory = '{dir}/'
logical, parameter :: FLOWS = .True.
"""
XLOCS = (-10.0, 15.0, 30.0)


class FakePipe:
    """Stands in for FwdAdjKernels: a source's records and kernels are functions of its position."""

    def __init__(self, run, model, specs, **kw):
        import torch
        self.run, self.nb, self.dev = run, len(specs), torch.device("cpu")
        self.xlocs = [s.xloc for s in specs]

    def forward(self):
        import torch
        return torch.stack([torch.full((self.run.nrec, self.run.nx), x) for x in self.xlocs])

    def adjoint(self, src):
        self.src = src

    def final_kernels(self, summed=False):
        import torch
        vals = torch.tensor(self.xlocs, dtype=torch.float64)[:, None, None] + 100.0
        out = {k: vals.expand(self.nb, self.run.nz, self.run.nx).clone()
               for k in ("kernel_c", "kernel_vx", "kernel_vz", "kernel_psi")}
        out["hessian"] = -out["kernel_psi"]  # grad.py sums |hessian|
        return out

    def close(self):
        pass


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def _worker(rank, world, port, code, out):
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port), SPARC_NSTEPS="46",
                      SPARC_ADJOINT_SOURCE="waveform")
    os.chdir(code)
    import sparc_flows_gb300.pipeline as P
    from sparc_flows_gb300 import full_batched
    P.FwdAdjKernels = FakePipe
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        tot = full_batched.run_iteration(None, "00", rank, world)
        out[rank] = {k: float(v.mean()) for k, v in tot.items()}
    finally:
        dist.destroy_process_group()


def test_sources_sharded_over_two_ranks(tmp_path):
    code, data = tmp_path / "code", tmp_path / "data_dir"
    code.mkdir()
    data.mkdir()
    (code / "params.i").write_text(PARAMS.format(dir=str(data)))
    np.savetxt(code / "polytrope_gen", M.polytrope(300), fmt="%.17e")
    (data / "master.pixels").write_text("".join(f"{x}\n" for x in XLOCS))
    world = 2
    out = mp.get_context("spawn").Manager().dict()
    mp.start_processes(_worker, args=(world, _free_port(), str(code), out), nprocs=world, start_method="spawn")
    want = sum(x + 100.0 for x in XLOCS)
    for r in range(world):
        assert abs(out[r]["kernel_psi"] - want) < 1e-9 and abs(out[r]["hessian"] - want) < 1e-9
    for s, x in enumerate(XLOCS, start=1):  # each source's files, whichever rank ran it
        rec = fits.read(str(data / f"forward_src{s:02d}_ls00" / "vz_cc.fits"))
        assert np.all(rec == x)
        assert np.all(fits.read(str(data / "kernel" / f"kernel_psi_{s:02d}.fits")) == x + 100.0)
    for name in ("kernel_psi", "hessian"):
        assert np.allclose(fits.read(str(data / "kernel" / f"{name}_sum.fits")), want)
