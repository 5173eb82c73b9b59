"""full_batched's orchestration on the host, the GPU pipeline replaced by a stand-in: every
source's records go to its own forward_srcNN_lsMM files, the adjoint run receives each source's
adjoint_srcNN/source.fits in source order, and each source's kernels land in kernel/*_NN.fits."""
import os

import numpy as np

from sparc_flows_gb300 import fits, full_batched
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


class FakePipe:
    """Stands in for FwdAdjKernels: source b's records are b + 1 everywhere, its kernels b + 10."""
    last = None

    def __init__(self, run, model, specs, **kw):
        import torch
        self.run, self.nb, self.dev = run, len(specs), torch.device("cpu")
        self.xlocs = [s.xloc for s in specs]
        FakePipe.last = self

    def forward(self):
        import torch
        nrec = self.run.nrec
        return torch.stack([torch.full((nrec, self.run.nx), float(b + 1)) for b in range(self.nb)])

    def adjoint(self, src):
        self.src = src.cpu().numpy()

    def final_kernels(self, summed=False):
        import torch
        shape = (self.nb, self.run.nz, self.run.nx)
        vals = torch.arange(self.nb, dtype=torch.float64)[:, None, None] + 10.0
        return {k: vals.expand(shape) for k in ("kernel_c", "kernel_vx", "kernel_vz", "kernel_psi", "hessian")}

    def close(self):
        pass


def test_files_per_source(tmp_path, monkeypatch):
    code, data = tmp_path / "code", tmp_path / "data_dir"
    code.mkdir()
    data.mkdir()
    (code / "params.i").write_text(PARAMS.format(dir=str(data)))
    np.savetxt(code / "polytrope_gen", M.polytrope(300), fmt="%.17e")
    (data / "master.pixels").write_text("-10.0\n15.0\n30.0\n")
    monkeypatch.chdir(code)
    monkeypatch.setenv("SPARC_NSTEPS", "46")
    monkeypatch.setenv("SPARC_ADJOINT_SOURCE", "waveform")
    import sparc_flows_gb300.pipeline as P
    monkeypatch.setattr(P, "FwdAdjKernels", FakePipe)
    assert full_batched.main(["--sources", "1,3"]) == 0
    fake = FakePipe.last
    assert fake.xlocs == [-10.0, 30.0]
    for b, nn in enumerate(("01", "03")):
        rec = fits.read(str(data / f"forward_src{nn}_ls00" / "vz_cc.fits"))
        assert rec.shape == (4, 1, 64) and np.all(rec == b + 1)
        src = fits.read(str(data / f"adjoint_src{nn}" / "source.fits")).reshape(-1, 64)
        assert np.array_equal(fake.src[b][: src.shape[0]], src[: fake.src.shape[1]])
        assert np.all(fits.read(str(data / "kernel" / f"kernel_c_{nn}.fits")) == b + 10)
        assert (data / f"adjoint_src{nn}" / "kernel_info").exists()
    assert not (data / "forward_src02_ls00").exists()
