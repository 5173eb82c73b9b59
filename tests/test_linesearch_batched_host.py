"""linesearch_batched's orchestration on the host, the GPU solver replaced by a stand-in: one
solve per (source, trial model) pair with the pair's own stream function, each pair's records in
forward_srcNN_lsMM, trial models counted as linesearch.py counts them."""
import numpy as np

from sparc_flows_gb300 import fits, linesearch_batched
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


class FakeSolver:
    """Stands in for WaveSolver: solve b's records are b + 1 everywhere."""
    last = None

    def __init__(self, run, model, nbatch=1, precision=64, psi=None, device="cpu", **kw):
        self.run, self.nb, self.psi = run, nbatch, psi
        FakeSolver.last = self

    def set_forward_sources(self, specs):
        self.xlocs = [s.xloc for s in specs]

    def forward(self):
        import torch
        return torch.stack([torch.full((self.run.nrec, self.run.nx), float(b + 1)) for b in range(self.nb)])

    def close(self):
        pass


def test_pairs_models_and_files(tmp_path, monkeypatch):
    code, data = tmp_path / "code", tmp_path / "data_dir"
    code.mkdir()
    data.mkdir()
    (code / "params.i").write_text(PARAMS.format(dir=str(data)))
    np.savetxt(code / "polytrope_gen", M.polytrope(300), fmt="%.17e")
    (data / "master.pixels").write_text("-10.0\n15.0\n")
    for m in (1, 2):
        (data / f"forward_src01_ls{m:02d}").mkdir()
        fits.write(str(data / f"model_psi_ls{m:02d}.fits"), np.full((300, 1, 64), float(m)))
    (code / "linesearch").write_text("")
    monkeypatch.chdir(code)
    monkeypatch.setenv("SPARC_NSTEPS", "46")
    monkeypatch.setenv("SPARC_ADJOINT_SOURCE", "waveform")
    import sparc_flows_gb300.solver as S
    monkeypatch.setattr(S, "WaveSolver", FakeSolver)
    assert linesearch_batched.main([]) == 0
    fake = FakeSolver.last
    pairs = [(s, m) for m in (1, 2) for s in (1, 2)]
    assert fake.nb == 4 and fake.xlocs == [-10.0, 15.0, -10.0, 15.0]
    for b, (s, m) in enumerate(pairs):
        assert np.all(fake.psi[b] == m)
        rec = fits.read(str(data / f"forward_src{s:02d}_ls{m:02d}" / "vz_cc.fits"))
        assert rec.shape == (4, 1, 64) and np.all(rec == b + 1)
    assert not (data / "forward_src01_ls03").exists()
