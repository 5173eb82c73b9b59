"""linesearch_batched on the GPU: every (source, trial model) pair of a line search as one solve of
a single batch with per-solve stream functions (linesearch.py:39-56 runs one sparc process per
pair); each pair's forward_srcNN_lsMM/vz_cc.fits must equal the records of that pair solved
alone."""
import numpy as np
import pytest

from sparc_flows_gb300 import fits
from sparc_flows_gb300 import model as M

pytestmark = pytest.mark.gpu

PARAMS = """\
integer nx, ny, nz
parameter (nx = 128, ny = 1, nz = 300)
real(kind=real64) xlength, ylength, timestep
parameter (xlength = 200.0 * 10**(8), ylength = xlength, timestep = 2.0)
character (LEN = *), PARAMETER :: file_data = 'polytrope_gen'
character (LEN = *), PARAMETER :: directory = '{dir}/'
logical, parameter :: FLOWS = .True.
"""


def test_batched_pairs_equal_single_runs(tmp_path, monkeypatch):
    from sparc_flows_gb300 import cli, linesearch_batched
    from sparc_flows_gb300.config import parse_params_i, run_config_from_params
    from sparc_flows_gb300.solver import WaveSolver

    code, data = tmp_path / "code", tmp_path / "data_dir"
    code.mkdir()
    data.mkdir()
    (code / "params.i").write_text(PARAMS.format(dir=str(data)))
    model = M.polytrope(300)
    np.savetxt(code / "polytrope_gen", model, fmt="%.17e")
    (data / "master.pixels").write_text("-30.0\n20.0\n")
    run = run_config_from_params(parse_params_i((code / "params.i").read_text())).replace(nsteps=61)
    unit = M.gaussian_psi(run, model, M.psi_amplitude_for_peak(run, model, 1.0))
    for m, vpeak in ((1, 200.0), (2, 80.0)):
        (data / f"forward_src01_ls{m:02d}").mkdir()
        fits.write(str(data / f"model_psi_ls{m:02d}.fits"), (unit * vpeak)[:, None, :])
    (code / "linesearch").write_text("")
    monkeypatch.chdir(code)
    monkeypatch.setenv("SPARC_NSTEPS", str(run.nsteps))
    monkeypatch.setenv("SPARC_ADJOINT_SOURCE", "waveform")
    monkeypatch.setenv("SPARC_PRECISION", "64")
    assert linesearch_batched.main([]) == 0
    recs = {}
    for m in (1, 2):
        psi = cli._flow_inputs(run, str(data) + "/", f"{m:02d}", False)[0]
        for s, x in ((1, -30.0), (2, 20.0)):
            ws = WaveSolver(run, model, nbatch=1, precision=64, psi=psi)
            ws.set_forward_sources([M.SourceSpec(x, M.SPATIAL_REFERENCE, 0.5, M.TEMPORAL_REFERENCE, 0.003)])
            one = ws.forward().cpu().numpy()[0]
            ws.close()
            got = fits.read(str(data / f"forward_src{s:02d}_ls{m:02d}" / "vz_cc.fits")).reshape(one.shape)
            assert np.abs(one).max() > 0
            assert np.linalg.norm(got - one) <= 1e-12 * np.linalg.norm(one), (s, m)
            recs[(s, m)] = got
    # the trial models really differ
    assert np.linalg.norm(recs[(1, 1)] - recs[(1, 2)]) > 1e-6 * np.linalg.norm(recs[(1, 1)])
