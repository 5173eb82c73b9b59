"""The sparc drop-in end to end: params.i, master.pixels, Instruction files and model file in a
working directory; forward (Spectral), adjoint (Adjoint) and kernel stage (no instruction file)
produce the reference's output files, and the kernels equal the in-memory pipeline's."""
import os
import shutil
import subprocess
import sys

import numpy as np
import pytest

from sparc_flows_gb300 import fits
from sparc_flows_gb300 import model as M

pytestmark = pytest.mark.gpu

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))

PARAMS = """\
integer nx, ny, nz
parameter (nx = 128, ny = 1, nz = 300)
real(kind=real64) xlength, ylength, timestep
parameter (xlength = 200.0 * 10**(8), ylength = xlength, timestep = 2.0)
character (LEN = *), PARAMETER :: file_data = 'polytrope_gen'
character (LEN = *), PARAMETER :: directory = '{dir}/'
real(kind=real64) cadforcing
parameter( cadforcing = 30.0)
logical, parameter :: FLOWS = .True.
integer npmlhor
parameter (npmlhor = 9)
integer npmltop, npmlbot,nzpml
parameter(npmlbot = 10, npmltop = 10, nzpml = (npmlbot + npmltop))
real(kind=real64) solartime
parameter (solartime = 4.0)
real(kind=real64) obsheight
parameter (obsheight = 20000000.0)
real(kind=real64) outputcad
parameter (outputcad = 30.0)
real(kind=real64) excitdep
parameter( excitdep = - 15000000.0)
"""


def run_sparc(cwd, nn, mm, env):
    cmd = [os.path.join(ROOT, "sparc_flows_gb300", "bin", "mpiexec"), "-np", "1",
           sys.executable, os.path.join(ROOT, "sparc_flows_gb300", "bin", "sparc"), nn, mm]
    return subprocess.run(cmd, cwd=cwd, env=env, capture_output=True, text=True)


def test_forward_adjoint_kernel_files(tmp_path):
    code = tmp_path / "code"
    data = tmp_path / "data_dir"
    code.mkdir()
    data.mkdir()
    (code / "params.i").write_text(PARAMS.format(dir=str(data)))
    np.savetxt(code / "polytrope_gen", M.polytrope(300), fmt="%.17e")
    (data / "master.pixels").write_text("-10.0\n15.0\n")
    from sparc_flows_gb300.config import RunConfig
    run = RunConfig(nx=128, nz=300, xlength_cm=200e8, nsteps=46)
    psi = M.gaussian_psi(run, M.polytrope(300), 0.05)
    fits.write(str(data / "model_psi_ls00.fits"), psi[:, None, :])
    env = dict(os.environ, SPARC_NSTEPS="46", SPARC_PRECISION="64")
    shutil.copy(os.path.join(ROOT, "tests", "golden", "Spectral"), code / "Instruction_src02_ls00")
    r = run_sparc(code, "02", "00", env)
    assert r.returncode == 0, r.stderr
    fdir = data / "forward_src02_ls00"
    vz = fits.read(str(fdir / "vz_cc.fits"))
    assert vz.shape == (4, 1, 128) and np.abs(vz).max() > 0
    assert not (code / "Instruction_src02_ls00").exists()
    assert (data / "adjoint_src02" / "source.fits").exists()
    shutil.copy(os.path.join(ROOT, "tests", "golden", "Adjoint"), code / "Instruction_src02_ls00")
    r = run_sparc(code, "02", "00", env)
    assert r.returncode == 0, r.stderr
    os.remove(code / "Instruction_src02_ls00")
    r = run_sparc(code, "02", "00", env)
    assert r.returncode == 0, r.stderr
    for name in ("kernel_c", "kernel_vx", "kernel_vz", "kernel_psi", "hessian"):
        k = fits.read(str(data / "kernel" / f"{name}_02.fits"))
        assert k.shape == (300, 1, 128) and np.all(np.isfinite(k)), name
    assert np.abs(fits.read(str(data / "kernel" / "kernel_c_02.fits"))).max() > 0
    assert not (fdir / "partial_states.npy").exists()


def test_unknown_source_fails_with_nonzero_status(tmp_path):
    code = tmp_path / "code"
    data = tmp_path / "d"
    code.mkdir()
    data.mkdir()
    (code / "params.i").write_text(PARAMS.format(dir=str(data)))
    np.savetxt(code / "polytrope_gen", M.polytrope(300), fmt="%.17e")
    (data / "master.pixels").write_text("0.0\n")
    shutil.copy(os.path.join(ROOT, "tests", "golden", "Spectral"), code / "Instruction_src05_ls00")
    r = run_sparc(code, "05", "00", dict(os.environ, SPARC_NSTEPS="16"))
    assert r.returncode != 0
