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
    # the waveform adjoint source: no params.<pord> files, so the travel-time source would be zero
    env = dict(os.environ, SPARC_NSTEPS="46", SPARC_PRECISION="64", SPARC_ADJOINT_SOURCE="waveform")
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


def test_partial_states_as_reference_fits_files(tmp_path):
    """SPARC_PARTIAL_FITS=1: forward and adjoint runs write the reference's *_partial.fits files
    (xix, xiz, vx, vz, acc_x, acc_z per record; v and acc only for the adjoint), the kernel stage
    reads them and gives the kernels of the array-file path, then removes them."""
    outs = {}
    for mode in ("0", "1"):
        code = tmp_path / f"code{mode}"
        data = tmp_path / f"data{mode}"
        code.mkdir()
        data.mkdir()
        (code / "params.i").write_text(PARAMS.format(dir=str(data)))
        np.savetxt(code / "polytrope_gen", M.polytrope(300), fmt="%.17e")
        (data / "master.pixels").write_text("-10.0\n15.0\n")
        env = dict(os.environ, SPARC_NSTEPS="46", SPARC_PRECISION="64", SPARC_ADJOINT_SOURCE="waveform",
                   SPARC_PARTIAL_FITS=mode)
        shutil.copy(os.path.join(ROOT, "tests", "golden", "Spectral"), code / "Instruction_src01_ls00")
        assert run_sparc(code, "01", "00", env).returncode == 0
        shutil.copy(os.path.join(ROOT, "tests", "golden", "Adjoint"), code / "Instruction_src01_ls00")
        assert run_sparc(code, "01", "00", env).returncode == 0
        fdir, adir = data / "forward_src01_ls00", data / "adjoint_src01"
        if mode == "1":
            assert sorted(f for f in os.listdir(fdir) if f.endswith("_000015_partial.fits")) == [
                "acc_x_000015_partial.fits", "acc_z_000015_partial.fits", "vx_000015_partial.fits",
                "vz_000015_partial.fits", "xix_000015_partial.fits", "xiz_000015_partial.fits"]
            assert not (adir / "xix_000015_partial.fits").exists() and (adir / "vx_000015_partial.fits").exists()
            assert fits.read(str(fdir / "vz_000030_partial.fits")).shape == (300, 1, 128)
        os.remove(code / "Instruction_src01_ls00")
        r = run_sparc(code, "01", "00", env)
        assert r.returncode == 0, r.stderr
        assert not any(f.endswith("_partial.fits") for f in os.listdir(fdir))
        outs[mode] = {n: fits.read(str(data / "kernel" / f"{n}_01.fits")) for n in ("kernel_c", "kernel_psi", "hessian")}
    for n in outs["0"]:
        assert np.array_equal(outs["0"][n], outs["1"][n]), n


def test_forward_writes_the_travel_time_adjoint_source(tmp_path):
    """A forward run with params.0 present measures f-mode travel times (ADJOINT_SOURCE_FILT):
    ttdiff.0, windows.0, adjoint_src02/{source.fits, information}, kernel/misfit_02_00."""
    code = tmp_path / "code"
    data = tmp_path / "data_dir"
    code.mkdir()
    (data / "data").mkdir(parents=True)
    (code / "params.i").write_text(PARAMS.format(dir=str(data)))
    np.savetxt(code / "polytrope_gen", M.polytrope(300), fmt="%.17e")
    (data / "master.pixels").write_text("-10.0\n15.0\n")
    (data / "params.0").write_text("3.0\n9.0\n6.0\n")
    nsteps = 601
    env = dict(os.environ, SPARC_NSTEPS=str(nsteps), SPARC_PRECISION="64")
    # observed data: the synthetic of a run with the source 0.4 Mm further away
    (data / "master.pixels").write_text("-10.0\n15.4\n")
    open(code / "compute_data", "w").close()
    shutil.copy(os.path.join(ROOT, "tests", "golden", "Spectral"), code / "Instruction_src02_ls00")
    assert run_sparc(code, "02", "00", env).returncode == 0
    os.remove(code / "compute_data")
    shutil.copy(data / "forward_src02_ls00" / "vz_cc.fits", data / "data" / "02.fits")
    (data / "master.pixels").write_text("-10.0\n15.0\n")
    shutil.copy(os.path.join(ROOT, "tests", "golden", "Spectral"), code / "Instruction_src02_ls00")
    r = run_sparc(code, "02", "00", env)
    assert r.returncode == 0, r.stderr
    rows = np.loadtxt(data / "forward_src02_ls00" / "ttdiff.0", ndmin=2)
    assert rows.shape[1] == 7 and rows.shape[0] > 0 and np.isfinite(rows[:, 1]).all()
    win = np.loadtxt(data / "forward_src02_ls00" / "windows.0", ndmin=2)
    assert win.shape == (rows.shape[0], 2)
    src = fits.read(str(data / "adjoint_src02" / "source.fits"))
    assert src.shape == (nsteps // 15 + 1, 1, 128) and np.isfinite(src).all() and np.abs(src).max() > 0
    info = (data / "adjoint_src02" / "information").read_text().split()
    assert int(info[0]) == nsteps // 15 + 1 and info[-1] == "2D"
    mis = np.loadtxt(data / "kernel" / "misfit_02_00")
    assert int(mis[0]) == 2 and int(mis[1]) == rows.shape[0] and mis[2] > 0
    lines = (data / "kernel" / "misfit_all_02_00").read_text().splitlines()
    assert len(lines) == 9 and lines[0].split()[:2] == ["#", "2"]
    assert all((data / "forward_src02_ls00" / f"windows.all.00.{fb}").exists() for fb in (1, 2, 3))


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


def test_batched_iteration_equals_per_source_runs(tmp_path, monkeypatch):
    """full_batched (all sources in one FwdAdjKernels batch) writes the same records and kernel
    files as the three sparc runs per source that full.py makes (full.py:18-59)."""
    from sparc_flows_gb300 import cli, full_batched
    from sparc_flows_gb300.config import RunConfig
    code = tmp_path / "code"
    data = tmp_path / "data_dir"
    code.mkdir()
    data.mkdir()
    (code / "params.i").write_text(PARAMS.format(dir=str(data)))
    np.savetxt(code / "polytrope_gen", M.polytrope(300), fmt="%.17e")
    (data / "master.pixels").write_text("-10.0\n15.0\n")
    run = RunConfig(nx=128, nz=300, xlength_cm=200e8, nsteps=46)
    fits.write(str(data / "model_psi_ls00.fits"), M.gaussian_psi(run, M.polytrope(300), 0.05)[:, None, :])
    monkeypatch.chdir(code)
    for k, v in dict(SPARC_NSTEPS="46", SPARC_PRECISION="64", SPARC_ADJOINT_SOURCE="waveform").items():
        monkeypatch.setenv(k, v)
    names = ("kernel_c", "kernel_vx", "kernel_vz", "kernel_psi", "hessian")
    for nn in ("01", "02"):  # forward, adjoint, kernel stage per source
        for instr in ("Spectral", "Adjoint", None):
            if instr:
                shutil.copy(os.path.join(ROOT, "tests", "golden", instr), code / f"Instruction_src{nn}_ls00")
            assert cli.main([nn, "00"]) == 0
            if instr == "Adjoint":
                os.remove(code / f"Instruction_src{nn}_ls00")
    per = {(nn, n): fits.read(str(data / "kernel" / f"{n}_{nn}.fits")) for nn in ("01", "02") for n in names}
    vz = {nn: fits.read(str(data / f"forward_src{nn}_ls00" / "vz_cc.fits")) for nn in ("01", "02")}
    shutil.rmtree(data / "kernel")
    assert full_batched.main([]) == 0
    for nn in ("01", "02"):
        assert np.array_equal(fits.read(str(data / f"forward_src{nn}_ls00" / "vz_cc.fits")), vz[nn])
        for n in names:
            got = fits.read(str(data / "kernel" / f"{n}_{nn}.fits"))
            assert np.abs(per[(nn, n)]).max() > 0
            assert np.allclose(got, per[(nn, n)], rtol=1e-12, atol=1e-12 * np.abs(per[(nn, n)]).max()), (nn, n)
