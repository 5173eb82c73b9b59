"""The sparc file contract on the host: params.i parsing against golden values produced by the
reference's own read_params.py, FITS round trips, instruction-file parsing and maxtime."""
import json
import os

import numpy as np

from sparc_flows_gb300 import fits
from sparc_flows_gb300.config import parse_params_i, reference_maxtime, run_config_from_params
from sparc_flows_gb300.cli import _read_instruction

GOLD = json.load(open(os.path.join(os.path.dirname(__file__), "golden", "params_reference.json")))


def test_params_i_matches_reference_parser():
    p = parse_params_i(GOLD["params_i"])
    assert p["nx"] == GOLD["get_nx"] and p["nz"] == GOLD["get_nz"]
    assert p["xlength"] == GOLD["get_xlength"] * 1e8          # read_params returns Mm
    assert p["outputcad"] == GOLD["get_dt"]
    assert p["timestep"] == GOLD["get_dt_simulation"]
    assert p["solartime"] == GOLD["get_total_simulation_time"]
    assert p["file_data"] == GOLD["get_solarmodel"]
    assert p["excitdep"] == GOLD["get_excitedepth"]
    assert p["obsheight"] == GOLD["get_obs_depth"]
    assert p["directory"].rstrip("/") == GOLD["get_directory"]
    assert p["npmlbot"] == 10 and p["npmltop"] == 10 and p["npmlhor"] == 9
    assert p["flows"] is True and p["magnetic"] is False


def test_run_config_from_reference_params():
    p = parse_params_i(GOLD["params_i"])
    rc = run_config_from_params(p)
    nupeak = float(np.float32(0.0017))
    maxtime = reference_maxtime(4.0, 2.0, 30.0, nupeak)
    # floor((4*3600 + 2/0.0017)/2) + 2 rounded down to a multiple of 15 (initialize.f90:998-1000)
    assert maxtime == 15 * ((int((4 * 3600 + 2 / nupeak) / 2) + 2) // 15)
    assert rc.nsteps == maxtime + 1 and rc.steps_out == 15 and rc.nx == 512


def test_fits_round_trip(tmp_path):
    a = np.random.default_rng(0).standard_normal((7, 1, 33))
    p = str(tmp_path / "x.fits")
    fits.write(p, a, time=12)
    raw = open(p, "rb").read()
    assert len(raw) % 2880 == 0 and b"BITPIX  =                  -64" in raw
    assert b"NAXIS1  =                   33" in raw and b"NAXIS3  =                    7" in raw
    assert np.array_equal(fits.read(p), a)


def test_instruction_files(tmp_path):
    for name, kind in (("Spectral", "spectral"), ("Adjoint", "adjoint")):
        f = tmp_path / name
        f.write_text(f"{kind}\n2D\n" + ("T\n" if kind == "spectral" else ""))
        k, twod = _read_instruction(str(f))
        assert k == kind and twod


def test_cli_refuses_3d_instruction(tmp_path, monkeypatch):
    """An instruction without the '2D' line selects option 16 (initialize.f90:833-837, 1094); with
    ny > 1 the executable exits with status 2 before touching a model file or the GPU."""
    from sparc_flows_gb300 import cli
    text = GOLD["params_i"].replace("ny = 1", "ny = 64")
    assert text != GOLD["params_i"]
    (tmp_path / "params.i").write_text(text)
    (tmp_path / "Instruction_src01_ls00").write_text("spectral\n3D\n")
    monkeypatch.chdir(tmp_path)
    assert cli.main(["01", "00"]) == 2
    assert (tmp_path / "Instruction_src01_ls00").exists()
