"""``sparc NN MM`` drop-in for the reference executable (driver.f90:1-331, READ_PARAMETERS
initialize.f90:984-1144), backed by the GPU solver.

Callers (data_forward.py:15-18, full.py:18-59, linesearch.py:16-19) run
``mpiexec -np 1 ./sparc NN MM`` in the code directory and check the exit status.  The mode is
chosen exactly as in READ_PARAMETERS:
  Instruction_srcNN_lsMM line 1 'spectral' -> forward solve (the instruction file is removed,
                                              driver.f90:243);
  line 1 'adjoint'                         -> adjoint solve;
  no instruction file                      -> kernel construction (PRODUCE_KERNELS).
Marker files in the working directory: compute_data, linesearch, compute_synth.
Option: with KERNEL_MODE, READ_PARAMETERS sets option 17 whenever the instruction's second line is
'2D' (initialize.f90:1094, 1135-1138), overriding PARSE_OPTIONS; the Spectral and Adjoint
templates the callers copy carry that line, and option 17 is the solve run here.  Options 5 and 6
are unreachable through the reference executable (TEST_IN_2D is only set by READ_PARAMETERS) and
are the WaveSolverSponge API.  An instruction without '2D' selects option 16: with ny = 1 it is
run as option 17 (the same equations with no y-dependence), with ny > 1 the executable exits with
status 2 (the 3-D solver is the WaveSolver3D API).

Files written (same names and FITS layout as the reference):
  <dir>/forward_srcNN_lsMM/{vz_cc.fits, timeline, kernel_info, rms_hist}
  <dir>/adjoint_srcNN/{kernel_info, timeline, rms_hist}
  <dir>/kernel/{kernel_c_NN, kernel_vx_NN, kernel_vz_NN, kernel_psi_NN, hessian_NN}.fits
The partial states the reference dumps every 15 steps as ~3000 FITS files
(all_modules.f90:750-784) are kept as one array file per run (partial_states.npy) in the same
folders, or with SPARC_PARTIAL_FITS=1 written as the reference's own *_partial.fits files
(payloads encoded on the GPU); the kernel stage reads either, so it also consumes partial
states written by the reference, and removes them as PRODUCE_KERNELS does.

Adjoint source: a forward run that is not a data run computes the travel-time adjoint source
of ADJOINT_SOURCE_FILT (driver.f90:1758-2238; ttadjoint.py, csrc/sparc_tt.cu) from the ridge
filters selected by <dir>/params.<pord> and <dir>/filter.params.* and writes
adjoint_srcNN/{source.fits, information}, forward_srcNN_lsMM/ttdiff.<pord>,
forward_srcNN_ls00/windows.<pord> and kernel/misfit_NN_MM; SPARC_ADJOINT_SOURCE=waveform
writes the time-reversed waveform residual (synthetic minus <dir>/data/NN.fits) instead.

Environment: SPARC_PRECISION (64, or 32), SPARC_DEVICE (cuda:0), SPARC_NSTEPS (override maxtime+1),
SPARC_ADJOINT_SOURCE (tt, or waveform), SPARC_PARTIAL_FITS (0, or 1).
"""
from __future__ import annotations

import math
import os
import sys

import numpy as np

from . import fits
from .config import DIMC, parse_params_i, run_config_from_params
from .model import SourceSpec, load_model, SPATIAL_REFERENCE, TEMPORAL_REFERENCE


def _read_instruction(path):
    with open(path) as f:
        lines = [ln.strip() for ln in f.read().splitlines()]
    kind = lines[0].strip().lower() if lines else ""
    twod = len(lines) > 1 and lines[1].strip().upper() == "2D"
    return kind, twod


def _master_pixel(directory, src):
    with open(os.path.join(directory, "master.pixels")) as f:
        vals = [float(ln.split()[0]) for ln in f if ln.strip()][:100]
    if src < 1 or src > len(vals):
        raise SystemExit(f"sparc: source {src} not in master.pixels ({len(vals)} entries)")
    return vals[src - 1]


def main(argv=None) -> int:
    argv = list(sys.argv[1:] if argv is None else argv)
    if len(argv) < 2:
        print("usage: sparc <src NN> <job MM>", file=sys.stderr)
        return 2
    contrib, jobno = argv[0], argv[1]
    src = int(contrib)
    params = parse_params_i(open("params.i").read())
    directory = params["directory"]
    run = run_config_from_params(params)
    if os.environ.get("SPARC_NSTEPS"):
        run = run.replace(nsteps=int(os.environ["SPARC_NSTEPS"]))
    precision = int(os.environ.get("SPARC_PRECISION", "64"))
    device = os.environ.get("SPARC_DEVICE", "cuda:0")
    instr = f"Instruction_src{contrib}_ls{jobno}"
    kind, twod = _read_instruction(instr) if os.path.exists(instr) else ("", True)
    if not twod and int(params.get("ny", 1)) > 1:
        # no '2D' line and ny > 1: PARSE_OPTIONS picks the 3-D option 16 (initialize.f90:833-837),
        # which this executable does not run -- the 3-D solver is the WaveSolver3D API
        print("sparc: 3-D instruction (option 16) with ny > 1: use sparc_flows_gb300.solver3d", file=sys.stderr)
        return 2
    model = load_model(params.get("file_data", "solar_deep"), run.nz)
    compute_data = os.path.exists("compute_data")
    if os.path.exists(instr):
        if kind == "spectral":
            rc = _forward(run, model, directory, contrib, jobno, src, precision, device, compute_data)
            if os.path.exists(instr):
                os.remove(instr)
            return rc
        if kind == "adjoint":
            return _adjoint(run, model, directory, contrib, jobno, precision, device)
        print(f"sparc: unknown instruction {kind!r}", file=sys.stderr)
        return 2
    return _kernels(run, model, directory, contrib, jobno, precision, device)


def _flow_inputs(run, directory, jobno, compute_data):
    """Stream function or direct flow (driver.f90:63-147)."""
    if not run.flows:
        return None, None
    if compute_data and os.path.exists("true_vx.fits"):
        vx = fits.read("true_vx.fits").reshape(run.nz, run.nx) * 1e2 / DIMC
        vz = fits.read("true_vz.fits").reshape(run.nz, run.nx) * 1e2 / DIMC
        return None, (vx, vz)
    p = os.path.join(directory, f"model_psi_ls{jobno}.fits")
    if os.path.exists(p):
        return fits.read(p).reshape(run.nz, run.nx), None
    return None, None


def _solver(run, model, directory, jobno, precision, device, compute_data, nb=1):
    import torch
    from .solver import WaveSolver

    psi, direct = _flow_inputs(run, directory, jobno, compute_data)
    ws = WaveSolver(run, model, nbatch=nb, precision=precision, psi=psi, device=device)
    if direct is not None:
        ws.set_flow_direct(torch.as_tensor(direct[0]), torch.as_tensor(direct[1]))
    return ws


def _forward(run, model, directory, contrib, jobno, src, precision, device, compute_data):
    import torch

    out = os.path.join(directory, f"forward_src{contrib}_ls{jobno}")
    os.makedirs(out, exist_ok=True)
    xloc = _master_pixel(directory, src)
    ws = _solver(run, model, directory, jobno, precision, device, compute_data)
    ws.set_forward_sources([SourceSpec(xloc, SPATIAL_REFERENCE, 0.5, TEMPORAL_REFERENCE, 0.003)])
    keep = not (os.path.exists("compute_synth") or os.path.exists("linesearch") or compute_data)
    res = ws.forward(snapshots=keep)
    seis, snaps = (res if keep else (res, None))
    s = seis.double().cpu().numpy()[0]
    _write_forward_files(out, run, s)
    if keep:
        _save_partial_states(out, snaps[0], run.steps_out, forward=True)
    if not compute_data:
        _adjoint_source_files(run, directory, contrib, jobno, xloc, s, device)
    ws.close()
    return 0


def _write_forward_files(out, run, s):
    """vz_cc.fits (records (nrec, 1, nx)), kernel_info, timeline and rms_hist of a forward run
    (all_modules.f90:1081-1101, driver.f90:337-475)."""
    fits.write(os.path.join(out, "vz_cc.fits"), s[:, None, :])
    with open(os.path.join(out, "kernel_info"), "w") as f:
        f.write(f"{0}\n{run.nsteps - 1}\n")
    with open(os.path.join(out, "timeline"), "w") as f:
        for i in range(0, run.nsteps, run.steps_out):
            f.write(f"{i} {-run.solartime_h * 3600.0 + (i + 1) * run.timestep}\n")
    with open(os.path.join(out, "rms_hist"), "w") as f:
        f.write(f"{float(np.sqrt((s[-1] ** 2).sum()))}\n")


def _adjoint_source_files(run, directory, contrib, jobno, xloc, s, device):
    """The adjoint source of a forward run that is not a data run, against <dir>/data/NN.fits:
    the travel-time source and misfit files, or with SPARC_ADJOINT_SOURCE=waveform the
    time-reversed waveform residual, written to adjoint_srcNN/source.fits."""
    data_p = os.path.join(directory, "data", f"{contrib}.fits")
    data = fits.read(data_p).reshape(s.shape) if os.path.exists(data_p) else np.zeros_like(s)
    if os.environ.get("SPARC_ADJOINT_SOURCE", "tt") == "waveform":
        adir = os.path.join(directory, f"adjoint_src{contrib}")
        os.makedirs(adir, exist_ok=True)
        fits.write(os.path.join(adir, "source.fits"), (s - data)[::-1][:, None, :])
    else:
        _tt_adjoint(run, directory, contrib, jobno, xloc, s, data, device)


def _tt_adjoint(run, directory, contrib, jobno, xloc, synth, data, device):
    """ADJOINT_SOURCE_FILT (driver.f90:1758-2238) and MISFIT_ALL (driver.f90:2294-2651) after a
    forward run that is not a data run: travel times of the ridge-filtered records, adjoint
    source, misfit files."""
    import torch

    from .ttadjoint import (TTAdjoint, read_measurement_files, read_windows, read_windows_all, write_misfit_all,
                            write_outputs)

    linesearch = os.path.exists("linesearch")
    tl = np.loadtxt(os.path.join(directory, f"forward_src{contrib}_ls{jobno}", "timeline"), ndmin=2)[:, 1]
    t_min = -tl[::-1] / 60.0
    modes, freq = read_measurement_files(directory)
    windows = read_windows(directory, contrib, modes) if linesearch else None
    tt = TTAdjoint(run.nx, synth.shape[0], 1, run.xlength_cm, float(run.outputcad), device=device)
    res = tt.run(torch.as_tensor(synth[None]), torch.as_tensor(data[None]), [xloc], t_min, modes, freq, windows)
    write_outputs(directory, contrib, jobno, res, 0, t_min, linesearch, os.path.exists("compute_synth"))
    # MISFIT_ALL (driver.f90:276, 2294-2651)
    wall = read_windows_all(directory, contrib, modes) if linesearch else None
    bands = tt.misfit_all(torch.as_tensor(synth[None]), torch.as_tensor(data[None]), [xloc], t_min, modes, wall)
    write_misfit_all(directory, contrib, jobno, bands, 0, linesearch)
    tt.close()


def _adjoint(run, model, directory, contrib, jobno, precision, device):
    adir = os.path.join(directory, f"adjoint_src{contrib}")
    srcf = os.path.join(adir, "source.fits")
    if not os.path.exists(srcf):
        print(f"sparc: missing {srcf}", file=sys.stderr)
        return 1
    arun = run.replace(adjoint=True)
    ws = _solver(arun, model, directory, jobno, precision, device, False)
    vr = fits.read(srcf).reshape(-1, run.nx)[: run.forcing_length]
    ws.set_adjoint_sources(vr[None])
    _, snaps = ws.forward(snapshots=True)
    _save_partial_states(adir, snaps[0], run.steps_out, forward=False)
    _write_adjoint_info(adir, run)
    ws.close()
    return 0


def _write_adjoint_info(adir, run):
    with open(os.path.join(adir, "kernel_info"), "w") as f:
        f.write(f"{run.forcing_length}\n{((run.nsteps - 1) // run.cadforcing_step) * run.cadforcing_step}\n")


def _kernels(run, model, directory, contrib, jobno, precision, device):
    import torch

    from .pipeline import kernels_from_partial_states

    fdir = os.path.join(directory, f"forward_src{contrib}_ls{jobno}")
    adir = os.path.join(directory, f"adjoint_src{contrib}")
    ws = _solver(run, model, directory, jobno, precision, device, False)
    fsn = _load_partial_states(fdir, True, ws)
    asn = _load_partial_states(adir, False, ws)
    if fsn is None or asn is None:
        print("sparc: partial states of the forward and adjoint runs are missing", file=sys.stderr)
        ws.close()
        return 1
    ker = kernels_from_partial_states(ws, fsn, asn)
    _write_kernel_files(directory, contrib, ker)
    for d in (fdir, adir):  # kernels.f90:593-595 removes the partial states
        for f in os.listdir(d):
            if f == "partial_states.npy" or f.endswith("_partial.fits"):
                os.remove(os.path.join(d, f))
    ws.close()
    return 0


def _write_kernel_files(directory, contrib, ker):
    """kernel/{kernel_c, kernel_vx, kernel_vz, kernel_psi, hessian}_NN.fits, (nz, 1, nx) each
    (kernels.f90:583-590)."""
    kdir = os.path.join(directory, "kernel")
    os.makedirs(kdir, exist_ok=True)
    for name in ("kernel_c", "kernel_vx", "kernel_vz", "kernel_psi", "hessian"):
        fits.write(os.path.join(kdir, f"{name}_{contrib}.fits"), ker[name][:, None, :])


# partial-state fields of the reference's files (all_modules.f90:759-775) and their slot in the
# (6, nz, nx) records of this package: xi_x, xi_z, v_x, v_z, acc_x, acc_z
_PARTIAL_FWD = (("xix", 0), ("xiz", 1), ("vx", 2), ("vz", 3), ("acc_x", 4), ("acc_z", 5))
_PARTIAL_ADJ = (("vx", 2), ("vz", 3), ("acc_x", 4), ("acc_z", 5))


def _save_partial_states(d, snaps, steps_out, forward):
    """Partial states of a run: one array file, or with SPARC_PARTIAL_FITS=1 the reference's
    files {xix, xiz (forward only), vx, vz, acc_x, acc_z}_<6-digit step>_partial.fits
    (WRITE_OUT_PARTIAL_STATE, all_modules.f90:750-784), encoded on the GPU."""
    if os.environ.get("SPARC_PARTIAL_FITS", "0") != "1":
        np.save(os.path.join(d, "partial_states.npy"), snaps.cpu().numpy())
        return
    from .fits_gpu import write_fields

    nrec, _, nz, nx = snaps.shape
    names = _PARTIAL_FWD if forward else _PARTIAL_ADJ
    for r in range(nrec):
        t = r * steps_out
        write_fields([os.path.join(d, f"{nm}_{t:06d}_partial.fits") for nm, _ in names],
                     snaps[r, [j for _, j in names]], shape=(nz, 1, nx))


def _load_partial_states(d, forward, ws):
    """(nrec, 6, nz, nx) partial states of a run directory from partial_states.npy or from the
    reference's partial-state FITS files (read as kernels.f90:221-280 reads them, decoded on
    the GPU; fields an adjoint run does not write stay zero).  None when neither exists."""
    import torch

    npy = os.path.join(d, "partial_states.npy")
    if os.path.exists(npy):
        return np.load(npy)
    if not os.path.isdir(d):
        return None
    times = sorted(int(f[3:9]) for f in os.listdir(d) if f.startswith("vz_") and f.endswith("_partial.fits"))
    if not times:
        return None
    from .fits_gpu import read_fields

    names = _PARTIAL_FWD if forward else _PARTIAL_ADJ
    out = None
    for r, t in enumerate(times):
        flds = read_fields([os.path.join(d, f"{nm}_{t:06d}_partial.fits") for nm, _ in names], ws.dev,
                           precision=ws.precision)
        if out is None:
            nz, nx = flds.shape[1], flds.shape[-1]
            out = torch.zeros((len(times), 6, nz, nx), dtype=flds.dtype, device=ws.dev)
        for i, (_, j) in enumerate(names):
            out[r, j] = flds[i].reshape(nz, nx)
    return out


if __name__ == "__main__":
    sys.exit(main())
