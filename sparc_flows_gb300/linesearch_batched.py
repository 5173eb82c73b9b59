"""The line-search forward runs of an iteration in one process: the batched counterpart of
linesearch.py (linesearch.py:39-56, one ``sparc NN MM`` forward run per source NN and trial model
MM = 01.., each a PBS process), writing the same files.

Run in the code directory with the `linesearch` marker file present, as master.py sets it up:

  python -m sparc_flows_gb300.linesearch_batched [--sources 1,2,...] [--models 1,2,...]

Every (source, trial model) pair is one solve of a single WaveSolver batch, each with its own
stream function <dir>/model_psi_lsMM.fits (per-solve backgrounds); after the forward solve each
pair's forward_srcNN_lsMM/{vz_cc.fits, kernel_info, timeline, rms_hist} and its travel-time
misfit files are written exactly as the sparc forward run writes them in a line search
(cli._write_forward_files, cli._adjoint_source_files).  The trial models default to those whose
forward_src01_lsMM directory exists, as linesearch.py counts them.  Environment as the sparc
drop-in: SPARC_PRECISION, SPARC_DEVICE, SPARC_NSTEPS, SPARC_ADJOINT_SOURCE.
"""
from __future__ import annotations

import argparse
import fnmatch
import os
import sys

from . import cli
from .config import parse_params_i, run_config_from_params
from .model import SPATIAL_REFERENCE, TEMPORAL_REFERENCE, SourceSpec, load_model


def run_linesearch(sources: list[int] | None = None, models: list[int] | None = None) -> int:
    from .solver import WaveSolver

    params = parse_params_i(open("params.i").read())
    directory = params["directory"]
    run = run_config_from_params(params)
    if os.environ.get("SPARC_NSTEPS"):
        run = run.replace(nsteps=int(os.environ["SPARC_NSTEPS"]))
    precision = int(os.environ.get("SPARC_PRECISION", "64"))
    device = os.environ.get("SPARC_DEVICE", "cuda:0")
    model = load_model(params.get("file_data", "solar_deep"), run.nz)
    with open(os.path.join(directory, "master.pixels")) as f:
        npix = len([ln for ln in f if ln.strip()])
    sources = sources or list(range(1, min(npix, 100) + 1))
    if not models:  # linesearch.py: the forward_src01_ls[0-9][1-9] directories of the iteration
        models = sorted(int(d[-2:]) for d in fnmatch.filter(os.listdir(directory), "forward_src01_ls[0-9][1-9]"))
    if not models:
        print("linesearch_batched: no trial models (forward_src01_lsMM directories)", file=sys.stderr)
        return 1
    pairs = [(s, m) for m in models for s in sources]
    psis = {m: cli._flow_inputs(run, directory, f"{m:02d}", False)[0] for m in models}
    xlocs = {s: cli._master_pixel(directory, s) for s in sources}
    specs = [SourceSpec(xlocs[s], SPATIAL_REFERENCE, 0.5, TEMPORAL_REFERENCE, 0.003) for s, _ in pairs]
    ws = WaveSolver(run, model, nbatch=len(pairs), precision=precision, psi=[psis[m] for _, m in pairs],
                    device=device)
    ws.set_forward_sources(specs)
    seis = ws.forward().double().cpu().numpy()
    ws.close()
    for b, (s, m) in enumerate(pairs):
        nn, mm = f"{s:02d}", f"{m:02d}"
        out = os.path.join(directory, f"forward_src{nn}_ls{mm}")
        os.makedirs(out, exist_ok=True)
        cli._write_forward_files(out, run, seis[b])
        cli._adjoint_source_files(run, directory, nn, mm, xlocs[s], seis[b], device)
    return 0


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description="line-search forward runs of all sources and trial models")
    ap.add_argument("--sources", default="", help="comma-separated source numbers (default: all master pixels)")
    ap.add_argument("--models", default="", help="comma-separated trial model numbers MM (default: as linesearch.py)")
    a = ap.parse_args(argv)
    srcs = [int(v) for v in a.sources.split(",") if v.strip()] or None
    mods = [int(v) for v in a.models.split(",") if v.strip()] or None
    return run_linesearch(srcs, mods)


if __name__ == "__main__":
    sys.exit(main())
