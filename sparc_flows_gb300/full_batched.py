"""One inversion iteration's forward, adjoint and kernel stages for every source in one process:
the batched counterpart of full.py's per-source loop (full.py:18-59, which runs ``sparc NN 00``
three times per source: forward with the Spectral instruction, adjoint with Adjoint, then the
kernel stage), writing the same files.

Run in the code directory (params.i, the model file), like full.py:

  python -m sparc_flows_gb300.full_batched [--sources 1,2,...] [--jobno 00]

All sources share one FwdAdjKernels batch: the forward solves run together, each source's
forward files (forward_srcNN_lsMM/{vz_cc.fits, kernel_info, timeline, rms_hist}) and adjoint
source (the travel-time source with its misfit files, or the waveform residual with
SPARC_ADJOINT_SOURCE=waveform; adjoint_srcNN/source.fits) are written exactly as the sparc
forward run writes them (cli._write_forward_files, cli._adjoint_source_files), the adjoint
solves run together from those source files with the kernel integral accumulated in HBM, and
kernel/{kernel_c, kernel_vx, kernel_vz, kernel_psi, hessian}_NN.fits are written per source.
No partial states touch the disk.  Environment as the sparc drop-in: SPARC_PRECISION,
SPARC_DEVICE, SPARC_NSTEPS, SPARC_ADJOINT_SOURCE; SPARC_CHECKPOINT_EVERY=K keeps checkpoints
every K records instead of all partial states.
"""
from __future__ import annotations

import argparse
import os
import sys

import numpy as np

from . import cli, fits
from .config import parse_params_i, run_config_from_params
from .model import SPATIAL_REFERENCE, TEMPORAL_REFERENCE, SourceSpec, load_model


def run_iteration(sources: list[int] | None = None, jobno: str = "00") -> int:
    import torch

    from .pipeline import FwdAdjKernels

    params = parse_params_i(open("params.i").read())
    directory = params["directory"]
    run = run_config_from_params(params)
    if os.environ.get("SPARC_NSTEPS"):
        run = run.replace(nsteps=int(os.environ["SPARC_NSTEPS"]))
    precision = int(os.environ.get("SPARC_PRECISION", "64"))
    device = os.environ.get("SPARC_DEVICE", "cuda:0")
    ck = int(os.environ.get("SPARC_CHECKPOINT_EVERY", "0")) or None
    model = load_model(params.get("file_data", "solar_deep"), run.nz)
    with open(os.path.join(directory, "master.pixels")) as f:
        npix = len([ln for ln in f if ln.strip()])
    sources = sources or list(range(1, min(npix, 100) + 1))
    contribs = [f"{s:02d}" for s in sources]
    xlocs = [cli._master_pixel(directory, s) for s in sources]
    psi, direct = cli._flow_inputs(run, directory, jobno, False)
    specs = [SourceSpec(x, SPATIAL_REFERENCE, 0.5, TEMPORAL_REFERENCE, 0.003) for x in xlocs]
    pipe = FwdAdjKernels(run, model, specs, psi=psi, precision=precision, device=device, checkpoint_every=ck)
    if direct is not None:
        for ws in (pipe.fwd, pipe.adj):
            ws.set_flow_direct(torch.as_tensor(direct[0]), torch.as_tensor(direct[1]))
    seis = pipe.forward().double().cpu().numpy()
    for b, (contrib, xloc) in enumerate(zip(contribs, xlocs)):
        out = os.path.join(directory, f"forward_src{contrib}_ls{jobno}")
        os.makedirs(out, exist_ok=True)
        cli._write_forward_files(out, run, seis[b])
        cli._adjoint_source_files(run, directory, contrib, jobno, xloc, seis[b], device)
    src = np.stack([fits.read(os.path.join(directory, f"adjoint_src{c}", "source.fits")).reshape(-1, run.nx)
                    [: run.forcing_length] for c in contribs])
    pipe.adjoint(torch.as_tensor(src, dtype=torch.float64, device=pipe.dev))
    ker = {k: v.cpu().numpy() for k, v in pipe.final_kernels(summed=False).items()}
    for b, contrib in enumerate(contribs):
        cli._write_kernel_files(directory, contrib, {k: v[b] for k, v in ker.items()})
        cli._write_adjoint_info(os.path.join(directory, f"adjoint_src{contrib}"), run)
    pipe.close()
    return 0


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description="forward, adjoint and kernels of all sources in one process")
    ap.add_argument("--sources", default="", help="comma-separated source numbers (default: all master pixels)")
    ap.add_argument("--jobno", default="00")
    a = ap.parse_args(argv)
    srcs = [int(v) for v in a.sources.split(",") if v.strip()] or None
    return run_iteration(srcs, a.jobno)


if __name__ == "__main__":
    sys.exit(main())
