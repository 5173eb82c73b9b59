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

Several GPUs: launched under torchrun (RANK, WORLD_SIZE, LOCAL_RANK and MASTER_* in the
environment), every rank takes its contiguous share of the sources (distributed.shard; the
reference runs one sparc process per source, full.py:85-93), runs it on cuda:LOCAL_RANK and writes
that share's files; the kernel sums grad.py forms over all sources (grad.py:188-196: the sum of
kernel_psi and of |hessian|) are then one all-reduce (distributed.sum_kernels), and rank 0 writes
them to kernel/kernel_psi_sum.fits and kernel/hessian_sum.fits (no reference counterpart: grad.py
re-reads the per-source files, which are all written as before).
"""
from __future__ import annotations

import argparse
import os
import sys

import numpy as np

from . import cli, fits
from .config import parse_params_i, run_config_from_params
from .distributed import shard, sum_kernels
from .model import SPATIAL_REFERENCE, TEMPORAL_REFERENCE, SourceSpec, load_model


def run_iteration(sources: list[int] | None = None, jobno: str = "00", rank: int = 0, world: int = 1) -> dict:
    """Forward, adjoint and kernel stages of this rank's share of the sources; returns the kernel
    sums over every source of every rank ({"kernel_psi", "hessian"}: sum of kernel_psi and of
    |hessian|, (nz, nx) FP64, on every rank)."""
    import torch

    from .pipeline import FwdAdjKernels

    params = parse_params_i(open("params.i").read())
    directory = params["directory"]
    run = run_config_from_params(params)
    if os.environ.get("SPARC_NSTEPS"):
        run = run.replace(nsteps=int(os.environ["SPARC_NSTEPS"]))
    precision = int(os.environ.get("SPARC_PRECISION", "64"))
    device = os.environ.get("SPARC_DEVICE", f"cuda:{int(os.environ.get('LOCAL_RANK', '0'))}")
    ck = int(os.environ.get("SPARC_CHECKPOINT_EVERY", "0")) or None
    model = load_model(params.get("file_data", "solar_deep"), run.nz)
    with open(os.path.join(directory, "master.pixels")) as f:
        npix = len([ln for ln in f if ln.strip()])
    sources = shard(sources or list(range(1, min(npix, 100) + 1)), rank, world)
    partial = {k: torch.zeros((run.nz, run.nx), dtype=torch.float64) for k in ("kernel_psi", "hessian")}
    if not sources:  # more ranks than sources: this rank only joins the kernel sum
        return _sum_and_write(partial, directory, rank)
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
    partial["kernel_psi"] += torch.as_tensor(ker["kernel_psi"]).sum(0)
    partial["hessian"] += torch.as_tensor(ker["hessian"]).abs().sum(0)
    return _sum_and_write(partial, directory, rank)


def _sum_and_write(partial: dict, directory: str, rank: int) -> dict:
    """The kernel sums over all ranks (grad.py:188-196); rank 0 writes them."""
    import torch
    import torch.distributed as dist

    if dist.is_available() and dist.is_initialized() and dist.get_backend() == "nccl":
        dev = torch.device("cuda", int(os.environ.get("LOCAL_RANK", "0")))
        partial = {k: v.to(dev) for k, v in partial.items()}
    tot = sum_kernels(partial)
    if rank == 0:
        os.makedirs(os.path.join(directory, "kernel"), exist_ok=True)
        for name in ("kernel_psi", "hessian"):
            fits.write(os.path.join(directory, "kernel", f"{name}_sum.fits"), tot[name].cpu().numpy()[:, None, :])
    return tot


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description="forward, adjoint and kernels of all sources in one process")
    ap.add_argument("--sources", default="", help="comma-separated source numbers (default: all master pixels)")
    ap.add_argument("--jobno", default="00")
    a = ap.parse_args(argv)
    srcs = [int(v) for v in a.sources.split(",") if v.strip()] or None
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("gloo" if os.environ.get("SPARC_DIST_BACKEND") == "gloo" else "nccl")
    try:
        run_iteration(srcs, a.jobno, rank, world)
    finally:
        if world > 1:
            import torch.distributed as dist
            dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
