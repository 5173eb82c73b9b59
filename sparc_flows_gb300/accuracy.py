"""FP32 batched path against the FP64 path on one source of a full-length workload.

The FP32 pipeline (forward, reference-style adjoint, kernel integral; the batched production
path) and the FP64 pipeline (the precision of the reference build, whose FP64 arithmetic the
oracle restates) run the same source of the same workload; the report gives the relative L2
error of the seismograms and of each scaled kernel (kernels.f90:495-581).
"""
from __future__ import annotations

import numpy as np
import torch

from . import model as M
from .pipeline import FwdAdjKernels


def rel_l2(a, b) -> float:
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def fp32_vs_fp64(workload: str = "batch32", source: int = 15, nsteps: int | None = None,
                 device: str = "cuda:0") -> dict:
    """Relative L2 errors of FP32 against FP64 for source ``source`` of ``workload``."""
    run, model, specs, psi, cmul = M.workload(workload)
    if nsteps:
        run = run.replace(nsteps=nsteps)
    spec = specs[min(source, len(specs) - 1)]
    out = {}
    for prec in (64, 32):
        pipe = FwdAdjKernels(run, model, [spec], psi=psi, cmul=cmul, precision=prec, device=device)
        seis, _ = pipe.run_all()
        torch.cuda.synchronize()
        ker = {k: v[0].cpu().numpy() for k, v in pipe.final_kernels(summed=False).items()}
        out[prec] = (seis[0].double().cpu().numpy(), ker)
        pipe.close()
    s64, k64 = out[64]
    s32, k32 = out[32]
    rep = {"workload": workload, "source_x_mm": spec.xloc, "nsteps": run.nsteps,
           "seismograms": rel_l2(s32, s64)}
    for name in k64:
        rep[name] = rel_l2(k32[name], k64[name])
    rep["max"] = max(v for k, v in rep.items() if k not in ("workload", "source_x_mm", "nsteps"))
    # the metric's condition: every seismogram and kernel within 1e-4 rel-L2 of FP64
    rep["bound"] = 1e-4
    rep["within_bound"] = {k: bool(rep[k] <= 1e-4) for k in ["seismograms", *k64]}
    rep["pass"] = all(rep["within_bound"].values())
    # the same over the physical interior: rows and columns of the absorbing layers left out
    zs = slice(run.npmlbot, run.nz - run.npmltop)
    xs = slice(run.npmlhor, run.nx - run.npmlhor)
    inner = {name: rel_l2(k32[name][zs, xs], k64[name][zs, xs]) for name in k64}
    inner["max"] = max(inner.values())
    rep["interior"] = dict(rows=[zs.start, zs.stop], columns=[xs.start, xs.stop], **inner)
    return rep
