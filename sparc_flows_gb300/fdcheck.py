"""Central-difference check of the exact flow gradient (discrete_adjoint.py) on the autograd
configuration: one source on the 512 x 300 polytrope grid over 400 Mm, the supergranule stream
function, 3600 steps of 2 s, 128 receivers 2 Mm apart; the misfit L = 1/2 |records(psi) - data|^2
with data the records of the true flow and psi half of it.  Each of `ndir` seeded random
perturbations d (white noise under the flow's envelope, scaled to `amp` times max |psi|) gives
the ratio (L(psi + d) - L(psi - d)) / (2 <dL/dpsi, d>), which is 1 for an exact gradient.

  python -m sparc_flows_gb300.fdcheck [--nsteps 3600] [--ndir 16] [--amp 1e-3]
"""
from __future__ import annotations

import argparse
import json
import time

import numpy as np
import torch

from . import model as M
from .discrete_adjoint import ExactGradient, records
from .pipeline import receiver_columns
from .solver import WaveSolver


def fd_check(nsteps: int = 3600, ndir: int = 16, amp: float = 1e-3, seed: int = 0, device: str = "cuda:0") -> dict:
    run, model, specs, psi_true, _ = M.workload("autograd32")
    run = run.replace(nsteps=nsteps)
    ws = WaveSolver(run, model, nbatch=1, precision=64, psi=psi_true, device=device)
    ws.set_forward_sources(specs)
    eg = ExactGradient(ws, receiver_columns(run), segment=100)
    pt = torch.as_tensor(psi_true, device=device)
    with torch.no_grad():
        data = records(pt, eg).clone()
    psi = (0.5 * pt).clone().requires_grad_(True)
    t0 = time.perf_counter()
    loss = 0.5 * ((records(psi, eg) - data) ** 2).sum()
    loss.backward()
    torch.cuda.synchronize()
    t_grad = time.perf_counter() - t0
    g = psi.grad.detach()
    env = pt.abs() / pt.abs().max()
    gen = torch.Generator(device="cpu").manual_seed(seed)
    ratios = []
    for _ in range(ndir):
        d = env * torch.randn(tuple(pt.shape), generator=gen, dtype=torch.float64).to(device)
        d = d * (amp * float(pt.abs().max()) / float(d.abs().max()))
        with torch.no_grad():
            lp = 0.5 * float(((records(psi.detach() + d, eg) - data) ** 2).sum())
            lm = 0.5 * float(((records(psi.detach() - d, eg) - data) ** 2).sum())
        ratios.append((lp - lm) / (2.0 * float((g * d).sum())))
    ws.close()
    r = np.asarray(ratios)
    return {"workload": f"autograd32: 1 source, nx={run.nx}, nz={run.nz}, {nsteps} steps, FP64, "
                        f"{len(eg.rcv)} receivers, psi = half the true flow",
            "directions": ndir, "amplitude": amp, "loss": float(loss.detach()),
            "max_abs_ratio_minus_1": float(np.abs(r - 1.0).max()), "ratios": ratios,
            "forward_plus_backward_s": t_grad}


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--nsteps", type=int, default=3600)
    ap.add_argument("--ndir", type=int, default=16)
    ap.add_argument("--amp", type=float, default=1e-3)
    a = ap.parse_args(argv)
    print(json.dumps(fd_check(a.nsteps, a.ndir, a.amp)), flush=True)


if __name__ == "__main__":
    main()
