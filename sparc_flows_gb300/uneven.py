"""The uneven batch: independent solves of different grids, lengths and backgrounds.

Solves sharing (nx, steps) form one batched plan (per-solve stream function and sound-speed
multiplier, a per-solve background in HBM); the groups run concurrently, each from its own host
thread on its own CUDA stream, so that small groups fill the GPU together.  autotune="alone"
picks each group's column-pass variant by timing the candidates on that group's own plan; a plan
timed alone is not a plan timed among eight concurrent ones (on the 48-solve workload those
choices, the 8-column TMA pass for the 256 and 384 grids, ran at 2.27e9 grid-point steps/s
against 2.46e9 for the default pass).  autotune="concurrent" (or True) times the candidates
under the load they will run in: every group steps at once on its own stream and host thread,
and the objective is the wall time of the whole set (autotune_concurrent).  Off by default.
The reference runs every solve as its own single-rank ``sparc`` process (data_forward.sh:28).
"""
from __future__ import annotations

import threading

import numpy as np
import torch

from . import model as M
from .pipeline import FwdAdjKernels, receiver_columns


def _rel(a: torch.Tensor, b: torch.Tensor) -> float:
    a, b = a.double(), b.double()
    return float(torch.linalg.vector_norm(a - b) / torch.linalg.vector_norm(b).clamp_min(1e-300))


def group_solves(solves: list) -> dict:
    """{(nx, nsteps): [indices into solves]}"""
    groups: dict = {}
    for i, s in enumerate(solves):
        groups.setdefault((s.nx, s.nsteps), []).append(i)
    return groups


# column-pass variants an autotuned plan chooses from: (column_impl, column_block)
COLUMN_CANDIDATES = {32: [(2, 32), (2, 16), (2, 8), (3, 8), (0, 32), (0, 8), (1, 8)],
                     64: [(0, 32), (0, 8), (1, 8)]}


def autotune_column(run, model, specs, psi, cmul, precision: int, device, nsteps: int = 8,
                    candidates=None) -> tuple[tuple[int, int], dict]:
    """Fastest column-pass variant for one group: each candidate plan (same grid, batch and
    backgrounds) is stepped nsteps times after a warm-up and timed per pass with CUDA events
    (sparc_profile_passes); the variant with the least time per step wins.  Returns
    ((column_impl, column_block), {candidate: ms per step})."""
    from .solver import WaveSolver

    cands = candidates or COLUMN_CANDIDATES[precision]
    times = {}
    for impl, block in cands:
        ws = WaveSolver(run, model, nbatch=len(specs), precision=precision, cmul=cmul, psi=psi, device=device,
                        column_impl=impl, column_block=block)
        ws.set_forward_sources(specs)
        ws.profile_passes(nsteps=2)
        p = ws.profile_passes(nsteps=nsteps)
        times[(impl, block)] = sum(p["per_class_ms"].values())
        ws.close()
    best = min(times, key=times.get)
    return best, times


def _concurrent_round(solvers: dict, nsteps: dict, streams: dict) -> float:
    """Wall seconds for every group's solver to advance nsteps[key] steps, all groups at once, each
    from its own host thread on its own stream (device-synchronised on both sides)."""
    import time

    errors = []

    def work(key):
        try:
            with torch.cuda.stream(streams[key]):
                solvers[key].run_steps(nsteps[key])
            streams[key].synchronize()
        except Exception as e:
            errors.append((key, e))

    torch.cuda.synchronize()
    t0 = time.perf_counter()
    threads = [threading.Thread(target=work, args=(k,)) for k in solvers]
    for t in threads:
        t.start()
    for t in threads:
        t.join()
    torch.cuda.synchronize()
    if errors:
        raise RuntimeError(f"autotune round, group {errors[0][0]}: {errors[0][1]}")
    return time.perf_counter() - t0


def autotune_concurrent(inputs: dict, precision: int, device, steps_per: int = 50, reps: int = 3,
                        candidates=None) -> tuple[dict, dict]:
    """Column-pass variant of every group chosen under concurrency.  inputs: {(nx, nsteps): (run,
    model, specs, psis, cmuls)}.  One round steps every group nsteps // steps_per steps at once
    (the groups' lengths in proportion, as in the full run), each on its own stream and host
    thread; its wall time (least of reps) is the objective.  Coordinate descent: groups in
    decreasing work (solves x nx x steps), each trying every candidate with the other groups'
    current choices held, keeping the fastest.  Returns ({key: (column_impl, column_block)},
    {key: {candidate: seconds of the round}})."""
    from .solver import WaveSolver

    cands = candidates or COLUMN_CANDIDATES[precision]
    dev = torch.device(device)
    cache: dict = {}

    def solver(key, cand):
        if (key, cand) not in cache:
            run, model, specs, psis, cmuls = inputs[key]
            ws = WaveSolver(run, model, nbatch=len(specs), precision=precision, cmul=cmuls, psi=psis,
                            device=device, column_impl=cand[0], column_block=cand[1])
            ws.set_forward_sources(specs)
            ws.run_steps(2)  # first launches, graph capture
            cache[(key, cand)] = ws
        return cache[(key, cand)]

    streams = {k: torch.cuda.Stream(device=dev) for k in inputs}
    nsteps = {k: max(1, k[1] // steps_per) for k in inputs}
    choice = {k: cands[0] for k in inputs}
    times: dict = {k: {} for k in inputs}
    order = sorted(inputs, key=lambda k: -len(inputs[k][2]) * k[0] * k[1])
    try:
        with torch.cuda.device(dev):
            for key in order:
                for cand in cands:
                    trial = dict(choice)
                    trial[key] = cand
                    solvers = {k: solver(k, c) for k, c in trial.items()}
                    for ws in solvers.values():
                        ws.reset(0)
                    torch.cuda.synchronize()
                    times[key][cand] = min(_concurrent_round(solvers, nsteps, streams) for _ in range(reps))
                choice[key] = min(times[key], key=times[key].get)
    finally:
        for ws in cache.values():
            ws.close()
    return choice, times


class UnevenBatch:
    def __init__(self, solves: list, precision: int = 32, device: str = "cuda:0", autotune=False):
        self.solves, self.dev = solves, torch.device(device)
        model = M.polytrope(300)
        self.groups = group_solves(solves)
        self.pipes, self.streams, self.tuned, self._inputs = {}, {}, {}, {}
        mode = "concurrent" if autotune is True else (autotune or None)
        if mode not in (None, "alone", "concurrent"):
            raise ValueError(f"autotune must be False, True, 'alone' or 'concurrent', not {autotune!r}")
        chosen: dict = {}
        if mode == "concurrent":
            tin = {}
            for key, idx in self.groups.items():
                run = M.uneven_run(*key)
                tin[key] = (run, model, *self._group_inputs(run, model, idx)[:3])
            chosen, times = autotune_concurrent(tin, precision, device)
            for key in self.groups:
                self.tuned[key] = {"choice": chosen[key], "how": "concurrent",
                                   "round_s": {f"{i},{b}": t for (i, b), t in times[key].items()}}
        for key, idx in self.groups.items():
            nx, nsteps = key
            run = M.uneven_run(nx, nsteps)
            specs, psis, cmuls, rcv = self._group_inputs(run, model, idx)
            col = {}
            if mode == "alone":
                best, times = autotune_column(run, model, specs, psis, cmuls, precision, device)
                self.tuned[key] = {"choice": best, "how": "alone",
                                   "ms_per_step": {f"{i},{b}": t for (i, b), t in times.items()}}
                col = dict(column_impl=best[0], column_block=best[1])
            elif mode == "concurrent":
                col = dict(column_impl=chosen[key][0], column_block=chosen[key][1])
            self.pipes[key] = FwdAdjKernels(run, model, specs, psi=psis, cmul=cmuls, precision=precision,
                                            receivers=rcv, device=device, **col)
            self.streams[key] = torch.cuda.Stream(device=self.dev)
            self._inputs[key] = (run, model, specs, psis, cmuls, rcv)

    def _group_inputs(self, run, model, idx):
        """Sources, stream functions, sound-speed multipliers and receivers of one group."""
        psis, cmuls, specs = [], [], []
        for i in idx:
            s = self.solves[i]
            psis.append(M.gaussian_psi(run, model, M.psi_amplitude_for_peak(run, model, 1.0)) * s.vpeak_ms)
            cmuls.append(M.c_bump(run, model, amp=s.dcc))
            specs.append(M.SourceSpec(s.xloc))
        half = 0.45 * run.nx * 0.78125
        rcv = receiver_columns(run, n=int(2 * half / 2.0), x0=-half, dx=2.0)
        return specs, psis, cmuls, rcv

    def point_steps(self) -> int:
        """Useful grid-point steps of one run (forward and adjoint counted once each)."""
        return sum(2 * s.nx * 300 * s.nsteps for s in self.solves)

    def run(self):
        """Forward + adjoint + kernel integral of every solve; groups concurrently."""
        errors = []

        def work(key):
            try:
                with torch.cuda.device(self.dev), torch.cuda.stream(self.streams[key]):
                    self.pipes[key].run_all()
                self.streams[key].synchronize()
            except Exception as e:  # reported after the join
                errors.append((key, e))

        threads = [threading.Thread(target=work, args=(k,)) for k in self.pipes]
        for t in threads:
            t.start()
        for t in threads:
            t.join()
        if errors:
            raise RuntimeError(f"uneven batch group {errors[0][0]} failed: {errors[0][1]}")

    def errors_against_fp64(self) -> list[dict]:
        """Relative L2 error of every solve's seismograms and scaled kernels from the last run()
        against the same solve in FP64 (the same inputs through FP64 plans, one group at a time);
        one dict per solve, in the order of the solves."""
        out: list = [None] * len(self.solves)
        for key, idx in self.groups.items():
            run, model, specs, psis, cmuls, rcv = self._inputs[key]
            p32 = self.pipes[key]
            p64 = FwdAdjKernels(run, model, specs, psi=psis, cmul=cmuls, precision=64, receivers=rcv,
                                device=str(self.dev))
            with torch.cuda.device(self.dev):
                p64.run_all()
                torch.cuda.synchronize()
                k32, k64 = p32.final_kernels(summed=False), p64.final_kernels(summed=False)
                for j, i in enumerate(idx):
                    e = {"nx": run.nx, "nsteps": run.nsteps,
                         "seismograms": _rel(p32.seis[j], p64.seis[j])}
                    e.update({name: _rel(k32[name][j], k64[name][j]) for name in k64})
                    out[i] = e
            p64.close()
        return out

    def seismograms(self, i: int) -> torch.Tensor:
        """Seismograms (nrec, nx) of solve i from the last run."""
        for key, idx in self.groups.items():
            if i in idx:
                return self.pipes[key].seis[idx.index(i)]
        raise IndexError(i)

    def close(self):
        for p in self.pipes.values():
            p.close()
