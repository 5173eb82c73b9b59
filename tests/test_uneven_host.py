"""The uneven batch's concurrent autotuner on the CPU: a stand-in solver and a synthetic round time
in place of the GPU, to check the coordinate descent itself (every group tries every candidate
with the other groups' choices held, keeps the fastest, every plan it made is closed)."""
import contextlib

import numpy as np
import pytest
import torch

from sparc_flows_gb300 import uneven
from sparc_flows_gb300.uneven import COLUMN_CANDIDATES, autotune_concurrent

# synthetic cost of a group's plan by column variant; the round takes the slowest group plus a
# contention term that makes the choices interact
COST = {(256, 1800): {(2, 32): 3.0, (2, 8): 1.0},
        (512, 3600): {(2, 32): 2.0, (0, 8): 1.5},
        (384, 2700): {(3, 8): 0.5}}


class FakeSolver:
    made, closed = [], []

    def __init__(self, run, model, nbatch, precision, cmul, psi, device, column_impl, column_block):
        self.key = (run.nx, run.nsteps)
        self.cand = (column_impl, column_block)
        self.steps = 0
        FakeSolver.made.append(self)

    def set_forward_sources(self, specs):
        pass

    def run_steps(self, n):
        self.steps += n

    def reset(self, t):
        pass

    def close(self):
        FakeSolver.closed.append(self)


def fake_round(solvers, nsteps, streams):
    costs = [COST[k].get(ws.cand, 4.0) for k, ws in solvers.items()]
    return max(costs) + 0.1 * sum(costs)


@pytest.fixture
def patched(monkeypatch):
    import sparc_flows_gb300.solver as S
    FakeSolver.made, FakeSolver.closed = [], []
    monkeypatch.setattr(S, "WaveSolver", FakeSolver)
    monkeypatch.setattr(uneven, "_concurrent_round", fake_round)
    monkeypatch.setattr(torch.cuda, "Stream", lambda device=None: object())
    monkeypatch.setattr(torch.cuda, "device", lambda d: contextlib.nullcontext())
    monkeypatch.setattr(torch.cuda, "synchronize", lambda *a, **k: None)


def test_coordinate_descent_picks_each_groups_fastest_variant(patched):
    class Run:
        def __init__(self, nx, nsteps):
            self.nx, self.nsteps = nx, nsteps

    inputs = {k: (Run(*k), None, [object()] * (4 if k[0] == 512 else 2), None, None) for k in COST}
    choice, times = autotune_concurrent(inputs, 32, "cpu", reps=2)
    assert choice == {(256, 1800): (2, 8), (512, 3600): (0, 8), (384, 2700): (3, 8)}
    cands = COLUMN_CANDIDATES[32]
    for k in COST:
        assert set(times[k]) == set(cands)
        best = min(times[k], key=times[k].get)
        assert best == choice[k] and np.isfinite(times[k][best])
    # one plan per (group, candidate) at most, each stepped and closed
    assert len(FakeSolver.made) <= len(COST) * len(cands)
    assert len({(ws.key, ws.cand) for ws in FakeSolver.made}) == len(FakeSolver.made)
    assert all(ws.steps > 0 for ws in FakeSolver.made)
    assert sorted(map(id, FakeSolver.closed)) == sorted(map(id, FakeSolver.made))


def test_groups_tuned_in_decreasing_work(patched, monkeypatch):
    """The largest group (solves x nx x steps) is tuned first: its choice is made with every other
    group still on the first candidate."""
    order = []
    real = uneven._concurrent_round

    def recording_round(solvers, nsteps, streams):
        moving = [k for k, ws in solvers.items() if ws.cand != COLUMN_CANDIDATES[32][0]]
        if moving and (not order or order[-1] != moving[0]):
            order.append(moving[0])
        return real(solvers, nsteps, streams)

    monkeypatch.setattr(uneven, "_concurrent_round", recording_round)

    class Run:
        def __init__(self, nx, nsteps):
            self.nx, self.nsteps = nx, nsteps

    inputs = {k: (Run(*k), None, [object()] * (4 if k[0] == 512 else 2), None, None) for k in COST}
    autotune_concurrent(inputs, 32, "cpu", reps=1)
    assert order and order[0] == (512, 3600)
