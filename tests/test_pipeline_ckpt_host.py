"""FwdAdjKernels' checkpointed bookkeeping on the CPU, the 2-D plan replaced by a stand-in whose
records are their own indices: the forward run writes every seismogram record and a checkpoint
at the start of each segment of K records; the adjoint run pairs its ja-th record with forward
record nrec-1-ja (kernels.f90:215, 258) after 1 + ja*steps_out steps, recomputing each segment
from its checkpoint once, latest first, into a buffer of K records."""
import contextlib

import numpy as np
import pytest
import torch

from sparc_flows_gb300 import model as M
from sparc_flows_gb300 import pipeline
from sparc_flows_gb300.config import RunConfig


class Fake2D:
    LAUNCHES_PER_STEP = 12

    def __init__(self, run, model, nbatch=1, precision=32, cmul=None, psi=None, device="cpu", **kw):
        self.run, self.so = run, run.steps_out
        self.dtype = torch.float32 if precision == 32 else torch.float64
        self.t, self.loads, self.pairs = 0, [], []

    def set_forward_sources(self, specs):
        pass

    def set_adjoint_sources_device(self, src):
        self.src = src

    def checkpoint_bytes(self):
        return 64

    def reset(self, t=0):
        self.t = t

    def checkpoint_save(self, buf):
        buf[:8] = torch.tensor([self.t], dtype=torch.int64).view(torch.uint8)

    def checkpoint_load(self, buf):
        self.t = int(buf[:8].view(torch.int64)[0])
        self.loads.append(self.t)

    def run_steps(self, n, seis=None, snaps=None, nrec_cap=None, rec0=0):
        for _ in range(n):
            if self.t % self.so == 0:  # the step with index j*steps_out writes record j
                j = self.t // self.so
                if seis is not None and j < nrec_cap:
                    seis[:, j] = j
                if snaps is not None and 0 <= j - rec0 < nrec_cap:
                    snaps[:, j - rec0] = j
            self.t += 1

    def kernels_accumulate(self, buf, slot, kacc):
        self.pairs.append((self.t, int(buf[0, slot].reshape(-1)[0])))

    def close(self):
        pass


@pytest.mark.parametrize("nsteps,so,K", [(61, 5, 4), (60, 5, 3), (41, 4, 10), (36, 7, 2)])
def test_checkpointed_records_pairs_and_segments(monkeypatch, nsteps, so, K):
    monkeypatch.setattr(pipeline, "WaveSolver", Fake2D)
    monkeypatch.setattr(torch.cuda, "device", lambda d: contextlib.nullcontext())
    run = RunConfig(nx=16, nz=12, nsteps=nsteps, timestep=2.0, outputcad=so * 2.0, cadforcing=so * 2.0)
    assert run.steps_out == so
    pipe = pipeline.FwdAdjKernels(run, M.polytrope(12), [M.SourceSpec(0.0)] * 2, device="cpu",
                                  receivers=np.arange(4), checkpoint_every=K)
    nrec = run.nrec
    seis, _ = pipe.run_all()
    assert seis[0, :, 0].tolist() == list(range(nrec))
    assert pipe.snaps.shape[1] == K  # a buffer of one segment, not of every record
    nseg = -(-nrec // K)
    assert pipe.adj.pairs == [(1 + ja * so, nrec - 1 - ja) for ja in range(nrec)]
    assert pipe.adj.t == nsteps
    assert pipe.fwd.loads == [m * K * so for m in reversed(range(nseg))]
    pipe.close()


def test_checkpoint_every_bounds(monkeypatch):
    monkeypatch.setattr(pipeline, "WaveSolver", Fake2D)
    monkeypatch.setattr(torch.cuda, "device", lambda d: contextlib.nullcontext())
    run = RunConfig(nx=16, nz=12, nsteps=21, timestep=2.0, outputcad=10.0, cadforcing=10.0)
    with pytest.raises(ValueError):
        pipeline.FwdAdjKernels(run, M.polytrope(12), [M.SourceSpec(0.0)], device="cpu", checkpoint_every=run.nrec)
