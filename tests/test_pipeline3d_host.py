"""FwdAdjKernels3D's bookkeeping on the CPU, the 3-D plan replaced by a stand-in whose records are
their own indices: the forward run keeps every v_z record in order and a checkpoint at the start
of each segment; the adjoint run pairs its ja-th record with forward record nrec-1-ja
(kernels.f90:215, 258) after 1 + ja*steps_out steps, and restores and recomputes each segment
holding records exactly once, latest first."""
import numpy as np
import pytest
import torch

from sparc_flows_gb300 import model as M
from sparc_flows_gb300 import pipeline3d


class Fake3D:
    def __init__(self, nx, ny, model, xlength_cm, nbatch=1, precision=32, steps_out=1, flows=False,
                 timestep=2.0, device="cpu", **kw):
        self.nx, self.ny, self.nz, self.nb, self.so = nx, ny, model.shape[0], nbatch, steps_out
        self.dtype = torch.float32 if precision == 32 else torch.float64
        self.t, self.loads, self.pairs = 0, [], []

    def set_flow(self, *v):
        pass

    def set_source(self, pattern, amp):
        pass

    def reset(self, t=0):
        self.t = t

    def checkpoint_bytes(self):
        return 64

    def checkpoint_save(self, buf):
        buf[:8] = torch.tensor([self.t], dtype=torch.int64).view(torch.uint8)
        return self.t

    def checkpoint_load(self, buf, time):
        self.t = int(buf[:8].view(torch.int64)[0])
        assert self.t == time
        self.loads.append(time)

    def forward_records(self, n, snaps, rec0=0, seis=None):
        made = 0
        for _ in range(n):
            if self.t % self.so == 0:  # the step with index j*steps_out makes record j
                j = self.t // self.so
                if snaps is not None and 0 <= j - rec0 < snaps.shape[0]:
                    snaps[j - rec0] = j
                if seis is not None and made < seis.shape[0]:
                    seis[made] = j
                made += 1
            self.t += 1
        return made

    def record_buffer(self, nslot):
        return torch.full((nslot,), -1.0, dtype=torch.float64)

    def set_adjoint_source(self, src, w, idx, scale=None):
        self.src = src

    def kernels_accumulate(self, snaps, slot, out):
        self.pairs.append((self.t, int(snaps[slot])))

    def close(self):
        pass


@pytest.mark.parametrize("nsteps,so,K", [(40, 5, 15), (41, 5, 10), (37, 4, 100), (30, 7, 3), (25, 5, 5)])
def test_records_pairs_and_segments(monkeypatch, nsteps, so, K):
    monkeypatch.setattr(pipeline3d, "WaveSolver3D", Fake3D)
    model = M.polytrope(20)
    pats = np.ones((2, 8, 8))
    pipe = pipeline3d.FwdAdjKernels3D(8, 8, model, 200e8, pats, np.zeros(nsteps + 5), nsteps, steps_out=so,
                                      checkpoint_every=K, device="cpu")
    nrec = (nsteps - 1) // so + 1
    seis, _ = pipe.run_all()
    assert pipe.nrec == nrec
    # forward: every record, in order; a checkpoint at the start of each segment
    assert seis[:, 0, 0, 0].tolist() == list(range(nrec))
    assert pipe.ckpt_time == [m * K for m in range(pipe.nseg)]
    # adjoint: record ja (after 1 + ja*so steps) against forward record nrec-1-ja
    assert pipe.adj.pairs == [(1 + ja * so, nrec - 1 - ja) for ja in range(nrec)]
    assert pipe.adj.t == nsteps
    # each segment holding records restored and recomputed once, latest first
    with_recs = [m for m in range(pipe.nseg) if pipe._records_of(m)]
    assert pipe.fwd.loads == [m * K for m in reversed(with_recs)]
    pipe.close()
