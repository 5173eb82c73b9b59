"""Checkpoint segments of FwdAdjKernels on the host: for every record interval K the segments
tile the run's steps exactly, and segment m's steps produce exactly the records m K .. m K + K - 1
(a record after every step whose index is a multiple of steps_out, all_modules.f90:750-784)."""
import types

import pytest

from sparc_flows_gb300.pipeline import FwdAdjKernels


@pytest.mark.parametrize("nsteps,so", [(3601, 15), (226, 15), (91, 15), (100, 7)])
def test_segments_tile_the_run(nsteps, so):
    nrec = (nsteps - 1) // so + 1
    for K in range(1, nrec):
        fake = types.SimpleNamespace(ck=K, run=types.SimpleNamespace(steps_out=so, nsteps=nsteps))
        nseg = -(-nrec // K)
        start = 0
        for m in range(nseg):
            n = FwdAdjKernels._segment_steps(fake, m)
            assert n > 0 and start == m * K * so
            recs = [s // so for s in range(start, start + n) if s % so == 0]
            assert recs == list(range(m * K, min((m + 1) * K, nrec)))
            start += n
        assert start == nsteps
