"""The uneven batch: grouped solves on concurrent streams give each solve's own results."""
import numpy as np
import pytest
import torch

from sparc_flows_gb300 import model as M

pytestmark = pytest.mark.gpu


def test_grouped_concurrent_run_equals_single_solves():
    from sparc_flows_gb300.uneven import UnevenBatch
    solves = [M.Solve(256, 60, 100.0, 0.02, -10.0), M.Solve(256, 60, 200.0, 0.03, 15.0),
              M.Solve(384, 90, 50.0, 0.01, 0.0), M.Solve(256, 90, 0.0, 0.0, 5.0)]
    ub = UnevenBatch(solves, precision=32, autotune=False)  # the same column variant as the single runs
    assert sorted(len(v) for v in ub.groups.values()) == [1, 1, 2]
    ub.run()
    batched = [ub.seismograms(i).double().cpu().numpy() for i in range(len(solves))]
    ker = {}
    for key, idx in ub.groups.items():
        k = ub.pipes[key].final_kernels(summed=False)["kernel_c"]
        for j, i in enumerate(idx):
            ker[i] = k[j].cpu().numpy()
    ub.close()
    for i, s in enumerate(solves):
        one = UnevenBatch([s], precision=32, autotune=False)
        one.run()
        ref = one.seismograms(0).double().cpu().numpy()
        kref = one.pipes[(s.nx, s.nsteps)].final_kernels(summed=False)["kernel_c"][0].cpu().numpy()
        one.close()
        assert np.abs(ref).max() > 0
        assert np.linalg.norm(batched[i] - ref) <= 1e-6 * np.linalg.norm(ref), i
        assert np.linalg.norm(ker[i] - kref) <= 1e-6 * np.linalg.norm(kref), i


@pytest.mark.parametrize("mode", ["alone", "concurrent"])
def test_autotuned_groups_pick_a_candidate_and_agree(mode):
    """Each group's column variant is one of the timed candidates (timed on the group's plan alone,
    or in rounds of every group at once), and its seismograms agree with the default variant's to
    FP32 accuracy (different variants round differently)."""
    from sparc_flows_gb300.uneven import COLUMN_CANDIDATES, UnevenBatch
    solves = [M.Solve(256, 60, 100.0, 0.02, -10.0), M.Solve(384, 60, 50.0, 0.01, 0.0)]
    tuned = UnevenBatch(solves, precision=32, autotune=mode)
    assert len(tuned.tuned) == 2
    for key, t in tuned.tuned.items():
        assert tuple(t["choice"]) in COLUMN_CANDIDATES[32]
        assert t["how"] == mode
        timed = t["ms_per_step"] if mode == "alone" else t["round_s"]
        assert len(timed) == len(COLUMN_CANDIDATES[32]) and min(timed.values()) > 0
    tuned.run()
    plain = UnevenBatch(solves, precision=32, autotune=False)
    plain.run()
    for i in range(len(solves)):
        a = tuned.seismograms(i).double().cpu().numpy()
        b = plain.seismograms(i).double().cpu().numpy()
        assert np.linalg.norm(a - b) <= 1e-4 * np.linalg.norm(b), i
    tuned.close()
    plain.close()
