"""Host side of the travel-time adjoint source: the product's filter masks and window ranges
against the oracle's literal restatement of driver.f90 (no GPU)."""
import numpy as np
import pytest

from oracle import tt_oracle as TO
from sparc_flows_gb300 import ttadjoint as TT


@pytest.mark.parametrize("nx,nt,xl", [(64, 240, 200e8), (128, 241, 400e8)])
def test_ridge_filters_match_oracle(nx, nt, xl):
    got = TT.ridge_filters(nx, nt, xl, 30.0)
    for p in range(9):
        want = TO.ridge_filter(p, nx, nt, xl, 30.0)
        assert np.abs(got[p] - want).max() <= 1e-13, p
        assert got[p].max() > 0.5  # every ridge passes something at these sizes


def test_frequency_filters_and_their_carry_over():
    nx, nt, xl = 64, 240, 200e8
    freq = {"allmodes": (2.0, 5.0), 1: (2.5, 4.0)}
    got = TT.mode_filters(nx, nt, xl, 30.0, freq)
    fa = TO.freq_filter(2.0, 5.0, nt, 30.0)
    f1 = TO.freq_filter(2.5, 4.0, nt, 30.0)
    rid = [TO.ridge_filter(p, nx, nt, xl, 30.0) for p in range(9)]
    assert np.allclose(got[0], rid[0] * (fa * fa)[:, None], atol=1e-14)   # no .0 file: all-modes twice
    assert np.allclose(got[1], rid[1] * (fa * f1)[:, None], atol=1e-14)
    assert np.allclose(got[2], rid[2] * (fa * f1)[:, None], atol=1e-14)   # no .2 file: carries .1
    assert np.allclose(got[5], rid[5] * fa[:, None], atol=1e-14)


def test_search_ranges_match_oracle():
    row = np.zeros(240)
    row[100] = 1.0
    for pord in range(9):
        for dist in (3.7, 12.0, 25.5):
            ts, tf = TT.search_range(pord, dist, 0.5)
            wb = TO.window_bounds(pord, dist, 0.5, row, 10)
            if wb is not None:
                assert (ts, tf) == (wb[3], wb[4])


def test_signed_index_is_distmat():
    for n in (7, 8, 241, 512):
        assert np.array_equal(TT.signed_index(n), TO.distmat(n))


def test_measurement_files(tmp_path):
    (tmp_path / "params.0").write_text("5.0\n40.0\n12.5\n")
    (tmp_path / "params.8").write_text("10 60 20\n")
    (tmp_path / "filter.params.allmodes").write_text("1.5\n5.5\n")
    modes, freq = TT.read_measurement_files(str(tmp_path))
    assert modes == {0: (5.0, 40.0, 12.5), 8: (10.0, 60.0, 20.0)}
    assert freq == {"allmodes": (1.5, 5.5)}


def test_misfit_search_ranges_match_oracle():
    for pord in range(9):
        for dist in (3.7, 12.0, 25.5, 55.0):
            assert TT.misfit_search_range(pord, dist, 0.5) == TO.misfit_search_range(pord, dist, 0.5)


def test_compute_tt_of_a_shifted_pulse():
    """A Gaussian pulse delayed by 0.8 records: COMPUTE_TT returns the delay (positive = late)."""
    t = np.arange(41, dtype=float)
    u0 = np.exp(-((t - 20.0) / 3.0) ** 2)
    u = np.exp(-((t - 20.8) / 3.0) ** 2)
    tau = TO.compute_tt(u0, u, 0.5)
    assert abs(tau - 0.4) < 0.02
