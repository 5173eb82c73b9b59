"""Host logic of the grad.py drop-in (no GPU): the epslist bookkeeping (grad.py:401-428) and
the argument conventions of grad.py's main (grad.py:126-145)."""
import os

import numpy as np

from sparc_flows_gb300 import gradient as G

GOLD = np.load(os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "grad_small.npz"))


def test_epslist_first_pass_matches_reference(tmp_path):
    p = str(tmp_path / "epslist.npz")
    G._update_epslist(p, 0, list(GOLD["eps"]))
    G._update_epslist(p, 1, list(GOLD["eps"]))
    with np.load(p) as f:
        assert sorted(f.files) == ["0", "1"]
        assert np.array_equal(f["1"], GOLD["epslist_1"])


def test_epslist_second_pass_keeps_the_first_in_rows_2_3(tmp_path):
    p = str(tmp_path / "epslist.npz")
    G._update_epslist(p, 3, [0.01, 0.02])
    with np.load(p) as f:
        a = f["3"].copy()
    a[1] = [5.0, 6.0]  # misfits written by the line search
    np.savez(p, **{"3": a})
    G._update_epslist(p, 3, [0.03, 0.04])
    with np.load(p) as f:
        b = f["3"]
    assert np.array_equal(b[0], [0.03, 0.04]) and not b[1].any()
    assert np.array_equal(b[2], [0.01, 0.02]) and np.array_equal(b[3], [5.0, 6.0])


def test_argument_conventions():
    assert G._isfloat("0.01") and G._isfloat("1E-2") and not G._isfloat("algo=cg")
    assert G.ALGOS["cg"] == G.ALGOS["conjugate gradient"] == 1
    assert G.ALGOS["sd"] == G.ALGOS["steepest descent"] == 0
    assert G.SYM["asym"] == -1 and G.ZFILT["gaussian"] == 1
