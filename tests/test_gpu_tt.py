"""Travel-time adjoint source on the GPU (csrc/sparc_tt.cu) against the oracle's per-receiver
restatement of ADJOINT_SOURCE_FILT (oracle/tt_oracle.py)."""
import numpy as np
import pytest
import torch

from oracle import tt_oracle as TO
from sparc_flows_gb300 import ttadjoint as TT

pytestmark = pytest.mark.gpu

NX, NT, XL, CAD = 64, 240, 200e8, 30.0
MODES = {0: (5.0, 30.0, 10.0), 1: (5.0, 40.0, 12.0), 8: (8.0, 60.0, 20.0)}
FREQ = {"allmodes": (1.5, 6.0), 0: (2.0, 5.0)}
X00 = [-10.0, 15.0]


def _records(seed):
    rng = np.random.default_rng(seed)
    s = rng.standard_normal((len(X00), NT, NX))
    d = np.roll(s, 2, axis=1) + 0.1 * rng.standard_normal(s.shape)
    return s, d


def _tmin():
    timeline = CAD * (np.arange(NT) + 1.0)
    return -timeline[::-1] / 60.0


def test_adjoint_source_matches_oracle():
    s, d = _records(0)
    tt = TT.TTAdjoint(NX, NT, len(X00), XL, CAD)
    res = tt.run(torch.as_tensor(s, device="cuda"), torch.as_tensor(d, device="cuda"), X00, _tmin(), MODES, FREQ)
    adj = res["adj"].cpu().numpy()
    for b, x00 in enumerate(X00):
        ref = TO.adjoint_source(s[b], d[b], x00, XL, _tmin(), CAD, MODES, FREQ)
        assert res["nmeas"][b] == ref["nmeas"] > 0
        assert abs(res["misfit"][b] - 0.5 * ref["misfit"]) <= 1e-10 * abs(ref["misfit"])
        for pord in MODES:
            got = res["rows"][pord].get(b, [])
            want = ref["rows"][pord]
            assert [g[2:7] for g in got] == [w[2:7] for w in want]          # windows and picks exact
            assert [g[0] for g in got] == [w[0] for w in want]
            assert np.allclose([g[1] for g in got], [w[1] for w in want], rtol=1e-9, atol=1e-12)
        assert np.linalg.norm(adj[b] - ref["adj"]) <= 1e-10 * np.linalg.norm(ref["adj"])
    # line search: the same windows given back reproduce the travel times
    res2 = tt.run(torch.as_tensor(s, device="cuda"), torch.as_tensor(d, device="cuda"), X00, _tmin(), MODES, FREQ,
                  windows=res["windows"])
    for pord in MODES:
        for b in range(len(X00)):
            assert np.allclose([r[1] for r in res2["rows"][pord].get(b, [])],
                               [r[1] for r in res["rows"][pord].get(b, [])], rtol=1e-12)
    tt.close()


def test_no_measurement_gives_zero_source():
    s, d = _records(1)
    tt = TT.TTAdjoint(NX, NT, len(X00), XL, CAD)
    res = tt.run(torch.as_tensor(s, device="cuda"), torch.as_tensor(d, device="cuda"), X00, _tmin(), {})
    assert (res["adj"] == 0).all() and (res["nmeas"] == 0).all()
    tt.close()


def test_misfit_all_matches_oracle():
    s, d = _records(2)
    tt = TT.TTAdjoint(NX, NT, len(X00), XL, CAD)
    bands = tt.misfit_all(torch.as_tensor(s, device="cuda"), torch.as_tensor(d, device="cuda"), X00, _tmin(), MODES)
    assert len(bands) == 3
    for b, x00 in enumerate(X00):
        ref = TO.misfit_all(s[b], d[b], x00, XL, _tmin(), CAD, MODES)
        for fb in range(3):
            assert bands[fb]["band"] == ref[fb]["band"]
            assert np.array_equal(bands[fb]["nmeas"][b], ref[fb]["nmeas"])
            assert np.allclose(bands[fb]["misfit"][b], ref[fb]["misfit"], rtol=1e-9, atol=0)
            for pord in MODES:
                assert bands[fb]["windows"][pord].get(b, []) == ref[fb]["windows"][pord]
    assert sum(int(bd["nmeas"].sum()) for bd in bands) > 0
    # line search: the picked windows given back reproduce the misfits
    given = {fb + 1: bands[fb]["windows"] for fb in range(3)}
    again = tt.misfit_all(torch.as_tensor(s, device="cuda"), torch.as_tensor(d, device="cuda"), X00, _tmin(), MODES,
                          windows=given)
    for fb in range(3):
        assert np.allclose(again[fb]["misfit"], bands[fb]["misfit"], rtol=1e-12)
    tt.close()


@pytest.mark.parametrize("nt", [37, 241, 520])
def test_record_counts(nt):
    """Both t transforms: Bluestein's chirp-z (nt <= 512; 241 is prime) and the direct DFT (nt > 512)."""
    rng = np.random.default_rng(nt)
    s = rng.standard_normal((1, nt, NX))
    d = np.roll(s, 1, axis=1) + 0.05 * rng.standard_normal(s.shape)
    tmin = -(CAD * (np.arange(nt) + 1.0))[::-1] / 60.0
    modes = {0: (3.0, 20.0, 10.0)}
    tt = TT.TTAdjoint(NX, nt, 1, XL, CAD)
    res = tt.run(torch.as_tensor(s, device="cuda"), torch.as_tensor(d, device="cuda"), [0.0], tmin, modes)
    tt.close()
    ref = TO.adjoint_source(s[0], d[0], 0.0, XL, tmin, CAD, modes)
    assert res["nmeas"][0] == ref["nmeas"] > 0
    adj = res["adj"][0].cpu().numpy()
    assert np.linalg.norm(adj - ref["adj"]) <= 1e-10 * np.linalg.norm(ref["adj"])
