"""2-D velocity-pressure-density solvers (option 5 with the sponge, option 6 with the PML,
option 12 with the PML and a background magnetic field, sparc5_*) against the CPU oracle of
MP_QUIET_SPONGE_2D / MP_QUIET_PML_2D / MP_MHD_PML_2d (oracle/sparc_oracle_sponge.c), and the
FP32 plans of options 5 and 6 against their FP64 plans."""
import numpy as np
import pytest

from oracle.oracle_sponge import SimSponge
from sparc_flows_gb300 import capi
from sparc_flows_gb300 import model as M
from sparc_flows_gb300.solver_sponge import WaveSolverSponge

pytestmark = pytest.mark.gpu
NX, XL = 128, 200e8


def _inputs(nb=2, nsteps=40):
    x = (np.arange(NX) - NX / 2) / NX
    pats = np.stack([np.exp(-((x - 0.1 * b) ** 2) / 0.002) for b in range(nb)])
    return M.polytrope(300), pats, np.sin(np.arange(nsteps + 5) * 0.3) * 1e-6


def _gpu(precision, nsteps, nb=2, option=5):
    model, pats, amp = _inputs(nb, nsteps)
    ws = WaveSolverSponge(NX, model, XL, nbatch=nb, precision=precision, steps_out=15, obsheight_cm=-100e5,
                          option=option)
    ws.set_source(pats, amp)
    ws.reset(0)
    seis = ws.forward(nsteps).double().cpu().numpy()
    st = ws.state().double().cpu().numpy()
    ws.close()
    return st, seis


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("option", [5, 6])
def test_fp64_matches_oracle(option):
    nsteps, nb = 31, 2
    st, seis = _gpu(64, nsteps, nb, option)
    model, pats, amp = _inputs(nb, nsteps)
    for b in range(nb):
        s = SimSponge(NX, model, XL, steps_out=15, obsheight_cm=-100e5, option=option)
        s.set_source(pats[b], amp)
        rec = s.run(nsteps)
        want = s.state()
        s.close()
        assert rec.shape[0] == seis.shape[0] == 3 and np.abs(rec).max() > 0
        for v in (0, 1, 3, 4):
            assert rel(st[v, :, b], want[v]) < 1e-10, (b, v, rel(st[v, :, b], want[v]))
        assert not st[2].any()
        assert rel(seis[:, b], rec) < 1e-10


@pytest.mark.parametrize("option", [5, 6])
def test_fp32_tracks_fp64(option):
    st32, s32 = _gpu(32, 60, option=option)
    st64, s64 = _gpu(64, 60, option=option)
    for v in (0, 1, 3, 4):
        assert rel(st32[v], st64[v]) < 1e-4, (v, rel(st32[v], st64[v]))


def test_bad_grid_is_rejected():
    with pytest.raises(capi.SparcError, match="FFT table"):
        WaveSolverSponge(500, M.polytrope(300), XL)


def _gpu12(precision, nsteps, nb=2, b_gauss=100.0):
    model, pats, amp = _inputs(nb, nsteps)
    box, boz = M.potential_field(NX, model, XL, b_gauss)
    ws = WaveSolverSponge(NX, model, XL, nbatch=nb, precision=precision, steps_out=15, obsheight_cm=-100e5,
                          option=12, box=box, boz=boz)
    ws.set_source(pats, amp)
    ws.reset(0)
    seis = ws.forward(nsteps).double().cpu().numpy()
    st = ws.state().double().cpu().numpy()
    ws.close()
    return st, seis


def test_option12_fp64_matches_oracle():
    """MP_MHD_PML_2d (physics2d.f90:411-474) with a 100 G current-free background field: all
    eight fields and the records against the oracle (31 steps: the reference's smoothing of
    dv_z/dz on the top PML rows grows an odd-even mode on this polytrope over longer runs)."""
    nsteps, nb = 31, 2
    st, seis = _gpu12(64, nsteps, nb)
    model, pats, amp = _inputs(nb, nsteps)
    box, boz = M.potential_field(NX, model, XL, 100.0)
    for b in range(nb):
        s = SimSponge(NX, model, XL, steps_out=15, obsheight_cm=-100e5, option=12)
        s.set_magnetic(box, boz)
        s.set_source(pats[b], amp)
        rec = s.run(nsteps)
        want = s.state()
        s.close()
        assert want.shape[0] == 8 and np.abs(want[5]).max() > 0 and np.abs(want[7]).max() > 0
        for v in (0, 1, 3, 4, 5, 7):
            assert rel(st[v, :, b], want[v]) < 1e-10, (b, v, rel(st[v, :, b], want[v]))
        assert not st[2].any() and not st[6].any()
        assert rel(seis[:, b], rec) < 1e-10
