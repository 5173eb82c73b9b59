"""The velocity-formulation oracle on the host (oracle/sparc_oracle_sponge.c): option 11,
MP_MHD_SPONGE_2D (physics2d.f90:588-658), against option 5 with the field off, and with a
current-free field."""
import numpy as np

from oracle.oracle_sponge import SimSponge
from sparc_flows_gb300 import model as M

NX, XL = 128, 200e8


def _run(option, b_gauss=0.0, nsteps=40):
    model = M.polytrope(300)
    s = SimSponge(NX, model, XL, option=option, obsheight_cm=-100e5)
    if option in (11, 12):
        s.set_magnetic(*M.potential_field(NX, model, XL, b_gauss))
    x = (np.arange(NX) - NX / 2) / NX
    s.set_source(np.exp(-x ** 2 / 0.002), np.sin(np.arange(nsteps + 5) * 0.3) * 1e-6)
    rec = s.run(nsteps)
    st = s.state()
    s.close()
    return rec, st


def _rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def test_option11_without_field_is_option5_away_from_the_boundary_rows():
    """With B = 0 the MHD sponge step differs from MP_QUIET_SPONGE_2D only on the top and bottom
    rows (all eight RHS zeroed there, d p/dz with caller-set boundary rows, ibc 4)."""
    r5, s5 = _run(5)
    r11, s11 = _run(11)
    assert s11.shape[0] == 8 and not s11[5:].any()
    assert _rel(r11, r5) < 1e-9
    for v in (0, 1, 3, 4):
        assert _rel(s11[v, 30:-30], s5[v, 30:-30]) < 1e-7, v


def test_option11_with_field_couples_and_stays_bounded():
    r, st = _run(11, 100.0, 200)
    assert np.isfinite(st).all() and np.abs(st[:5]).max() < 1e-6
    assert np.abs(st[5]).max() > 0 and np.abs(st[7]).max() > 0
