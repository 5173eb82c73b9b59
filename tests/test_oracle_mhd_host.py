"""The displacement oracle's option 18, MP_MHD_PML_2D_DISPL (physics2d.f90:719-938), on the host:
with the field off it is option 17 without flows except at the boundary rows (its top row is not
zeroed and d p/dz takes ibc 0 where option 17 takes ibc 2), and a current-free field couples
into the records while the run stays bounded."""
import numpy as np

from oracle import oracle as O
from sparc_flows_gb300 import model as M
from sparc_flows_gb300.config import RunConfig

RUN = RunConfig(nx=128, nz=300, xlength_cm=200e8, nsteps=160, flows=False)


def _sim(b_gauss=None, nsteps=150):
    model = M.polytrope(300)
    s = O.OracleSim(RUN, model)
    if b_gauss is not None:
        s.set_magnetic(*M.potential_field(RUN.nx, model, RUN.xlength_cm, b_gauss))
    spec = M.SourceSpec(-20.0)
    s.set_forward_source(spec.xloc, spec.spatial, spec.sigma, spec.temporal, spec.nu0, RUN.nsteps + 8)
    rec = s.run_steps(nsteps)
    a = s.get("a").reshape(6, RUN.nz, RUN.nx)
    s.close()
    return rec, a


def _rel(x, y):
    return float(np.linalg.norm(x - y) / np.linalg.norm(y))


def test_option18_without_field_is_option17_away_from_the_boundary_rows():
    r17, a17 = _sim()
    r18, a18 = _sim(0.0)
    assert _rel(r18, r17) < 1e-2
    for v in (0, 2, 3, 5):
        assert _rel(a18[v, 30:-30], a17[v, 30:-30]) < 1e-3, v


def test_option18_field_couples_and_stays_bounded():
    r0, a0 = _sim(0.0)
    r1, a1 = _sim(100.0)
    assert np.isfinite(a1).all() and np.abs(a1).max() < 1.0
    assert 1e-6 < _rel(r1, r0) < 1e-1


def test_option18_needs_a_run_without_flow():
    s = O.OracleSim(RUN.replace(flows=True), M.polytrope(300))
    try:
        with np.testing.assert_raises(ValueError):
            s.set_magnetic(np.zeros((RUN.nz, RUN.nx)), np.zeros((RUN.nz, RUN.nx)))
    finally:
        s.close()
