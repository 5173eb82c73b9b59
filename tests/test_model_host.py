"""Synthetic backgrounds of model.py on the host: the option-12 background field is current-free
(its curl, formed as the reference forms curlboy with ddz and ddx, physics2d.f90:166-168,
vanishes to rounding away from the boundary rows, where dbyd2's one-sided ibc-1 closures leave a
residue the solver's curlboy shares) and has the requested strength at z = 1."""
import numpy as np

from oracle import oracle as O
from sparc_flows_gb300 import model as M
from sparc_flows_gb300.config import RSUN_CM


def test_potential_field_is_current_free():
    nx, xl = 128, 200e8
    model = M.polytrope(300)
    box, boz = M.potential_field(nx, model, xl, 100.0)
    z = model[:, 0]
    stretch = 1.0 / O.dbyd2(z, 1)
    dzbox = O.dbyd2(box, 1) * stretch[:, None]
    dxboz = O.np_ddx(boz, RSUN_CM / xl)
    curl = dzbox - dxboz
    assert np.abs(curl[30:-30]).max() < 1e-10 * np.abs(dzbox).max()  # the closure residue decays as 0.38^d
    k1 = int(np.argmin(np.abs(z - 1.0)))
    bmag = np.sqrt(box[k1] ** 2 + boz[k1] ** 2)
    assert np.allclose(bmag * M.DIMB, 100.0 * np.exp(2 * np.pi * RSUN_CM / xl * (z[k1] - 1.0)), rtol=1e-12)
