"""The 3-D CPU oracle (sparc_oracle3d.c): its derivatives against analytic derivatives and the
2-D oracle's dbyd2, and x <-> y symmetry of a run with a symmetric source and no flow."""
import numpy as np
import pytest

from oracle import oracle as O
from oracle.oracle3d import Sim3D
from sparc_flows_gb300 import model as M


@pytest.fixture(scope="module")
def sim():
    s = Sim3D(64, 64, 100, M.polytrope(100), 200e8, 200e8)
    yield s
    s.close()


def test_horizontal_derivatives_are_spectral(sim):
    nx, ny, nz = 64, 64, 100
    x = np.arange(nx) / nx
    y = np.arange(ny) / ny
    X, Y = np.meshgrid(x, y)  # (ny, nx)
    f = np.sin(2 * np.pi * 3 * X) * np.cos(2 * np.pi * 5 * Y) + np.cos(2 * np.pi * 31 * X)
    F = np.broadcast_to(f, (nz, ny, nx)).copy()
    sx, sy = sim.get_double("stretchx"), sim.get_double("stretchy")
    dfx = (2 * np.pi * 3 * np.cos(2 * np.pi * 3 * X) * np.cos(2 * np.pi * 5 * Y)
           - 2 * np.pi * 31 * np.sin(2 * np.pi * 31 * X)) * sx
    dfy = -2 * np.pi * 5 * np.sin(2 * np.pi * 3 * X) * np.sin(2 * np.pi * 5 * Y) * sy
    assert np.abs(sim.ddx(F) - dfx).max() < 1e-10 * np.abs(dfx).max()
    assert np.abs(sim.ddy(F) - dfy).max() < 1e-10 * np.abs(dfy).max()


def test_vertical_derivative_is_dbyd2_times_stretch(sim):
    rng = np.random.default_rng(0)
    F = rng.standard_normal((100, 64, 64))
    st = sim.profile("stretch")
    for bc in (0, 1):
        want = np.zeros_like(F)
        L = O.lib()
        import ctypes
        flat = np.ascontiguousarray(F.reshape(100, -1))
        out = np.zeros_like(flat)
        dp = ctypes.POINTER(ctypes.c_double)
        L.orc_dbyd2(out.ctypes.data_as(dp), flat.ctypes.data_as(dp), flat.shape[1], 100, bc)
        want = (out * st[:, None]).reshape(F.shape)
        assert np.array_equal(sim.ddz(F, bc), want)


def test_symmetric_source_gives_symmetric_wavefield():
    nx = ny = 64
    s = Sim3D(nx, ny, 100, M.polytrope(100), 200e8, 200e8)
    x = (np.arange(nx) - nx / 2) / nx
    X, Y = np.meshgrid(x, x)
    s.set_source(np.exp(-(X ** 2 + Y ** 2) / 0.002), np.sin(np.arange(40) * 0.3) * 1e-6)
    seis = s.run(6, max_records=1)
    a = s.state()
    s.close()
    assert np.isfinite(a).all() and np.abs(a[5]).max() > 0
    assert seis.shape == (1, ny, nx)
    # xi_x(z, y, x) = xi_y(z, x, y), v_z symmetric under x <-> y
    assert np.allclose(a[0], a[1].transpose(0, 2, 1), rtol=0, atol=1e-12 * np.abs(a[0]).max())
    assert np.allclose(a[5], a[5].transpose(0, 2, 1), rtol=0, atol=1e-12 * np.abs(a[5]).max())
