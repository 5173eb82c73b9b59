"""Known-answer tests that pin the CPU oracle (FFT, spectral and compact derivatives, RK)."""
import numpy as np
import pytest

from oracle import oracle as O
from sparc_flows_gb300 import model as M
from sparc_flows_gb300.config import RunConfig


@pytest.mark.parametrize("n", [12, 64, 256, 384, 512])
def test_fft_matches_numpy(n):
    rng = np.random.default_rng(n)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    ref = np.fft.fft(x)
    got = O.fft(x.real, x.imag, -1)
    assert np.abs(got - ref).max() <= 1e-13 * np.abs(ref).max()
    back = O.fft(got.real, got.imag, +1) / n
    assert np.abs(back - x).max() < 1e-14 * np.abs(x).max() * n


@pytest.fixture(scope="module")
def small_sim():
    run = RunConfig(nx=64, nz=60, xlength_cm=100e8, nsteps=30, flows=True)
    model = M.polytrope(60)
    sim = O.OracleSim(run, model)
    yield run, model, sim
    sim.close()


def test_ddx_trig_exact(small_sim):
    run, _, sim = small_sim
    nx, nz = run.nx, run.nz
    x = np.arange(nx) / nx
    f = np.zeros((nz, nx))
    df = np.zeros((nz, nx))
    for k in range(nz):
        m = 1 + k % 7
        f[k] = np.sin(2 * np.pi * m * x) + 0.3 * np.cos(2 * np.pi * (m + 3) * x)
        df[k] = 2 * np.pi * m * np.cos(2 * np.pi * m * x) - 0.3 * 2 * np.pi * (m + 3) * np.sin(2 * np.pi * (m + 3) * x)
    got = sim.ddx(f)
    sx = sim.getd("stretchx")
    assert np.abs(got - df * sx).max() <= 1e-12 * np.abs(df * sx).max()
    # Nyquist mode is annihilated (eyekx(nx/2+1) = i*pi, dropped by c2r)
    nyq = np.cos(np.pi * np.arange(nx))[None, :].repeat(nz, 0)
    assert np.abs(sim.ddx(nyq)).max() < 1e-10
    # agrees with numpy's rfft/irfft restatement
    assert np.abs(got - O.np_ddx(f, sx)).max() <= 1e-12 * np.abs(got).max()


@pytest.mark.parametrize("ibc", [0, 1, 2, 3])
def test_dbyd2_c_matches_numpy(ibc):
    rng = np.random.default_rng(ibc)
    B = rng.standard_normal((300, 9))
    pre = rng.standard_normal((300, 9))
    a = O.dbyd2(B, ibc, preset=pre)
    b = O.np_dbyd2(B, ibc, preset=pre)
    assert np.abs(a - b).max() <= 1e-13 * np.abs(b).max()


def test_dbyd2_single_precision_coefficients():
    """d2i, C1, C2 of dbyd2.f are implicit REAL: a linear function's derivative carries the
    float32 rounding of the coefficients, not the exact value."""
    n = 300
    s = np.linspace(0.0, 1.0, n)
    d = O.dbyd2(s[:, None].copy(), 1)[:, 0]
    interior = d[2:n - 2]
    c1 = np.float32(np.float32(np.float32(n - 1) * np.float32(7.0)) / np.float32(9.0))
    c2 = np.float32(np.float32(n - 1) / np.float32(36.0))
    rhs = (2 * float(c1) + 4 * float(c2)) / (n - 1)
    # away from the boundaries the solution is the interior RHS divided by 1 + 2/3 (alpha=1/3 float)
    alpha = float(np.float32(1.0) / np.float32(3.0))
    assert abs(interior[n // 2] - rhs / (1 + 2 * alpha)) < 1e-12
    assert abs(interior[n // 2] - 1.0) > 1e-12  # differs from the exact slope at float32 level


def test_dbyd2_converges_sixth_order():
    errs = []
    for n in (40, 80, 160):
        s = np.linspace(0.0, 1.0, n)
        f = np.sin(3.0 * s)
        d = O.dbyd2(f[:, None].copy(), 1)[:, 0]
        errs.append(np.abs(d[n // 4:3 * n // 4] - 3.0 * np.cos(3.0 * s[n // 4:3 * n // 4])).max())
    # interior 6th order until the float32 coefficient floor (~1e-7) is reached
    assert errs[1] < errs[0] / 20 or errs[1] < 1e-6
    assert errs[2] < 1e-6


def test_rk_betas_and_amplification(small_sim):
    _, _, sim = small_sim
    dt = sim.getd("deltat")
    b = [sim.getd(f"betas{i}") / dt for i in range(5)]
    opt = [1.0, 0.5, float(np.float32(0.1665579725791151184)), float(np.float32(0.03950410250586729987)),
           float(np.float32(0.007810706393337838236))]
    assert b[0] == 0.0
    # amplification polynomial 1 + z + b5 z^2 + b5 b4 z^3 + ... equals the optimals (step.f90:28-40)
    assert abs(b[4] - opt[1]) < 1e-15
    assert abs(b[4] * b[3] - opt[2]) < 1e-15
    assert abs(b[4] * b[3] * b[2] - opt[3]) < 1e-15
    assert abs(b[4] * b[3] * b[2] * b[1] - opt[4]) < 1e-15


def test_forward_run_is_finite_and_linear():
    run = RunConfig(nx=64, nz=60, xlength_cm=100e8, nsteps=60, flows=True)
    model = M.polytrope(60)
    psi = M.gaussian_psi(run, model, 0.05, sx=8.0)
    outs = []
    for scale in (1.0, 2.0):
        sim = O.OracleSim(run, model)
        sim.set_psi(psi)
        sim.set_forward_source(0.0, M.SPATIAL_GAUSSIAN, 0.5, M.TEMPORAL_RICKER, 0.003, 80)
        # scale the source by rescaling the state after one step: linear system
        s = sim.run_steps(run.nsteps)
        outs.append(s)
        sim.close()
    assert np.all(np.isfinite(outs[0]))
    assert np.abs(outs[0]).max() > 0
    assert np.array_equal(outs[0], outs[1])  # deterministic


@pytest.mark.parametrize("kst,allx", [(6, False), (2, False), (2, True)])
def test_filter_coverage_options(kst, allx):
    """FILTER_VARS_2D writes rows kst..nz-1 (1-based) of columns [npmlhor, nx-npmlhor+1] (or all
    columns): 11-point rows 6..nz-5, 2-point averages on rows 2..5 and nz-4..nz-1
    (physics2d.f90:524-556)."""
    nz, nx = 60, 64
    run = RunConfig(nx=nx, nz=nz, xlength_cm=100e8, nsteps=2, flows=False, filter_kst=kst, filter_all_x=allx)
    sim = O.OracleSim(run, M.polytrope(nz))
    a6 = np.random.default_rng(kst).standard_normal((6, nz, nx))
    sim.set_state(a6)
    sim.apply_filter()
    out = sim.get("a").reshape(6, nz, nx)
    sim.close()
    ref = a6.copy()
    t = O.np_filter_z(a6[:, :, :].transpose(1, 0, 2))   # (nz, 6, nx)
    t = t.transpose(1, 0, 2)
    for k in list(range(1, 5)) + list(range(nz - 5, nz - 1)):
        t[:, k] = 0.5 * (a6[:, k + 1] + a6[:, k - 1])
    nh = run.npmlhor
    cols = slice(0, nx) if allx else slice(nh - 1, nx - nh + 1)
    rows = slice(kst - 1, nz - 1)
    ref[:, rows, cols] = t[:, rows, cols]
    assert np.abs(out - ref).max() <= 1e-14 * np.abs(ref).max()
