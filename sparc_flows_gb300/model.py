"""Synthetic inputs for the wave solver: background model, flows, sound-speed bumps, sources.

The background is written in the reference's 6-column model format (r/Rsun, c [cm/s],
rho [g/cc], p [dyn/cm^2], g [cm/s^2], Gamma1; deepest row first), the format solar_data
reads (initialize.f90:731-776).  No dataset is involved: every workload is generated here
from seeded, analytic definitions.
"""
from __future__ import annotations

import dataclasses
import math

import numpy as np

from .config import DIMC, DIMRHO, RSUN_CM, RunConfig

NUPEAK = float(np.float32(0.0017))   # params.i:66, single-precision literal
NUWIDTH = float(np.float32(0.0055))


def polytrope(nz: int = 300, m: float = 1.5, gamma1: float = 5.0 / 3.0, g_ms2: float = 274.0,
              z0_mm: float = 0.5, zbot_mm: float = -25.0, rho_surface: float = 2.78e-7,
              top_steps: float = 12.5) -> np.ndarray:
    """Adiabatic polytrope on a grid uniform in acoustic travel time.

    T is proportional to depth d = z0 - z, so c^2 = Gamma1 g d / (m+1), rho ~ d^m and
    p = rho g d / (m+1) (hydrostatic).  The nz points are uniform in travel time
    tau(d) = 2 sqrt(d/A), A = Gamma1 g/(m+1), from the bottom zbot up to ``top_steps``
    travel-time steps below z0 (d_top = A (top_steps dtau)^2 / 4: 41 km for the defaults, so
    the grid ends at z = +0.46 Mm).  Ending closer to the singular surface (c, rho -> 0 at z0)
    makes the (m+1) c^2/d d/dz term of the displacement equations stiff: with dt = 2 s a grid
    ending half a step below z0 diverges within 20 steps, and from about 8 steps it is stable.
    rho is normalised to ``rho_surface`` at z = 0.  Returns an (nz, 6) array in the reference
    model format.
    """
    g = g_ms2 * 100.0                       # cm/s^2
    z0 = z0_mm * 1e8                         # cm
    A = gamma1 * g / (m + 1.0)
    dmax = z0 - zbot_mm * 1e8
    tau_max = 2.0 * math.sqrt(dmax / A)
    dtau = tau_max / (nz - 1 + top_steps)
    tau = tau_max - dtau * np.arange(nz)     # deepest first
    d = A * tau * tau / 4.0
    z = z0 - d
    c = np.sqrt(A * d)
    rho = rho_surface * (d / z0) ** m
    p = rho * g * d / (m + 1.0)
    out = np.zeros((nz, 6))
    out[:, 0] = 1.0 + z / RSUN_CM
    out[:, 1] = c
    out[:, 2] = rho
    out[:, 3] = p
    out[:, 4] = g
    out[:, 5] = gamma1
    return out


def load_model(path: str, nz: int) -> np.ndarray:
    """Read the first nz rows of a 6-column model file (solar_data, initialize.f90:740-744)."""
    rows = []
    with open(path) as f:
        for line in f:
            if line.strip():
                rows.append([float(v.replace("D", "E").replace("d", "e")) for v in line.split()[:6]])
            if len(rows) == nz:
                break
    return np.asarray(rows, dtype=np.float64)


def x_mm(run: RunConfig) -> np.ndarray:
    """Horizontal coordinate in Mm relative to the box centre: (x - 0.5) * xlength."""
    x = np.arange(run.nx, dtype=np.float64) / run.nx
    return (x - 0.5) * run.xlength_cm * 1e-8


def z_mm(model: np.ndarray) -> np.ndarray:
    """Height above the photosphere in Mm for each model row."""
    return (model[:, 0] - 1.0) * RSUN_CM * 1e-8


def gaussian_psi(run: RunConfig, model: np.ndarray, amp: float = 1.0, x0: float = 0.0,
                 sx: float = 8.0, zc: float = -2.3, sz: float = 2.0) -> np.ndarray:
    """Supergranule stream function psi = amp exp(-((x-x0)/sx)^2) exp(-((z-zc)/sz)^2), in Mm.

    Shape (nz, nx), x fastest, the layout of model_psi_lsMM.fits (nz, 1, nx)."""
    X = x_mm(run)[None, :]
    Z = z_mm(model)[:, None]
    return amp * np.exp(-((X - x0) / sx) ** 2) * np.exp(-((Z - zc) / sz) ** 2)


def psi_amplitude_for_peak(run: RunConfig, model: np.ndarray, vx_peak_ms: float, **kw) -> float:
    """Amplitude A of ``gaussian_psi`` giving max |v0x| = vx_peak_ms.

    v0x = -d/dz(rho0 c psi/(Rsun/1 Mm))/rho0 (driver.f90:105-115) is evaluated with second-order
    differences on the model grid; the solver itself uses compact differences, so the realised
    peak agrees to the truncation error of this estimate.
    """
    psi = gaussian_psi(run, model, 1.0, **kw)
    zr = model[:, 0]
    rho = model[:, 2][:, None]
    c = (model[:, 1] / DIMC)[:, None]
    pv = rho * c * psi / (RSUN_CM / 1e8)
    dz = np.gradient(pv, zr, axis=0)
    v0x = -dz / rho
    peak = float(np.max(np.abs(v0x))) * DIMC * 1e-2
    return vx_peak_ms / peak


def c_bump(run: RunConfig, model: np.ndarray, amp: float = 0.05, sigma: float = 5.0, zc: float = -3.0,
           x0: float = 0.0) -> np.ndarray:
    """Multiplier on c: 1 + amp exp(-((x-x0)^2 + (z-zc)^2)/(2 sigma^2)), shape (nz, nx)."""
    X = x_mm(run)[None, :]
    Z = z_mm(model)[:, None]
    return 1.0 + amp * np.exp(-(((X - x0) ** 2) + (Z - zc) ** 2) / (2.0 * sigma * sigma))


# --------------------------------------------------------------------------------------
# Sources: DETERMINE_STATUS (driver.f90:536-553) and FORWARD_SOURCE (driver.f90:1120-1145)
# --------------------------------------------------------------------------------------
SPATIAL_REFERENCE, SPATIAL_GAUSSIAN = 0, 1
TEMPORAL_REFERENCE, TEMPORAL_RICKER = 0, 1


@dataclasses.dataclass
class SourceSpec:
    xloc: float = 0.0                 # Mm from the box centre (master.pixels value)
    spatial: int = SPATIAL_GAUSSIAN
    sigma: float = 0.5                # Mm, Gaussian profile
    temporal: int = TEMPORAL_RICKER
    nu0: float = 0.003                # Hz, Ricker peak frequency


DIMB = (4.0 * np.pi * DIMC ** 2 * DIMRHO) ** 0.5  # magnetic unit, initialize.f90:759


def potential_field(nx: int, model: np.ndarray, xlength_cm: float, b_gauss: float, m: int = 1):
    """A current-free background field for the 2-D MHD step: B = curl(A y) with
    A = (B0 / k) cos(k X) exp(k (z - 1)), k = 2 pi m R / xlength, X the horizontal coordinate and z
    the radius in solar radii, B0 = b_gauss at z = 1; box = -dA/dz, boz = dA/dX as the reference
    forms them from a flux function (physics2d.f90:124-134).  Its curl vanishes, so it needs no
    change of the hydrostatic stratification.  Returns (box, boz), (nz, nx), in units of dimb."""
    X = np.arange(nx) / nx * xlength_cm / RSUN_CM
    k = 2.0 * np.pi * m * RSUN_CM / xlength_cm
    e = np.exp(k * (model[:, 0] - 1.0))[:, None]
    b0 = b_gauss / DIMB
    return -b0 * np.cos(k * X)[None, :] * e, -b0 * np.sin(k * X)[None, :] * e


def source_profile(run: RunConfig, spec: SourceSpec) -> np.ndarray:
    """vr(x): the horizontal source profile (nx,)."""
    nx = run.nx
    x = np.arange(nx, dtype=np.float64) / nx
    l1e8 = float(np.float32(1e-8))    # 10.**(-8) is a single-precision constant (driver.f90:545)
    dx = (x[1] - x[0]) * run.xlength_cm * l1e8
    xd = (x - 0.5) * run.xlength_cm * l1e8 - spec.xloc
    if spec.spatial == SPATIAL_REFERENCE:
        l043 = float(np.float32(0.43))
        with np.errstate(invalid="ignore", divide="ignore"):
            sx = np.sin(l043 * math.pi * xd) / (l043 * math.pi * xd)
        sx[int(np.argmin(np.abs(xd)))] = 1.0
        return np.exp(-(xd * xd) / (400.0 * (dx * dx))) * sx
    return np.exp(-(xd * xd) / (2.0 * spec.sigma * spec.sigma))


def source_time_series(run: RunConfig, spec: SourceSpec, nt: int) -> np.ndarray:
    """fwdsource(k), k = 1..nt at t = (k-1) dt (driver.f90:1128-1133)."""
    t = np.arange(nt, dtype=np.float64) * run.timestep
    if spec.temporal == TEMPORAL_REFERENCE:
        dd = t - 0.5 / NUPEAK
        v = np.cos(2.0 * math.pi * NUPEAK * t) * np.exp(-2.0 * (dd * dd) * (NUWIDTH * NUWIDTH))
        v[np.abs(v) < float(np.float32(0.00001))] = 0.0
        return v * float(np.float32(1e-5))
    arg = math.pi * spec.nu0 * (t - 1.5 / spec.nu0)
    return (1.0 - 2.0 * arg * arg) * np.exp(-arg * arg) * 1e-5


def lagrange_weights(run: RunConfig, nsteps: int, num_steps: int, nsrc_rows: int):
    """LAGRANGE_INTERP (physics.f90:678-737) as per-step (first row index, 7 weights).

    forcing(t) = sum_j w[t, j] * src[idx[t] + j] where src has cadforcing cadence and rows
    beyond its length are zero (driver.f90:584-594)."""
    cad, ts = run.cadforcing, run.timestep
    idx = np.zeros(nsteps, dtype=np.int32)
    w = np.zeros((nsteps, 7))
    for time in range(nsteps):
        xt = float(time) * ts / cad
        time1 = int(math.floor(xt)) + 1
        xt = time * ts
        xs = [(time1 - 4 + j) * cad for j in range(7)]
        use = [xs[j] >= 0 for j in range(4)] + [True, time1 < num_steps, time1 < num_steps - 1]
        idx[time] = time1 - 4
        for j in range(7):
            r = time1 - 4 + j
            if not use[j] or r < 0 or r >= nsrc_rows:
                continue
            den, num = 1.0, 1.0
            for m in range(7):
                if m != j:
                    den *= xs[j] - xs[m]
                    num *= xt - xs[m]
            w[time, j] = num / den
    return idx, w


# --------------------------------------------------------------------------------------
# Benchmark workloads (FP64 plain run, autograd run, source batch)
# --------------------------------------------------------------------------------------
def workload(name: str):
    """Return (RunConfig, model, list[SourceSpec], psi or None, cmul or None) for a workload.

    plain64   : nx=256 over 200 Mm, nz=300 polytrope, no flow, 1 source, 1800 steps (FP64 plain).
    autograd32: nx=512 over 400 Mm, supergranule psi flow (vx peak 240 m/s), 1 source, 3600 steps,
                20-layer bottom PML (10 at the top).
    batch32   : as autograd32 with 32 sources at x = -200 + 12.5 (s + 0.5) Mm and a 5 % Gaussian
                sound-speed bump (sigma 5 Mm at -3 Mm), 3600 steps.
    """
    model = polytrope(300)
    if name == "plain64":
        run = RunConfig(nx=256, nz=300, xlength_cm=200e8, nsteps=1800, flows=False)
        return run, model, [SourceSpec(0.0)], None, None
    # 20 bottom PML layers: with 10, the bottom PML of this polytrope (CFL 0.8 where c is largest)
    # carries a mode growing 0.4 % per step, which FP32 rounding seeds at 1e-7 and brings to O(1)
    # within 3600 steps; from 15 layers on it decays (measured with the FP64 oracle).
    run = RunConfig(nx=512, nz=300, xlength_cm=400e8, nsteps=3600, flows=True, npmlbot=20)
    amp = psi_amplitude_for_peak(run, model, 240.0)
    psi = gaussian_psi(run, model, amp)
    if name == "autograd32":
        return run, model, [SourceSpec(0.0)], psi, None
    if name == "batch32":
        srcs = [SourceSpec(-200.0 + 12.5 * (s + 0.5)) for s in range(32)]
        return run, model, srcs, psi, c_bump(run, model)
    raise KeyError(name)


# --------------------------------------------------------------------------------------
# The uneven batch: solves of different grids, lengths and backgrounds
# --------------------------------------------------------------------------------------
@dataclasses.dataclass
class Solve:
    """One independent solve of the uneven batch."""
    nx: int
    nsteps: int
    vpeak_ms: float      # flow amplitude (max |v0x| of the supergranule stream function)
    dcc: float           # sound-speed bump amplitude dc/c
    xloc: float          # source position, Mm from the box centre


def uneven_solves(n: int = 48, seed: int = 0) -> list[Solve]:
    """n solves, seeded: nx ~ U{256, 384, 512} (0.78125 Mm spacing, so 200 / 300 / 400 Mm boxes),
    steps ~ U{1800, 2700, 3600}, flow amplitude ~ U(0, 300) m/s, dc/c ~ U(0, 0.05), the flow and
    bump shapes of the batch32 workload, source positions uniform over the inner 80 % of the box."""
    rng = np.random.default_rng(seed)
    out = []
    for _ in range(n):
        nx = int(rng.choice([256, 384, 512]))
        steps = int(rng.choice([1800, 2700, 3600]))
        vpeak = float(rng.uniform(0.0, 300.0))
        dcc = float(rng.uniform(0.0, 0.05))
        xloc = float(rng.uniform(-0.4, 0.4)) * nx * 0.78125
        out.append(Solve(nx, steps, vpeak, dcc, xloc))
    return out


def uneven_run(nx: int, nsteps: int) -> RunConfig:
    """Run configuration of one group of the uneven batch (batch32 physics, 20-layer bottom PML)."""
    return RunConfig(nx=nx, nz=300, xlength_cm=nx * 0.78125e8, nsteps=nsteps, flows=True, npmlbot=20)


# ---------------------------------------------------------------------------------------------
# 3-D configuration (256 x 256 x 300, 200 Mm box, 4 sources, axisymmetric outflow): synthetic
# inputs for the option-16 solver (solver3d.py).
# ---------------------------------------------------------------------------------------------
def outflow_3d(nx: int, ny: int, model: np.ndarray, xlength_cm: float, u0_ms: float = 300.0,
               sigma_mm: float = 10.0, zc_mm: float = -2.0, zw_mm: float = 2.0, zret_mm: float = -6.0,
               zwret_mm: float = 3.0):
    """Axisymmetric outflow u_r(r, z) = u0 (r/sigma) exp(1/2 - r^2/(2 sigma^2)) f(z) about the box
    centre, f(z) = exp(-((z-zc)/zw)^2) - a exp(-((z-zret)/zwret)^2), with v_z from
    d(rho0 v_z)/dz = -rho0 div_h(u) integrated upward from the bottom (trapezoid rule in z,
    spectral horizontal divergence).  The deeper return flow (a set so that the integral of
    rho0 f vanishes) closes the mass flux of each column: without it v_z = flux / rho0 grows to
    ~190 km/s where rho0 falls off at the top.  Returns (v0x, v0y, v0z), each (nz, ny, nx),
    nondimensional (cm/s / dimc)."""
    L = xlength_cm * 1e-8
    x = (np.arange(nx) / nx - 0.5) * L
    y = (np.arange(ny) / ny - 0.5) * L
    X, Y = np.meshgrid(x, y)  # (ny, nx), Mm
    r = np.sqrt(X * X + Y * Y)
    z = z_mm(model)
    rho = model[:, 2]
    zc = z * 1e8  # cm
    f1 = np.exp(-((z - zc_mm) / zw_mm) ** 2)
    f2 = np.exp(-((z - zret_mm) / zwret_mm) ** 2)
    w = np.gradient(zc)
    prof = f1 - (np.sum(rho * f1 * w) / np.sum(rho * f2 * w)) * f2
    ur = u0_ms * 100.0 * (r / sigma_mm) * np.exp(0.5 - r * r / (2 * sigma_mm ** 2))  # cm/s
    with np.errstate(invalid="ignore", divide="ignore"):
        cx = np.where(r > 0, X / r, 0.0)
        cy = np.where(r > 0, Y / r, 0.0)
    ux = (ur * cx)[None] * prof[:, None, None]
    uy = (ur * cy)[None] * prof[:, None, None]
    kx = 2 * np.pi * np.fft.fftfreq(nx, d=L * 1e8 / nx)
    ky = 2 * np.pi * np.fft.fftfreq(ny, d=L * 1e8 / ny)
    divh = (np.fft.ifft(1j * kx[None, None, :] * np.fft.fft(ux, axis=2), axis=2).real
            + np.fft.ifft(1j * ky[None, :, None] * np.fft.fft(uy, axis=1), axis=1).real)  # 1/s
    flux = np.zeros_like(divh)
    src = -rho[:, None, None] * divh
    for k in range(1, len(z)):
        flux[k] = flux[k - 1] + 0.5 * (src[k] + src[k - 1]) * (zc[k] - zc[k - 1])
    uz = flux / rho[:, None, None]
    return ux / DIMC, uy / DIMC, uz / DIMC


def point_source_pattern(nx: int, ny: int, xlength_cm: float, xs_mm: float, ys_mm: float) -> np.ndarray:
    """Radial form of the reference's source profile exp(-d^2/(400 dx^2)) sinc(0.43 pi d)
    (driver.f90:541-547) about (xs, ys), d the horizontal distance in Mm: (ny, nx)."""
    L = xlength_cm * 1e-8
    x = (np.arange(nx) / nx - 0.5) * L
    y = (np.arange(ny) / ny - 0.5) * L
    X, Y = np.meshgrid(x, y)
    d = np.sqrt((X - xs_mm) ** 2 + (Y - ys_mm) ** 2)
    dx = L / nx
    return np.exp(-d * d / (400.0 * dx * dx)) * np.sinc(0.43 * d)


def workload_3d(nx: int = 256, ny: int = 256, nz: int = 300, nsrc: int = 4):
    """The 3-D configuration: polytrope, 200 Mm box, outflow, sources at (+-50, +-50) Mm."""
    model = polytrope(nz)
    xl = 200e8
    v0 = outflow_3d(nx, ny, model, xl)
    pos = [(-50.0, -50.0), (50.0, -50.0), (-50.0, 50.0), (50.0, 50.0)][:nsrc]
    pats = np.stack([point_source_pattern(nx, ny, xl, xs, ys) for xs, ys in pos])
    return model, xl, v0, pats
