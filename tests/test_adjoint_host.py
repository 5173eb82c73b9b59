"""The discrete adjoint's step algebra (discrete_adjoint.StepOperators) on the CPU: with the
oracle's primitives standing in for the device ones (its ddx, dense matrices of its dbyd2, a
matrix product for the column operator), one step equals the oracle's restatement of STEP
(step.f90:43-119) with MP_QUIET_PML_2D_DISPL (physics2d.f90:943-1094), the tabulated z filter
equals its FILTER_VARS_2D (physics2d.f90:509-583), and the stage and step transposes pass
dot-product tests."""
import numpy as np
import torch

from oracle import oracle as O
from sparc_flows_gb300 import model as M
from sparc_flows_gb300.config import RunConfig
from sparc_flows_gb300.discrete_adjoint import StepOperators, filter_matrix

F64 = torch.float64


class CpuOps(StepOperators):
    """StepOperators whose primitives are the oracle's (CPU, FP64); the stage, step and transpose
    algebra is the class's own."""

    def __init__(self, sim, run):  # the device set-up of StepOperators is replaced, not called
        nx, nz = run.nx, run.nz
        self.nx, self.nz, self.nb = nx, nz, 1
        nbt, ntp, nh = run.npmlbot, run.npmltop, run.npmlhor
        self.nzpml, self.nhx = nbt + ntp, 2 * nh
        self.prow = torch.as_tensor(list(range(nbt)) + list(range(nz - ntp, nz)))
        self.xcol = torch.as_tensor(list(range(nh)) + list(range(nx - nh, nx)))
        get = lambda n: torch.as_tensor(sim.get(n))  # noqa: E731
        plane = lambda n: get(n).reshape(nz, nx)  # noqa: E731
        self.gp0, self.gr0 = plane("gradp0_z"), plane("gradrho0_z")
        self.c2rho0, self.rho0, self.rhoinv = plane("c2rho0"), plane("rho0"), plane("rhoinv")
        self.g = get("g").reshape(nz, 1)
        self.az, self.bz = plane("az")[self.prow], plane("bzpml")[self.prow]
        self.ax, self.bx = get("axpml").reshape(nz, self.nhx), get("bxpml").reshape(nz, self.nhx)
        st = sim.get("stretch")
        self.ut = float(sim.get("unstretch")[nz - 1])
        self.dt = sim.getd("deltat")
        self.betas = [sim.getd(f"betas{i}") for i in range(5)]
        self.k_inj, self.k_obs = sim.geti("e_rad"), sim.geti("o_rad")
        self.stretchx = sim.getd("stretchx")
        self.M, self.MT = {}, {}
        for ibc in (1, 2, 3):
            m = st[:, None] * O.dbyd2(np.eye(nz), ibc)
            self.M[ibc], self.MT[ibc] = torch.as_tensor(m), torch.as_tensor(m.T.copy())
        pre = np.zeros((nz, 1))
        pre[nz - 1] = 1.0
        self.m3p = torch.as_tensor(st[:, None] * O.dbyd2(np.zeros((nz, 1)), 3, preset=pre)).reshape(1, nz, 1)
        Fm = filter_matrix(nz, run.filter_kst - 1)
        self.Fm, self.FmT = torch.as_tensor(Fm), torch.as_tensor(Fm.T.copy())
        self.fi0, self.fi1 = (0, nx - 1) if run.filter_all_x else (nh - 1, nx - nh)

    def dx(self, f):
        return torch.as_tensor(O.np_ddx(f.numpy(), self.stretchx))

    def colmat(self, W, f, i0=0, i1=None):
        i1 = self.nx - 1 if i1 is None else i1
        out = f.clone()
        out[..., i0:i1 + 1] = torch.einsum("km,...mj->...kj", W, f[..., i0:i1 + 1])
        return out


def _sim():
    run = RunConfig(nx=128, nz=300, xlength_cm=200e8, nsteps=40, flows=True)
    model = M.polytrope(300)
    psi = M.gaussian_psi(run, model, M.psi_amplitude_for_peak(run, model, 240.0))
    sim = O.OracleSim(run, model)
    sim.set_psi(psi)
    spec = M.SourceSpec(-20.0)
    sim.set_forward_source(spec.xloc, spec.spatial, spec.sigma, spec.temporal, spec.nu0, run.nsteps + 8)
    return run, sim


def _state(sim, run):
    nx, nz = run.nx, run.nz
    a = sim.get("a").reshape(6, nz, nx)
    X = torch.as_tensor(a[[0, 2, 3, 5]][None].copy())
    Pz = torch.as_tensor(sim.get("pmlvars").reshape(1, 2, run.npmlbot + run.npmltop, nx))
    Px = torch.as_tensor(sim.get("pmlvarsx").reshape(1, 2, nz, 2 * run.npmlhor))
    return X, Pz, Px


def _rel(a, b):
    return float((a - b).norm() / b.norm())


def test_filter_matrix_equals_oracle_filter():
    run, sim = _sim()
    ops = CpuOps(sim, run)
    rng = np.random.default_rng(0)
    a6 = rng.standard_normal((6, run.nz, run.nx))
    sim.set_state(a6)
    sim.apply_filter()
    want = sim.get("a").reshape(6, run.nz, run.nx)
    got = ops.filt(torch.as_tensor(a6)).numpy()
    sim.close()
    assert np.abs(got - want).max() <= 1e-14 * np.abs(want).max()


def test_step_equals_oracle_step():
    run, sim = _sim()
    ops = CpuOps(sim, run)
    sim.run_steps(30)
    X, Pz, Px = _state(sim, run)
    assert float(Pz.abs().max()) > 0 and float(Px.abs().max()) > 0
    t = sim.geti("time")
    nz, nx = run.nz, run.nx
    rho0 = sim.get("rho0").reshape(nz, nx)
    forcing = sim.get("vr")[:nx] * sim.get("fwdsource")[t] * sim.getd("delta_width") / rho0[ops.k_inj]
    v0x = torch.as_tensor(sim.get("v0x").reshape(nz, nx))
    v0z = torch.as_tensor(sim.get("v0z").reshape(nz, nx))
    got = ops.step(X, Pz, Px, v0x, v0z, torch.as_tensor(forcing)[None])[:3]
    sim.step()
    want = _state(sim, run)
    sim.close()
    for g, w in zip(got, want):
        assert _rel(g, w) < 1e-12, _rel(g, w)


def _shapes(ops):
    return ((1, 4, ops.nz, ops.nx), (1, 2, ops.nzpml, ops.nx), (1, 2, ops.nz, ops.nhx))


def _dot(xs, ys):
    return sum(float((x * y).sum()) for x, y in zip(xs, ys))


def test_stage_and_step_transposes():
    run, sim = _sim()
    ops = CpuOps(sim, run)
    v0x = torch.as_tensor(sim.get("v0x").reshape(run.nz, run.nx))
    v0z = torch.as_tensor(sim.get("v0z").reshape(run.nz, run.nx))
    sim.close()
    gen = torch.Generator().manual_seed(1)
    u = [torch.randn(s, generator=gen, dtype=F64) for s in _shapes(ops)]
    lam = [torch.randn(s, generator=gen, dtype=F64) for s in _shapes(ops)]
    zeros = [torch.zeros_like(u[0][:, 0])] * 4
    # one stage
    Ru = ops.rhs(*u, v0x, v0z)[:3]
    RTl = ops.rhs_T(*lam, v0x, v0z, zeros)[:3]
    lhs, rhs = _dot(lam, Ru), _dot(RTl, u)
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs)
    # one step (the source is affine and left out)
    Su = ops.step(*u, v0x, v0z)[:3]
    STl = ops.step_T(*lam, v0x, v0z, [zeros] * 5)[:3]
    lhs, rhs = _dot(lam, Su), _dot(STl, u)
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs)
