"""Exact discrete adjoint of the option-17 step (discrete_adjoint.py): the stage and step
transposes pass dot-product tests against the forward operators (the step against the plan's
fused device step), and the gradient of a seismogram misfit with respect to the stream function
agrees with central finite differences."""
import numpy as np
import pytest
import torch

from sparc_flows_gb300 import model as M
from sparc_flows_gb300.config import RunConfig
from sparc_flows_gb300.pipeline import receiver_columns

pytestmark = pytest.mark.gpu

F64 = torch.float64


def _solver(nsteps=60, nb=2):
    from sparc_flows_gb300.solver import WaveSolver
    run = RunConfig(nx=128, nz=300, xlength_cm=200e8, nsteps=nsteps, flows=True)
    model = M.polytrope(300)
    psi = M.gaussian_psi(run, model, M.psi_amplitude_for_peak(run, model, 240.0))
    ws = WaveSolver(run, model, nbatch=nb, precision=64, psi=psi)
    ws.set_forward_sources([M.SourceSpec(-20.0), M.SourceSpec(25.0)][:nb])
    return run, model, psi, ws


def _rand(shape, seed, dev="cuda"):
    g = torch.Generator(device="cpu").manual_seed(seed)
    return torch.randn(shape, generator=g, dtype=F64).to(dev)


def _dot(xs, ys):
    return sum(float((x * y).sum()) for x, y in zip(xs, ys))


def _shapes(ops):
    return ((ops.nb, 4, ops.nz, ops.nx), (ops.nb, 2, ops.nzpml, ops.nx), (ops.nb, 2, ops.nz, ops.nhx))


def test_stage_transpose_dot_product():
    from sparc_flows_gb300.discrete_adjoint import StepOperators
    run, model, psi, ws = _solver()
    ops = StepOperators(ws)
    v0x, v0z = ws.bg["v0x"][0], ws.bg["v0z"][0]
    sa, sz, sw = _shapes(ops)
    X, Z, W = _rand(sa, 1), _rand(sz, 2), _rand(sw, 3)
    lR, lZ, lW = _rand(sa, 4), _rand(sz, 5), _rand(sw, 6)
    R, RZ, RW, _ = ops.rhs(X, Z, W, v0x, v0z)
    tX, tZ, tW = ops.rhs_T(lR, lZ, lW, v0x, v0z, [torch.zeros_like(X[:, 0])] * 4)[:3]
    lhs = _dot((lR, lZ, lW), (R, RZ, RW))
    rhs = _dot((tX, tZ, tW), (X, Z, W))
    ws.close()
    assert abs(lhs - rhs) <= 1e-11 * max(abs(lhs), abs(rhs)), (lhs, rhs)


def _device_step(ws, eg, a, Pz, Px, time):
    """One fused device step from (a, Pz, Px) at step index time; returns the new state."""
    blob = torch.zeros(eg.row, dtype=torch.uint8, device="cuda")
    blob[:4].view(torch.int32)[0] = time - 1
    va, vz, vw = eg._views(blob)
    va.copy_(a), vz.copy_(Pz), vw.copy_(Px)
    ws.checkpoint_load(blob)
    ws.run_steps(1, None, None, 0)
    out = torch.zeros_like(blob)
    ws.checkpoint_save(out)
    return [t.clone() for t in eg._views(out)]


def test_unfused_step_equals_device_step():
    from sparc_flows_gb300.discrete_adjoint import ExactGradient
    run, model, psi, ws = _solver()
    eg = ExactGradient(ws, receivers=[10, 20], segment=10)
    ws.reset(0)
    ws.run_steps(30, None, None, 0)
    blob = torch.zeros(eg.row, dtype=torch.uint8, device="cuda")
    ws.checkpoint_save(blob)
    a, Pz, Px = [t.clone() for t in eg._views(blob)]
    assert float(a.abs().max()) > 0 and float(Pz.abs().max()) > 0 and float(Px.abs().max()) > 0
    want = _device_step(ws, eg, a, Pz, Px, 30)
    got = eg.ops.step(a, Pz, Px, ws.bg["v0x"][0], ws.bg["v0z"][0], eg._forcing(30))[:3]
    ws.close()
    for g, w in zip(got, want):
        assert float((g - w).norm() / w.norm()) < 1e-12


def test_step_transpose_against_device_step():
    """<l, S u> = <S^T l, u> with S the linear part of the fused device step."""
    from sparc_flows_gb300.discrete_adjoint import ExactGradient
    run, model, psi, ws = _solver()
    eg = ExactGradient(ws, receivers=[10, 20], segment=10)
    ops = eg.ops
    sa, sz, sw = _shapes(ops)
    u = (_rand(sa, 11), _rand(sz, 12), _rand(sw, 13))
    lam = (_rand(sa, 14), _rand(sz, 15), _rand(sw, 16))
    zero = [torch.zeros_like(t) for t in u]
    su = [x - y for x, y in zip(_device_step(ws, eg, *u, time=40), _device_step(ws, eg, *zero, time=40))]
    caches = [[torch.zeros_like(u[0][:, 0])] * 4] * 5
    st = ops.step_T(*lam, ws.bg["v0x"][0], ws.bg["v0z"][0], caches)[:3]
    ws.close()
    lhs, rhs = _dot(lam, su), _dot(st, u)
    assert abs(lhs - rhs) <= 1e-10 * max(abs(lhs), abs(rhs)), (lhs, rhs)


def test_gradient_matches_central_differences():
    """dL/dpsi of L = 1/2 |records(psi) - data|^2 at 32 receivers, 2 sources, 150 steps, against
    central differences along four directions."""
    from sparc_flows_gb300.discrete_adjoint import ExactGradient, records
    run, model, psi_true, ws = _solver(nsteps=150)
    rcv = receiver_columns(run, n=32, x0=-62.0, dx=4.0)
    eg = ExactGradient(ws, rcv, segment=40)
    pt = torch.as_tensor(psi_true, device="cuda")
    with torch.no_grad():
        data = records(pt, eg).clone()
    psi = (0.5 * pt).clone().requires_grad_(True)
    loss = 0.5 * ((records(psi, eg) - data) ** 2).sum()
    loss.backward()
    g = psi.grad.detach().clone()
    assert eg._graph is not None  # the reverse step ran from its CUDA graph
    eager = ExactGradient(ws, rcv, segment=40, use_graph=False)
    eager.forward(psi.detach())
    ge = eager.gradient(psi.detach(), records(psi.detach(), eg) - data)
    assert torch.allclose(ge, g, rtol=1e-12, atol=0.0)
    env = pt.abs() / pt.abs().max()
    dirs = [pt, torch.roll(pt, 9, dims=1), env * _rand(tuple(pt.shape), 21),
            env * torch.sin(torch.arange(pt.shape[1], device="cuda", dtype=F64) * 0.3)[None, :] * pt.abs().max()]
    ratios = []
    for d in dirs:
        eps = 1e-4 * float(pt.abs().max()) / float(d.abs().max())
        with torch.no_grad():
            lp = 0.5 * float(((records(psi.detach() + eps * d, eg) - data) ** 2).sum())
            lm = 0.5 * float(((records(psi.detach() - eps * d, eg) - data) ** 2).sum())
        fd = (lp - lm) / (2 * eps)
        ratios.append(fd / float((g * d).sum()))
    ws.close()
    assert float(loss.detach()) > 0
    for r in ratios:
        assert abs(r - 1.0) < 1e-7, ratios


def test_sound_speed_gradient_matches_central_differences():
    """dL/d(c^2 rho0) (PML profiles fixed) against central differences along three directions:
    data from the plan with a 5 % sound-speed bump, gradient at the unperturbed field."""
    from sparc_flows_gb300.discrete_adjoint import ExactGradient, records
    from sparc_flows_gb300.solver import WaveSolver
    run = RunConfig(nx=128, nz=300, xlength_cm=200e8, nsteps=150, flows=True)
    model = M.polytrope(300)
    psi = torch.as_tensor(M.gaussian_psi(run, model, M.psi_amplitude_for_peak(run, model, 240.0)), device="cuda")
    ws = WaveSolver(run, model, nbatch=2, precision=64, psi=psi.cpu().numpy(), cmul=M.c_bump(run, model))
    ws.set_forward_sources([M.SourceSpec(-20.0), M.SourceSpec(25.0)])
    rcv = receiver_columns(run, n=32, x0=-62.0, dx=4.0)
    eg = ExactGradient(ws, rcv, segment=40)
    c_true = ws.bg["c2rho0"][0].clone()
    with torch.no_grad():
        data = records(psi, eg).clone()
    nz, nx = c_true.shape
    base = c_true[:, :1].expand(nz, nx).contiguous()  # the depth profile without the bump
    eg.set_c2rho0(base)
    rec = eg.forward(psi)
    eg.gradient(psi, rec - data)
    g = eg.last["c2rho0"]
    zc = torch.arange(nz, device="cuda", dtype=F64)[:, None]
    env = torch.exp(-((zc - 200.0) / 40.0) ** 2) * torch.ones((1, nx), device="cuda", dtype=F64)
    dev = {}
    for seed in (31, 32, 33):
        d = env * base * _rand((nz, nx), seed)
        for eps in (1e-4, 1e-5):
            lp_ = []
            for sgn in (1.0, -1.0):
                eg.set_c2rho0(base + sgn * eps * d)
                lp_.append(0.5 * float(((eg.forward(psi) - data) ** 2).sum()))
            dev[(seed, eps)] = (lp_[0] - lp_[1]) / (2 * eps) / float((g * d).sum()) - 1.0
    ws.close()
    for seed in (31, 32, 33):
        # central-difference truncation is O(eps^2): 10x smaller steps, ~100x smaller deviation
        assert abs(dev[(seed, 1e-5)]) < 1e-7, dev
        assert abs(dev[(seed, 1e-5)]) < 0.05 * abs(dev[(seed, 1e-4)]) + 1e-9, dev
