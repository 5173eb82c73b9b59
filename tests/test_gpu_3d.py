"""3-D GPU solver (sparc3d_*, csrc/sparc_3d.cu) against the 3-D CPU oracle (sparc_oracle3d.c),
and its FP32 plan against its FP64 plan."""
import numpy as np
import pytest
import torch

from oracle.oracle3d import Sim3D
from sparc_flows_gb300 import capi
from sparc_flows_gb300 import model as M
from sparc_flows_gb300.solver3d import WaveSolver3D

pytestmark = pytest.mark.gpu

NX = NY = 64
NZ = 100
XL = 200e8
OBS = -100e5  # records near the source depth, so that the first records carry signal


def _inputs(nb=2, nsteps=12):
    model = M.polytrope(NZ)
    x = (np.arange(NX) - NX / 2) / NX
    X, Y = np.meshgrid(x, x)
    pats = np.stack([np.exp(-((X - 0.1 * b) ** 2 + (Y + 0.05 * b) ** 2) / 0.003) for b in range(nb)])
    amp = np.sin(np.arange(nsteps + 5) * 0.35) * 1e-6
    zz = np.linspace(-1, 1, NZ)[:, None, None]
    env = np.exp(-(zz / 0.3) ** 2)
    v0x = 0.02 * env * np.sin(2 * np.pi * X)[None] * np.cos(2 * np.pi * Y)[None]
    v0y = -0.015 * env * np.cos(2 * np.pi * X)[None] * np.sin(4 * np.pi * Y)[None]
    v0z = 0.01 * env * np.cos(2 * np.pi * (X + Y))[None]
    return model, pats, amp, (v0x, v0y, v0z)


def _gpu(precision, nsteps, flows=True, nb=2):
    model, pats, amp, v0 = _inputs(nb, nsteps)
    ws = WaveSolver3D(NX, NY, model, XL, nbatch=nb, precision=precision, flows=flows, steps_out=5,
                      obsheight_cm=OBS)
    if flows:
        ws.set_flow(*v0)
    ws.set_source(pats, amp)
    ws.reset(0)
    seis = ws.forward(nsteps)
    st = ws.state().double().cpu().numpy()
    ws.close()
    return st, seis.double().cpu().numpy()


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


@pytest.mark.parametrize("flows", [True, False])
def test_fp64_matches_oracle(flows):
    nsteps, nb = 12, 2
    st, seis = _gpu(64, nsteps, flows, nb)
    model, pats, amp, v0 = _inputs(nb, nsteps)
    for b in range(nb):
        s = Sim3D(NX, NY, NZ, model, XL, XL, steps_out=5, obsheight_cm=OBS)
        if flows:
            s.set_flow(*v0)
        s.set_source(pats[b], amp)
        rec = s.run(nsteps)
        want = s.state()
        s.close()
        assert rec.shape[0] == seis.shape[0] == 3 and np.abs(rec[-1]).max() > 0
        for v in range(6):
            assert rel(st[v, :, b], want[v]) < 1e-10, (b, v, rel(st[v, :, b], want[v]))
        assert rel(seis[:, b], rec) < 1e-10


def test_fp32_tracks_fp64():
    st32, s32 = _gpu(32, 40)
    st64, s64 = _gpu(64, 40)
    for v in range(6):
        assert rel(st32[v], st64[v]) < 1e-4, (v, rel(st32[v], st64[v]))
    assert rel(s32, s64) < 1e-4


def test_bad_grid_is_rejected():
    with pytest.raises(capi.SparcError, match="FFT table"):
        WaveSolver3D(500, 64, M.polytrope(NZ), XL)
