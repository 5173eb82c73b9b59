"""3-D adjoint run, kernel integral and HBM checkpoints (pipeline3d.FwdAdjKernels3D) against the
3-D CPU oracle: the reference's kernel-mode adjoint (displacement.f90:615-627) with LAGRANGE_INTERP
(physics.f90:678-737) and the flow negated (driver.f90:144-147), the kernel integrands of
kernels.f90:293-358 extended by the y terms, records paired as kernels.f90:215, 258."""
import numpy as np
import pytest

from oracle.oracle3d import Sim3D
from sparc_flows_gb300 import model as M
from sparc_flows_gb300.config import RunConfig

pytestmark = pytest.mark.gpu

NX = NY = 64
NZ = 100
XL = 200e8
OBS = -100e5  # records near the source depth, so that the first records carry signal
SO, NSTEPS, K = 5, 40, 15


def _inputs(nb=2, nsteps=NSTEPS):
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


def _gpu(precision, k_every, nb=2):
    from sparc_flows_gb300.pipeline3d import FwdAdjKernels3D
    model, pats, amp, v0 = _inputs(nb)
    pipe = FwdAdjKernels3D(NX, NY, model, XL, pats, amp, NSTEPS, flow=v0, precision=precision, steps_out=SO,
                           checkpoint_every=k_every, obsheight_cm=OBS)
    seis, kacc = pipe.run_all()
    out = (seis.double().cpu().numpy(), kacc.cpu().numpy(), pipe.adj.state().double().cpu().numpy())
    pipe.close()
    return out


def rel(a, b):
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def _oracle(b):
    """Forward, adjoint and kernel integrands of solve b on the CPU, as the pipeline runs them."""
    model, pats, amp, v0 = _inputs()
    fw = Sim3D(NX, NY, NZ, model, XL, XL, steps_out=SO, obsheight_cm=OBS)
    fw.set_flow(*v0)
    fw.set_source(pats[b], amp)
    o = fw.get_int("o_rad")
    recs, vz = [], []
    for _ in range(NSTEPS):
        if fw.advance() % SO == 0:
            recs.append(fw.kernel_record())
            vz.append(fw.state()[5, o].copy())
    z = model[:, 0]
    scale = 2.0 / (z[o + 1] - z[o - 1]) / fw.profile("rho0")[o]
    fw.close()
    nrec = len(recs)
    run = RunConfig(nx=NX, nz=NZ, nsteps=NSTEPS, timestep=2.0, outputcad=SO * 2.0, cadforcing=SO * 2.0)
    idx, w = M.lagrange_weights(run, NSTEPS + 1, run.num_steps, nrec)
    ad = Sim3D(NX, NY, NZ, model, XL, XL, steps_out=SO, obsheight_cm=OBS)
    ad.set_flow(*[-v for v in v0])
    ad.set_adjoint_source(np.stack(vz)[::-1], w[1:], idx[1:], scale)
    out = np.zeros((5, NZ, NY, NX))
    done = 0
    for ja in range(nrec):
        n = 1 if ja == 0 else SO
        for _ in range(n):
            ad.advance()
        done += n
        ad.kernels_accumulate(recs[nrec - 1 - ja], out)
    for _ in range(NSTEPS - done):
        ad.advance()
    st = ad.state()
    ad.close()
    return np.stack(vz), out, st


def test_fp64_adjoint_and_kernels_match_oracle():
    seis, kacc, adj = _gpu(64, K)
    for b in range(2):
        vz, kern, st = _oracle(b)
        assert rel(seis[:, b], vz) < 1e-10, b
        for v in range(6):
            assert rel(adj[v, :, b], st[v]) < 1e-10, (b, v, rel(adj[v, :, b], st[v]))
        for f in range(5):
            assert np.abs(kern[f]).max() > 0, (b, f)
            assert rel(kacc[f, :, b], kern[f]) < 1e-10, (b, f, rel(kacc[f, :, b], kern[f]))


@pytest.mark.parametrize("precision", [64, 32])
def test_checkpointed_equals_stored(precision):
    """Segments of 15 steps recomputed from their checkpoints give the same kernels, bit for bit,
    as one segment holding every record."""
    s1, k1, a1 = _gpu(precision, K)
    s2, k2, a2 = _gpu(precision, NSTEPS)
    assert np.array_equal(s1, s2) and np.array_equal(k1, k2) and np.array_equal(a1, a2)


def test_fp32_tracks_fp64():
    s64, k64, _ = _gpu(64, K)
    s32, k32, _ = _gpu(32, K)
    assert rel(s32, s64) < 1e-4
    for f in range(5):
        assert rel(k32[f], k64[f]) < 1e-3, (f, rel(k32[f], k64[f]))
