"""What the reference-style kernel is: kernel_psi of the continuous (time-reversal) adjoint and
PRODUCE_KERNELS (kernels.f90:209-358, 495-513) against the exact discrete gradient dL/dpsi of the
same waveform misfit (discrete_adjoint.py), on one 128 x 300 case of 900 steps.

Below the receiver layer, kernel_psi times the cell height dz (the kernel is a density, the
gradient a per-grid-point derivative on a grid stretched by a factor ~1000 over depth) is the
exact gradient times one constant: every 20-row band of rows 140..239 correlates to better than
0.99 (0.995-0.998 on a GB300) with the same least-squares scale (within 3 % of the median).  In
the top 20 rows -- the receiver and adjoint-source row o_rad and the top PML -- the time-reversed
continuous adjoint is not the discrete adjoint and the two disagree (correlation near 0).
Central differences along directions confined to rows 120..239 give ratios of one sign within
25 % of each other (12 % on a GB300), where directions over the whole flow envelope, which reach
into the top layer, gave ratios from -2e4 to -4e3 (unweighted pairing)."""
import numpy as np
import pytest
import torch

from sparc_flows_gb300 import model as M
from sparc_flows_gb300.config import RunConfig

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def gradients():
    from sparc_flows_gb300.autograd import seismograms
    from sparc_flows_gb300.discrete_adjoint import ExactGradient, records
    from sparc_flows_gb300.pipeline import FwdAdjKernels, receiver_columns
    from sparc_flows_gb300.solver import WaveSolver

    run = RunConfig(nx=128, nz=300, xlength_cm=200e8, nsteps=900, flows=True)
    model = M.polytrope(300)
    pt = torch.as_tensor(M.gaussian_psi(run, model, M.psi_amplitude_for_peak(run, model, 240.0)), device="cuda")
    rcv = receiver_columns(run, n=32, x0=-62.0, dx=4.0)
    spec = M.SourceSpec(-20.0)
    ws = WaveSolver(run, model, nbatch=1, precision=64, psi=pt.cpu().numpy())
    ws.set_forward_sources([spec])
    eg = ExactGradient(ws, rcv, segment=100)
    with torch.no_grad():
        data = records(pt, eg).clone()
    psi = (0.5 * pt).clone().requires_grad_(True)
    (0.5 * ((records(psi, eg) - data) ** 2).sum()).backward()
    gex = psi.grad.detach().clone()
    dz = ws.unstretch_t.reshape(-1, 1).double()
    ws.close()
    pipe = FwdAdjKernels(run, model, [spec], psi=np.zeros((300, 128)), precision=64, receivers=rcv)
    psi2 = (0.5 * pt).clone().requires_grad_(True)
    (0.5 * ((seismograms(psi2, pipe) - data) ** 2).sum()).backward()
    kref = psi2.grad.detach().clone()

    def loss(p):
        with torch.no_grad():
            return 0.5 * float(((seismograms(p, pipe) - data) ** 2).sum())

    env = pt.abs() / pt.abs().max()
    yield dict(gex=gex, kref=kref, dz=dz, env=env, psi=psi.detach(), loss=loss, pt=pt)
    pipe.close()


def _fit(a, e):
    return float((a * e).sum() / (a * a).sum()), float((a * e).sum() / torch.sqrt((a * a).sum() * (e * e).sum()))


def test_kernel_times_dz_is_the_gradient_below_the_receiver_layer(gradients):
    g = gradients
    a, e, mask = g["kref"] * g["dz"], g["gex"], g["env"] > 1e-3
    scales = []
    for k0 in range(140, 240, 20):
        m = mask[k0:k0 + 20]
        scale, corr = _fit(a[k0:k0 + 20][m], e[k0:k0 + 20][m])
        assert abs(corr) > 0.99, (k0, corr)
        scales.append(scale)
    med = float(np.median(scales))
    assert max(abs(s / med - 1.0) for s in scales) < 0.03, scales
    # the top 20 rows (o_rad and the top PML) do not follow
    m = mask[280:]
    _, corr_top = _fit(a[280:][m], e[280:][m])
    assert abs(corr_top) < 0.5, corr_top


def test_finite_differences_below_the_receiver_layer_give_one_ratio(gradients):
    g = gradients
    gen = torch.Generator(device="cpu").manual_seed(1)
    rows = torch.zeros_like(g["env"])
    rows[120:240] = 1.0
    ratios = []
    for _ in range(3):
        n = torch.randn(tuple(g["pt"].shape), generator=gen, dtype=torch.float64)
        n = torch.nn.functional.avg_pool2d(n[None, None], 5, 1, 2)[0, 0].to("cuda")
        d = g["env"] * rows * n
        d = d * (1e-4 * float(g["pt"].abs().max()) / float(d.abs().max()))
        fd = (g["loss"](g["psi"] + d) - g["loss"](g["psi"] - d)) / 2.0
        ratios.append(fd / float((g["kref"] * g["dz"] * d).sum()))
    r = np.asarray(ratios)
    assert np.all(np.sign(r) == np.sign(r[0]))
    assert float(np.abs(r / r.mean() - 1.0).max()) < 0.25, ratios
