"""GPU parity: the sm_103a library (through its C ABI) against the FP64 CPU oracle."""
import numpy as np
import pytest

from oracle import oracle as O
from sparc_flows_gb300 import model as M
from sparc_flows_gb300.config import RunConfig

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10   # rel-L2, FP64 GPU path vs the FP64 oracle
FP32_TOL = 1e-4    # rel-L2, FP32 GPU path vs the FP64 GPU path


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def make_case(nx=128, nz=300, nsteps=150, flows=True, bump=True, length=200e8):
    run = RunConfig(nx=nx, nz=nz, xlength_cm=length, nsteps=nsteps, flows=flows)
    model = M.polytrope(nz)
    psi = M.gaussian_psi(run, model, M.psi_amplitude_for_peak(run, model, 240.0)) if flows else None
    cmul = M.c_bump(run, model) if bump else None
    return run, model, psi, cmul


def oracle_for(run, model, psi, cmul, spec):
    sim = O.OracleSim(run, model, cmul=cmul)
    if psi is not None:
        sim.set_psi(psi)
    sim.set_forward_source(spec.xloc, spec.spatial, spec.sigma, spec.temporal, spec.nu0, run.nsteps + 8)
    return sim


def gpu_solver(run, model, psi, cmul, nb=1, precision=64):
    from sparc_flows_gb300.solver import WaveSolver
    return WaveSolver(run, model, nbatch=nb, precision=precision, cmul=cmul, psi=psi)


@pytest.fixture(scope="module")
def case():
    return make_case()


def test_setup_matches_oracle(case):
    run, model, psi, cmul = case
    sim = oracle_for(run, model, psi, cmul, M.SourceSpec(0.0))
    ws = gpu_solver(run, model, psi, cmul)
    nz, nx = run.nz, run.nx
    assert ws.e_rad == sim.geti("e_rad") and ws.o_rad == sim.geti("o_rad")
    assert abs(ws.deltat - sim.getd("deltat")) == 0.0
    for i in range(5):
        assert abs(ws.betas[i] - sim.getd(f"betas{i}")) <= 1e-15 * abs(ws.betas[i])
    st = ws.stretch_t.cpu().numpy()
    # 1/dbyd2(z): z ~ 1 with ~1e-6 spacing near the top, so operation order alone moves the
    # last digits (relative cancellation ~1e-10)
    assert rel_l2(st, sim.get("stretch")) < 1e-9
    gp = sim.get("gradp0_z").reshape(nz, nx)
    fdz = ws.bg["fdz"].cpu().numpy()[0]
    nb_, nt_ = run.npmlbot, run.npmltop
    mine = np.repeat(ws.gradp0_z[:, None], nx, 1)
    mine[:nb_] *= fdz[:nb_]
    mine[nz - nt_:] *= fdz[nb_:]
    assert rel_l2(mine, gp) < 1e-9
    assert rel_l2(ws.g, sim.get("g")) < 1e-12
    v0x = ws.v0x.cpu().numpy()[0]
    v0z = ws.v0z.cpu().numpy()[0]
    assert rel_l2(v0x, sim.get("v0x").reshape(nz, nx)) < 1e-9
    assert rel_l2(v0z, sim.get("v0z").reshape(nz, nx)) < 1e-9
    ax = ws.bg["ax"].cpu().numpy()[0]
    assert rel_l2(ax, sim.get("axpml").reshape(nz, -1)) < 1e-13
    az = ws.bg["az"].cpu().numpy()[0]
    az_o = sim.get("az").reshape(nz, nx)
    assert rel_l2(az, np.concatenate([az_o[:nb_], az_o[nz - nt_:]])) < 1e-13
    sim.close()
    ws.close()


def test_gpu_derivatives_match_oracle(case):
    import torch
    run, model, psi, cmul = case
    sim = oracle_for(run, model, psi, cmul, M.SourceSpec(0.0))
    ws = gpu_solver(run, model, psi, cmul)
    rng = np.random.default_rng(3)
    f = rng.standard_normal((run.nz, run.nx))
    ft = torch.tensor(f, dtype=torch.float64, device="cuda")
    out = torch.empty_like(ft)
    ws.ddx(ft, out, run.nz, ws.stretchx)
    assert rel_l2(out.cpu().numpy(), sim.ddx(f)) < 1e-13
    for ibc in (0, 1, 2, 3):
        pre = rng.standard_normal(run.nx)
        pre_full = np.zeros((run.nz, run.nx))
        if ibc == 2:
            pre_full[0] = pre
        if ibc == 3:
            pre_full[-1] = pre
        # same stretch on both sides: the two 1/dbyd2(z) arrays already differ at ~1e-10
        ref = O.dbyd2(f, ibc, preset=pre_full) * ws.stretch_t.cpu().numpy()[:, None]
        ws.ddz(ft, out, run.nx, ibc, stretch=ws.stretch_t, preset=torch.tensor(pre, device="cuda"))
        # random columns excite the grid-scale modes the compact operator amplifies most, so
        # FMA contraction and the partitioned solve order show up at ~1e-11 here
        assert rel_l2(out.cpu().numpy(), ref) < 1e-10, ibc
    sim.close()
    ws.close()


@pytest.mark.parametrize("flows,bump,kst,allx", [(False, False, 6, False), (True, True, 6, False),
                                                 (True, True, 2, True)])
def test_forward_fp64_matches_oracle(flows, bump, kst, allx):
    run, model, psi, cmul = make_case(flows=flows, bump=bump, nsteps=150)
    run = run.replace(filter_kst=kst, filter_all_x=allx)
    spec = M.SourceSpec(10.0)
    sim = oracle_for(run, model, psi, cmul, spec)
    seis_o = sim.run_steps(run.nsteps)
    a_o = sim.get("a").reshape(6, run.nz, run.nx)
    ws = gpu_solver(run, model, psi, cmul)
    ws.set_forward_sources([spec])
    seis = ws.forward().cpu().numpy()[0]
    st = ws.state().cpu().numpy()[0]
    assert seis.shape == seis_o.shape
    assert np.abs(seis_o).max() > 0
    assert rel_l2(seis, seis_o) < FP64_TOL
    for f, of in zip(range(4), (0, 2, 3, 5)):
        assert rel_l2(st[f], a_o[of]) < FP64_TOL, f
    assert ws.time() == run.nsteps
    sim.close()
    ws.close()


def test_batch_equals_single_runs():
    run, model, psi, cmul = make_case(nsteps=60)
    specs = [M.SourceSpec(-40.0), M.SourceSpec(0.0), M.SourceSpec(35.0)]
    ws = gpu_solver(run, model, psi, cmul, nb=3)
    ws.set_forward_sources(specs)
    batch = ws.forward().cpu().numpy()
    ws.close()
    for i, s in enumerate(specs):
        w1 = gpu_solver(run, model, psi, cmul, nb=1)
        w1.set_forward_sources([s])
        one = w1.forward().cpu().numpy()[0]
        w1.close()
        assert np.array_equal(one, batch[i])


def test_graph_replay_equals_stream_launches():
    run, model, psi, cmul = make_case(nsteps=40)
    ws = gpu_solver(run, model, psi, cmul)
    ws.set_forward_sources([M.SourceSpec(0.0)])
    a = ws.forward(use_graph=True).cpu().numpy()
    b = ws.forward(use_graph=False).cpu().numpy()
    ws.close()
    assert np.array_equal(a, b)


@pytest.fixture(scope="module")
def fp64_300():
    run, model, psi, cmul = make_case(nx=256, nsteps=300, length=400e8)
    spec = M.SourceSpec(0.0)
    w64 = gpu_solver(run, model, psi, cmul, precision=64)
    w64.set_forward_sources([spec])
    s64 = w64.forward().cpu().numpy()
    st64 = w64.state().cpu().numpy()
    w64.close()
    return (run, model, psi, cmul, spec), s64, st64


# column pass variants of FP32 plans: 0 partitioned solve, 1 partitioned solve with TMA tiles,
# 2 geometric band, 3 geometric band with TMA tiles; every block width of the banded pass
@pytest.mark.parametrize("impl,cw", [(0, 32), (1, 32), (2, 32), (2, 16), (2, 8), (3, 32)])
def test_fp32_tracks_fp64(fp64_300, monkeypatch, impl, cw):
    (run, model, psi, cmul, spec), s64, st64 = fp64_300
    monkeypatch.setenv("SPARC_COLUMN_IMPL", str(impl))
    monkeypatch.setenv("SPARC_COLUMN_BLOCK", str(cw))
    w32 = gpu_solver(run, model, psi, cmul, precision=32)
    w32.set_forward_sources([spec])
    s32 = w32.forward().cpu().numpy()
    st32 = w32.state().cpu().numpy()
    w32.check()  # raises on a TMA time-out flag or a non-finite state
    w32.close()
    assert rel_l2(s32, s64) < FP32_TOL
    for f in range(4):
        assert rel_l2(st32[0, f], st64[0, f]) < 10 * FP32_TOL, f


def test_fp32_plans_launch_the_banded_column_pass():
    """FP32 plans of the standard grids run the geometric-band column pass (a silent fallback to
    the partitioned solve would still pass the accuracy tests)."""
    run, model, psi, cmul = make_case(nx=512, nsteps=10, length=400e8)
    w = gpu_solver(run, model, psi, cmul, precision=32)
    d = w.describe()
    w.close()
    assert d["column"].startswith("col_band_kernel<32,10,512,300,1>"), d  # TMA-staged first phase
    assert d["stage_overlap"] == "1", d


def test_stage_overlap_is_bit_identical(monkeypatch):
    """The row pass started on the SMs the column pass's last wave leaves idle, each row block
    waiting for its own solve's column tiles, gives the same bits as the serialised step: state
    and seismograms of 60 steps of four solves, with and without the overlap."""
    run, model, psi, cmul = make_case(nx=512, nsteps=60, length=400e8)
    out = {}
    for ov in ("0", "1"):
        monkeypatch.setenv("SPARC_STAGE_OVERLAP", ov)
        w = gpu_solver(run, model, psi, cmul, nb=4, precision=32)
        assert w.describe()["stage_overlap"] == ov
        w.set_forward_sources([M.SourceSpec(x) for x in (-40.0, -10.0, 15.0, 50.0)])
        seis = w.forward().cpu().numpy()
        out[ov] = (seis, w.state().cpu().numpy())
        w.check()
        w.close()
    assert np.abs(out["0"][0]).max() > 0
    assert np.array_equal(out["0"][0], out["1"][0]) and np.array_equal(out["0"][1], out["1"][1])


def test_fp32_512_columns_track_fp64():
    """On 512-column grids FP32 row passes use the register-resident FFT (FP64 keeps the
    Stockham FFT): seismograms and state of 200 steps against FP64."""
    run, model, psi, cmul = make_case(nx=512, nsteps=200, length=400e8)
    spec = M.SourceSpec(20.0)
    out = {}
    for prec in (64, 32):
        w = gpu_solver(run, model, psi, cmul, precision=prec)
        w.set_forward_sources([spec])
        seis = w.forward().cpu().numpy()
        out[prec] = (seis, w.state().cpu().numpy())
        w.check()
        w.close()
    assert rel_l2(out[32][0], out[64][0]) < FP32_TOL
    for f in range(4):
        assert rel_l2(out[32][1][0, f], out[64][1][0, f]) < 10 * FP32_TOL, f


def test_state_check_detects_divergence():
    """Failure detection on the host side of the ABI: a non-finite state (planted through
    sparc_set_state, no device fault) is reported as SPARC_ERR_NONFINITE; a healthy state's norm
    equals the L2 norm of v_z (rms_hist)."""
    import torch
    from sparc_flows_gb300.capi import SparcError
    run, model, psi, cmul = make_case(nsteps=30)
    ws = gpu_solver(run, model, psi, cmul, nb=2)
    ws.set_forward_sources([M.SourceSpec(0.0), M.SourceSpec(20.0)])
    ws.forward()
    st = ws.state()
    norms = ws.check()
    ref = torch.linalg.vector_norm(st[:, 3].reshape(2, -1), dim=1).cpu().numpy()
    assert np.allclose(norms, ref, rtol=1e-12)
    bad = st.clone()
    bad[1, 3, 100, 7] = float("nan")
    ws.set_state(bad)
    with pytest.raises(SparcError, match="non-finite"):
        ws.check()
    ws.close()
