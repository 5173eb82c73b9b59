"""GPU parity at the configurations the short parity tests do not reach, each through the C ABI
against the FP64 CPU oracle (physics2d.f90:943-1094, step.f90:43-119):

- the plain FP64 configuration at its full size and length: nx = 256 over 200 Mm, nz = 300
  polytrope, no flow, one Gaussian x Ricker source at x = 0, 1800 steps of 2 s;
- a 384-column grid (the radix-3 Stockham FFT of the row pass and the generic column kernel);
- a batch with a background per solve (stream function and sound-speed bump differ from solve
  to solve, as the uneven batch builds them).

FP64 plans must equal the oracle to 1e-10 rel-L2 in v_z (seismograms) and in the final state;
FP32 plans of the 384-column and per-solve cases must stay within 1e-4 of the FP64 plans.
"""
import numpy as np
import pytest

from oracle import oracle as O
from sparc_flows_gb300 import model as M

pytestmark = pytest.mark.gpu

FP64_TOL = 1e-10   # rel-L2, FP64 GPU path vs the FP64 oracle
FP32_TOL = 1e-4    # rel-L2, FP32 GPU path vs the FP64 GPU path


def rel_l2(a, b):
    a = np.asarray(a, dtype=np.float64)
    b = np.asarray(b, dtype=np.float64)
    return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))


def oracle_run(run, model, spec, psi=None, cmul=None):
    sim = O.OracleSim(run, model, cmul=cmul)
    if psi is not None:
        sim.set_psi(psi)
    sim.set_forward_source(spec.xloc, spec.spatial, spec.sigma, spec.temporal, spec.nu0, run.nsteps + 8)
    seis = sim.run_steps(run.nsteps)
    a = sim.get("a").reshape(6, run.nz, run.nx)[[0, 2, 3, 5]]  # xi_x, xi_z, v_x, v_z
    sim.close()
    return seis, a


def gpu_run(run, model, specs, psi=None, cmul=None, precision=64):
    from sparc_flows_gb300.solver import WaveSolver
    ws = WaveSolver(run, model, nbatch=len(specs), precision=precision, cmul=cmul, psi=psi)
    ws.set_forward_sources(specs)
    seis = ws.forward().double().cpu().numpy()
    st = ws.state().double().cpu().numpy()
    desc = ws.describe()
    ws.check()
    ws.close()
    return seis, st, desc


@pytest.fixture(scope="module")
def plain64():
    run, model, specs, psi, cmul = M.workload("plain64")
    assert (run.nx, run.nz, run.nsteps, run.flows) == (256, 300, 1800, False)
    assert run.xlength_cm == 200e8 and len(specs) == 1 and specs[0].xloc == 0.0
    seis, st, _ = gpu_run(run, model, specs)
    return run, model, specs, seis, st


def test_plain64_full_length_matches_oracle(plain64):
    """The plain FP64 configuration exactly as the benchmark runs it (1800 steps): v_z -- the
    surface records and the final v_z field -- within 1e-10 of the oracle.  The other fields of
    the final state are held to 1e-9: after 1800 steps xi_x differs by 2.2e-10 (a GB300 run).
    xi_x is the field this configuration amplifies most: in the oracle, a relative perturbation
    of 1e-15 of the state at step 300 grows to 1.1e-12 in xi_x by step 1800, against 2.1e-13 in
    xi_z, 6.1e-14 in v_x and 5.0e-14 in v_z, so the two codes' per-step rounding differences
    (their FFTs and solve orders differ) show first in xi_x."""
    run, model, specs, seis, st = plain64
    seis_o, a_o = oracle_run(run, model, specs[0])
    assert seis.shape[1:] == seis_o.shape and np.abs(seis_o).max() > 0
    errs = [rel_l2(st[0, f], a_o[f]) for f in range(4)]
    assert rel_l2(seis[0], seis_o) < FP64_TOL, errs
    assert errs[3] < FP64_TOL, errs
    assert max(errs) < 10 * FP64_TOL, errs


def _case384(nsteps, nx=384):
    run = M.uneven_run(nx, nsteps)
    model = M.polytrope(300)
    psi = M.gaussian_psi(run, model, M.psi_amplitude_for_peak(run, model, 240.0))
    return run, model, psi, M.c_bump(run, model)


def test_nx384_fp64_matches_oracle():
    """384 columns: the mixed-radix (3 x 2^7) row FFT and the FP64 partitioned column pass."""
    run, model, psi, cmul = _case384(150)
    spec = M.SourceSpec(20.0)
    seis, st, desc = gpu_run(run, model, [spec], psi=psi, cmul=cmul)
    seis_o, a_o = oracle_run(run, model, spec, psi=psi, cmul=cmul)
    assert np.abs(seis_o).max() > 0
    assert rel_l2(seis[0], seis_o) < FP64_TOL
    for f in range(4):
        assert rel_l2(st[0, f], a_o[f]) < FP64_TOL, f


@pytest.mark.parametrize("nx,column", [(384, "col_band_kernel<32,10,384,300,1>"),  # specialised, TMA-staged
                                       (192, "col_band_kernel<32,10,0,0,0>")])  # generic grid
def test_fp32_tracks_fp64(nx, column):
    run, model, psi, cmul = _case384(300, nx)
    specs = [M.SourceSpec(-30.0), M.SourceSpec(45.0)]
    s64, st64, _ = gpu_run(run, model, specs, psi=psi, cmul=cmul)
    s32, st32, desc = gpu_run(run, model, specs, psi=psi, cmul=cmul, precision=32)
    assert desc["column"] == column, desc
    assert rel_l2(s32, s64) < FP32_TOL
    for b in range(2):
        for f in range(4):
            assert rel_l2(st32[b, f], st64[b, f]) < 10 * FP32_TOL, (b, f)


def _per_solve_case(nsteps):
    """Three solves of one grid, each with its own flow amplitude, sound-speed bump and source,
    built as the uneven batch builds its groups."""
    run = M.uneven_run(256, nsteps)
    model = M.polytrope(300)
    unit = M.gaussian_psi(run, model, M.psi_amplitude_for_peak(run, model, 1.0))
    solves = [(260.0, 0.045, -40.0), (35.0, 0.012, 5.0), (150.0, 0.0, 60.0)]
    psis = [unit * v for v, _, _ in solves]
    cmuls = [M.c_bump(run, model, amp=d) for _, d, _ in solves]
    specs = [M.SourceSpec(x) for _, _, x in solves]
    return run, model, psis, cmuls, specs


def test_per_solve_backgrounds_fp64_match_oracle():
    run, model, psis, cmuls, specs = _per_solve_case(150)
    seis, st, _ = gpu_run(run, model, specs, psi=psis, cmul=cmuls)
    for b in range(len(specs)):
        seis_o, a_o = oracle_run(run, model, specs[b], psi=psis[b], cmul=cmuls[b])
        assert np.abs(seis_o).max() > 0
        assert rel_l2(seis[b], seis_o) < FP64_TOL, b
        for f in range(4):
            assert rel_l2(st[b, f], a_o[f]) < FP64_TOL, (b, f)
    # the backgrounds really differ: solve 1 against solve 0's background with solve 1's source
    seis_x, _ = oracle_run(run, model, specs[1], psi=psis[0], cmul=cmuls[0])
    assert rel_l2(seis_x, seis[1]) > 1e-4


def test_per_solve_backgrounds_fp32_track_fp64():
    run, model, psis, cmuls, specs = _per_solve_case(300)
    s64, st64, _ = gpu_run(run, model, specs, psi=psis, cmul=cmuls)
    s32, st32, _ = gpu_run(run, model, specs, psi=psis, cmul=cmuls, precision=32)
    for b in range(len(specs)):
        assert rel_l2(s32[b], s64[b]) < FP32_TOL, b
        for f in range(4):
            assert rel_l2(st32[b, f], st64[b, f]) < 10 * FP32_TOL, (b, f)
