"""GPU gradient post-processing (csrc/sparc_grad.cu through the C ABI) against outputs of the
reference's own grad.py (tests/golden/grad_small.npz) and against the oracle at full size."""
import os
import sys

import numpy as np
import pytest
import torch

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
from oracle import grad_oracle as go  # noqa: E402

from sparc_flows_gb300 import fits  # noqa: E402
from sparc_flows_gb300 import gradient as G  # noqa: E402

pytestmark = pytest.mark.gpu
GOLD = np.load(os.path.join(ROOT, "tests", "golden", "grad_small.npz"))


def rel(a, b):
    a = a.detach().cpu().numpy() if torch.is_tensor(a) else np.asarray(a)
    return float(np.linalg.norm(a - b) / np.linalg.norm(b))


def cu(a):
    return torch.as_tensor(np.ascontiguousarray(a), dtype=torch.float64, device="cuda")


@pytest.mark.parametrize("it", [0, 1])
def test_gradient_matches_reference_main(it):
    g = G.gradient_psi(cu(GOLD[f"it{it}_kernels"]), cu(GOLD[f"it{it}_hessians"]), cu(GOLD["rho"]))
    assert rel(g, GOLD[f"it{it}_gradient"]) < 1e-13


def test_update_directions_match_reference_main():
    p0, b0 = G.update_direction("sd", cu(GOLD["it0_gradient"]))
    assert rel(p0, GOLD["it0_update"]) == 0.0 and b0 == 0.0
    p1, b1 = G.update_direction("cg", cu(GOLD["it1_gradient"]), cu(GOLD["it0_gradient"]), cu(GOLD["it0_update"]))
    assert rel(p1, GOLD["it1_update"]) < 1e-14
    assert abs(b1 - go.cg_beta(GOLD["it1_gradient"], GOLD["it0_gradient"])) <= 1e-12 * abs(b1)


@pytest.mark.parametrize("it", [0, 1])
def test_linesearch_models_match_reference_main(it):
    t = G.linesearch_models(cu(GOLD[f"it{it}_model"]), cu(GOLD[f"it{it}_update"]), GOLD["eps"])
    for i in range(len(GOLD["eps"])):
        assert rel(t[i], GOLD[f"it{it}_test_{i + 1}"]) < 1e-15


def test_filter_options_match_reference_functions():
    a = cu(GOLD["smooth_in"])
    one = torch.ones_like(a)
    wide = 1e9  # filterx with this width is the identity up to FFT rounding
    assert rel(G.filter_and_symmetrize(a, one, None, "smooth", nk=wide), GOLD["smooth_out"]) < 1e-13
    assert rel(G.filter_and_symmetrize(a, one, "sym", None, nk=wide), GOLD["sym_out"]) < 1e-13
    assert rel(G.filter_and_symmetrize(a, one, None, None, nk=5), GOLD["filterx_nk5"]) < 1e-13
    assert rel(G.filter_and_symmetrize(a, one, None, "gaussian", 3.0, nk=wide), GOLD["gauss3_out"]) < 1e-13


@pytest.mark.parametrize("nx,nz,nsrc", [(512, 300, 32), (384, 301, 5), (1024, 17, 1)])
def test_gradient_full_size_against_oracle(nx, nz, nsrc):
    rng = np.random.default_rng(nx + nz)
    kern = rng.standard_normal((nsrc, nz, nx)) * 1e-3
    hess = rng.standard_normal((nsrc, nz, nx)) ** 2 * 1e2
    rho = np.exp(np.linspace(10.0, 0.0, nz))
    want = go.gradient_psi(kern, hess, rho)
    got = G.gradient_psi(cu(kern), cu(hess), cu(rho))
    assert rel(got, want) < 1e-12


def test_gradient_is_deterministic():
    rng = np.random.default_rng(1)
    kern, hess = cu(rng.standard_normal((8, 300, 512))), cu(rng.random((8, 300, 512)))
    rho = cu(np.linspace(2.0, 1.0, 300))
    a = G.gradient_psi(kern, hess, rho)
    b = G.gradient_psi(kern, hess, rho)
    assert torch.equal(a, b)


def test_hestenes_stiefel_and_lbfgs_against_oracle():
    rng = np.random.default_rng(2)
    n = (300, 512)
    g, gp, pp = (rng.standard_normal(n) for _ in range(3))
    p, beta = G.update_direction("hs", cu(g), cu(gp), cu(pp))
    b_ref = np.sum(g * (g - gp)) / np.sum((g - gp) * pp)
    assert abs(beta - b_ref) <= 1e-12 * abs(b_ref)
    assert rel(p, -g + b_ref * pp) < 1e-13
    S = [rng.standard_normal(n) for _ in range(4)]
    Y = [s * (1.0 + rng.random(n)) for s in S]  # positive curvature pairs
    want = go.lbfgs_direction(g, S, Y)
    got = G.lbfgs_direction(cu(g), [cu(s) for s in S], [cu(y) for y in Y])
    assert rel(got, want) < 1e-12
    assert rel(G.lbfgs_direction(cu(g), [], []), -g) == 0.0


def _params_i(directory, model):
    return (f"character (LEN = *), PARAMETER :: directory = '{directory}/'\n"
            f"character (LEN = *), PARAMETER :: file_data = '{model}'\n")


def test_grad_main_file_contract(tmp_path, monkeypatch):
    """Two iterations of ``python grad.py algo=cg eps...`` against the reference's files."""
    data = tmp_path / "data"
    (data / "kernel").mkdir(parents=True)
    (data / "update").mkdir()
    nsrc, nz = int(GOLD["nsrc"]), int(GOLD["nz"])
    np.savetxt(data / "master.pixels", np.linspace(-20, 20, nsrc))
    back = np.ones((nz, 6))
    back[:, 2] = GOLD["rho"]
    np.savetxt(tmp_path / "model", back)
    (tmp_path / "params.i").write_text(_params_i(str(data), str(tmp_path / "model")))
    monkeypatch.chdir(tmp_path)
    for it in range(2):
        for s in range(nsrc):
            fits.write(str(data / "kernel" / f"kernel_psi_{s + 1:02d}.fits"), GOLD[f"it{it}_kernels"][s][:, None, :])
            fits.write(str(data / "kernel" / f"hessian_{s + 1:02d}.fits"), GOLD[f"it{it}_hessians"][s][:, None, :])
        fits.write(str(data / "update" / f"model_psi_{it:02d}.fits"), GOLD[f"it{it}_model"][:, None, :])
        (data / "update" / f"misfit_{it:02d}").write_text("")
        assert G.main(["algo=cg", *[str(e) for e in GOLD["eps"]]]) == 0
        rd = lambda n: fits.read(str(data / "update" / n))[:, 0, :]  # noqa: E731
        assert rel(rd(f"gradient_psi_{it:02d}.fits"), GOLD[f"it{it}_gradient"]) < 1e-13
        assert rel(rd(f"update_psi_{it:02d}.fits"), GOLD[f"it{it}_update"]) < 1e-12
        for i in range(len(GOLD["eps"])):
            assert rel(rd(f"test_psi_{i + 1}.fits"), GOLD[f"it{it}_test_{i + 1}"]) < 1e-12
    assert np.array_equal(np.load(data / "epslist.npz")["1"], GOLD["epslist_1"])


def test_bad_arguments_fail_loudly():
    a = cu(np.ones((20, 500)))  # 500 is not in the FFT table
    with pytest.raises(Exception, match="FFT table"):
        G.gradient_psi(a, a, cu(np.ones(20)))
