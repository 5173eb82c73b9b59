"""The gradient post-processing oracle against outputs of the reference's own grad.py
(tests/golden/grad_small.npz, made by tests/golden/make_grad_golden.py)."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
from oracle import grad_oracle as go  # noqa: E402

G = np.load(os.path.join(ROOT, "tests", "golden", "grad_small.npz"))


def rel(a, b):
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.mark.parametrize("it", [0, 1])
def test_gradient_matches_reference_main(it):
    g = go.gradient_psi(G[f"it{it}_kernels"], G[f"it{it}_hessians"], G["rho"])
    assert rel(g, G[f"it{it}_gradient"]) < 1e-13


def test_steepest_descent_then_conjugate_gradient():
    assert np.array_equal(go.sd_update(G["it0_gradient"]), G["it0_update"])
    u, beta = go.cg_update(G["it1_gradient"], G["it0_gradient"], G["it0_update"])
    assert rel(u, G["it1_update"]) < 1e-14
    assert beta != 0.0


@pytest.mark.parametrize("it", [0, 1])
def test_line_search_models(it):
    tests = go.ls_models(G[f"it{it}_model"], G[f"it{it}_update"], list(G["eps"]))
    for i, t in enumerate(tests):
        assert rel(t, G[f"it{it}_test_{i + 1}"]) < 1e-15


def test_epslist_records_the_steps():
    e = G["epslist_1"]
    assert np.array_equal(e[0], G["eps"]) and not e[1:].any()


def test_filter_options_outside_main():
    a = G["smooth_in"]
    assert rel(go.filterz_smooth(a), G["smooth_out"]) < 1e-15
    assert (go.filterz_smooth(a)[4] == 0).all() and (go.filterz_smooth(a)[-1] == 0).all()
    assert rel(go.symmetrize(a, +1), G["sym_out"]) < 1e-15
    assert rel(go.filterx(a, 5), G["filterx_nk5"]) < 1e-14
    assert rel(go.filterz_gaussian(a, 3.0), G["gauss3_out"]) < 1e-14


def test_reflect_index_matches_scipy_mode():
    from scipy.ndimage import correlate1d
    x = np.arange(5.0)
    for i in range(-12, 17):
        w = np.zeros(2 * 20 + 1)
        # a single tap at offset i picks x[reflect(k + i)] for k = 0
        w[20 + i] = 1.0
        assert correlate1d(x, w, mode="reflect")[0] == x[go.reflect_index(i, 5)]


def test_lbfgs_two_loop_is_the_bfgs_matrix_recursion():
    """The two-loop direction equals -H g with H from the dense BFGS update
    H <- (I - rho s y^T) H (I - rho y s^T) + rho s s^T over the pairs, oldest first, starting
    from H0 = (s.y / y.y) I of the newest pair; it satisfies the newest secant H y = s."""
    rng = np.random.default_rng(0)
    n = 6
    A = rng.standard_normal((n, n))
    A = A @ A.T + n * np.eye(n)
    S = [rng.standard_normal(n) for _ in range(4)]
    Y = [A @ s for s in S]
    g = rng.standard_normal(n)
    H = (S[-1] @ Y[-1]) / (Y[-1] @ Y[-1]) * np.eye(n)
    for s, y in zip(S, Y):
        r = 1.0 / (y @ s)
        V = np.eye(n) - r * np.outer(y, s)
        H = V.T @ H @ V + r * np.outer(s, s)
    assert np.allclose(go.lbfgs_direction(g, S, Y), -H @ g, rtol=1e-12, atol=1e-14)
    assert np.allclose(go.lbfgs_direction(Y[-1], S, Y), -S[-1], rtol=1e-12)
    assert np.allclose(go.lbfgs_direction(g, [], []), -g)
