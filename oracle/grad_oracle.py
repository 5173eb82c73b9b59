"""CPU oracle of the gradient post-processing (test infrastructure only).

A NumPy restatement of the reference's grad.py, used by the tests as the checker of the GPU
gradient path (sparc_flows_gb300/gradient.py and csrc/sparc_grad.cu).  Nothing in the
product imports it.  Arrays are (nz, nx) with x fastest, the (nx, 1, nz) Fortran order of
the reference's FITS files read in NumPy order.

Pinned against the reference itself: tests/golden/make_grad_golden.py runs grad.py's own
main() (two iterations, steepest descent then conjugate gradient) and its filter functions
with only file I/O and plotting stubbed, and tests/test_grad_oracle.py checks this module
against those outputs.

Followed lines (grad.py):
  precondition     188-196  kernel and |hessian| sums over sources, hessian * rho(z),
                            normalised by its maximum, floored at 5e-3
  filterx           42-52   Gaussian in x-wavenumber, exp(-k^2 / (2 nk^2)), rfft / irfft
  filterz           54-98   'gaussian' (scipy gaussian_filter1d along z, mode reflect,
                            truncate 4) and 'smooth' (11-point filter, 2-point ends)
  (anti)symmetrize 100-101  0.5 (a -/+ a reversed in x)
  filter_and_symmetrize 109-117
  rms              107
  steepest descent 208-211, conjugate gradient (Polak-Ribiere) 220-250
  create_ls_model  351-364  model + eps * update / max(update) * rms(model)
  L-BFGS           258-325  the reference's branch cannot run (np.dot with one argument,
                            undefined sound_speed_perturbed); restated here as the
                            published two-loop recursion (Nocedal and Wright, Numerical
                            Optimization, 2nd ed., Algorithm 7.4) with m = 4 pairs and
                            H0 = s.y / y.y, which is what those lines set out to compute.
"""
from __future__ import annotations

import numpy as np

HESS_FLOOR = 5e-3      # grad.py:196
FILTERX_NK = 30        # grad.py:111
ZSIGMA = 2.0           # grad.py:200
SMOOTH_COEFFS = (0.75390625, 0.41015625, -0.234375, 0.087890625, -0.01953125, 0.001953125)  # grad.py:70-75


def precondition(kernels: np.ndarray, hessians: np.ndarray, rho: np.ndarray, floor: float = HESS_FLOOR):
    """grad.py:188-196: (sum of kernels, preconditioner).  kernels, hessians: (nsrc, nz, nx)."""
    tot = np.zeros(kernels.shape[1:])
    hess = np.zeros(kernels.shape[1:])
    for s in range(kernels.shape[0]):
        tot += kernels[s]
        hess += np.abs(hessians[s])
    hess = hess * rho[:, None]
    hess = hess / np.abs(hess).max()
    hess[hess < floor] = floor
    return tot, hess


def filterx(kern: np.ndarray, nk: float = FILTERX_NK) -> np.ndarray:
    """grad.py:42-52 along the last (x) axis."""
    nx = kern.shape[-1]
    k = np.fft.rfftfreq(nx, 1.0 / nx)
    filt = np.exp(-k ** 2 / (2 * nk ** 2))
    return np.fft.irfft(np.fft.rfft(kern, axis=-1) * filt, axis=-1).real


def gaussian_weights(sigma: float, truncate: float = 4.0) -> np.ndarray:
    """Normalised Gaussian taps of scipy.ndimage.gaussian_filter1d (radius int(truncate sigma + 0.5))."""
    r = int(truncate * float(sigma) + 0.5)
    x = np.arange(-r, r + 1)
    w = np.exp(-0.5 / (sigma * sigma) * x ** 2)
    return w / w.sum()


def reflect_index(i: int, n: int) -> int:
    """scipy.ndimage mode 'reflect' (d c b a | a b c d | d c b a)."""
    p = i % (2 * n)
    return p if p < n else 2 * n - 1 - p


def filterz_gaussian(arr: np.ndarray, sigma: float) -> np.ndarray:
    """grad.py:96-97: gaussian_filter1d along z (axis 0 here), mode reflect, truncate 4."""
    nz = arr.shape[0]
    w = gaussian_weights(sigma)
    r = (len(w) - 1) // 2
    out = np.zeros_like(arr)
    for k in range(nz):
        acc = np.zeros(arr.shape[1:])
        for j in range(-r, r + 1):
            acc = acc + w[j + r] * arr[reflect_index(k + j, nz)]
        out[k] = acc
    return out


def filterz_smooth(arr: np.ndarray) -> np.ndarray:
    """grad.py:68-87: 11-point symmetric filter for k = 5..nz-6, two-point means for k = 1..3 and
    nz-5..nz-2; rows 1..nz-1 are replaced by the temporary, so rows 4 and nz-1 (never set in
    it) become zero; row 0 is kept."""
    nz = arr.shape[0]
    c = SMOOTH_COEFFS
    temp = np.zeros_like(arr)
    for k in range(5, nz - 5):
        temp[k] = (c[0] * arr[k] + 0.5 * c[1] * (arr[k - 1] + arr[k + 1]) + 0.5 * c[2] * (arr[k - 2] + arr[k + 2])
                   + 0.5 * c[3] * (arr[k - 3] + arr[k + 3]) + 0.5 * c[4] * (arr[k - 4] + arr[k + 4])
                   + 0.5 * c[5] * (arr[k - 5] + arr[k + 5]))
    temp[nz - 5:nz - 1] = 0.5 * (arr[nz - 4:] + arr[nz - 6:nz - 2])
    temp[1:4] = 0.5 * (arr[:3] + arr[2:5])
    out = arr.copy()
    out[1:nz] = temp[1:nz]
    return out


def symmetrize(arr: np.ndarray, sign: int) -> np.ndarray:
    """grad.py:100-101 along x: sign -1 antisymmetrize, +1 symmetrize."""
    return 0.5 * (arr + sign * arr[..., ::-1])


def filter_and_symmetrize(totkern, hess, sym=None, z_filt_algo="gaussian", z_filt_pix=0.3, nk=FILTERX_NK):
    """grad.py:109-117."""
    kern = totkern / hess
    kern = filterx(kern, nk)
    if sym == "sym":
        kern = symmetrize(kern, +1)
    elif sym == "asym":
        kern = symmetrize(kern, -1)
    if z_filt_algo == "gaussian":
        kern = filterz_gaussian(kern, z_filt_pix)
    elif z_filt_algo == "smooth":
        kern = filterz_smooth(kern)
    elif z_filt_algo is not None:
        raise ValueError(f"z filter {z_filt_algo!r} not restated")
    return kern


def gradient_psi(kernels, hessians, rho):
    """grad.py:188-200 as main() runs it."""
    tot, hess = precondition(kernels, hessians, rho)
    return filter_and_symmetrize(tot, hess, z_filt_algo="gaussian", z_filt_pix=ZSIGMA, sym="asym")


def rms(arr):
    """grad.py:107."""
    return np.sqrt(np.sum(arr ** 2) / np.prod(arr.shape))


def sd_update(grad):
    """grad.py:208-211."""
    return -grad


def cg_beta(grad, lastgrad):
    """grad.py:220-240, Polak-Ribiere."""
    beta = np.sum(grad * (grad - lastgrad))
    beta /= np.sum(lastgrad ** 2.0)
    return beta


def cg_update(grad, lastgrad, lastupdate):
    """grad.py:242-250."""
    beta = cg_beta(grad, lastgrad)
    return -grad + beta * lastupdate, beta


def lbfgs_direction(grad, s_hist, y_hist):
    """Two-loop recursion (Nocedal and Wright, Algorithm 7.4): s_hist, y_hist oldest first
    (at most m = 4 pairs, grad.py:258).  Returns the descent direction -H grad."""
    q = grad.copy()
    alphas = []
    rhos = [1.0 / np.sum(y * s) for s, y in zip(s_hist, y_hist)]
    for i in range(len(s_hist) - 1, -1, -1):
        a = rhos[i] * np.sum(s_hist[i] * q)
        alphas.append(a)
        q = q - a * y_hist[i]
    alphas = alphas[::-1]
    if s_hist:
        gamma = np.sum(s_hist[-1] * y_hist[-1]) / np.sum(y_hist[-1] ** 2)
    else:
        gamma = 1.0
    r = gamma * q
    for i in range(len(s_hist)):
        b = rhos[i] * np.sum(y_hist[i] * r)
        r = r + s_hist[i] * (alphas[i] - b)
    return -r


def ls_models(model, update, eps_list):
    """grad.py:351-364 (kind 'linear') for every eps of the line search."""
    update = update.copy()
    updatemax = update.max()
    if updatemax != 0:
        update /= updatemax
    scale = rms(model)
    if scale == 0:
        scale = 1
    return [model + e * update * scale for e in eps_list]
