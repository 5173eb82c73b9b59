"""Gradient post-processing on the GPU: the drop-in for the reference's grad.py.

grad.py (run by master.py:21, 212-224 as ``python grad.py algo=<cg|sd|LBFGS> eps1 eps2 ...``
in the code directory after the kernels of every source exist) sums the per-source kernels,
preconditions them by the summed hessian, smooths and antisymmetrises the result, forms the
update direction and writes the line-search models.  Here the array work runs in
csrc/sparc_grad.cu through the C ABI (sparc_gradient, sparc_update_direction,
sparc_lbfgs_direction, sparc_linesearch_models), next to the batched kernels:

  gradient_psi(kernels, hessians, rho)   grad.py:188-200 (K / H, filterx, antisymmetrize,
                                         Gaussian z filter of 2 rows)
  filter_and_symmetrize(totkern, hess)   grad.py:109-117
  update_direction(algo, ...)            grad.py:204-250 (steepest descent, Polak-Ribiere CG)
  lbfgs_direction(grad, s, y)            the two-loop recursion grad.py:257-325 sets out to
                                         compute (its own code cannot run, see the C header)
  linesearch_models(model, update, eps)  grad.py:351-378
  main(argv)                             the file contract of grad.py's main (grad.py:122-432)

Arrays are FP64 CUDA tensors (nz, nx), x fastest, as the kernels the pipeline produces.
"""
from __future__ import annotations

import ctypes
import fnmatch
import os
import sys

import numpy as np
import torch

from . import capi, fits
from .config import parse_params_i

SYM = {None: 0, "sym": 1, "asym": -1}
ZFILT = {None: 0, "none": 0, "gaussian": 1, "smooth": 2}
ALGOS = {"sd": 0, "steepest descent": 0, "cg": 1, "conjugate gradient": 1, "hs": 2, "LBFGS": 3}
LBFGS_M = 4  # grad.py:258


def _stream():
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _p(t: torch.Tensor | None):
    return ctypes.c_void_p(t.data_ptr()) if t is not None else None


def _dev(a, device) -> torch.Tensor:
    t = torch.as_tensor(a, dtype=torch.float64, device=device)
    return t.contiguous()


class Workspace:
    """Device workspace of the gradient calls (no call allocates inside the library)."""

    def __init__(self, nx: int, nz: int, device="cuda"):
        L = capi.lib()
        nbytes = int(L.sparc_grad_workspace_bytes(nx, nz))
        self.buf = torch.empty(nbytes // 8 + 1, dtype=torch.float64, device=device)
        self.nx, self.nz = nx, nz

    @property
    def ptr(self):
        return ctypes.c_void_p(self.buf.data_ptr())


def _work(nx: int, nz: int, device, ws: Workspace | None) -> Workspace:
    if ws is not None and ws.nx * ws.nz >= nx * nz and ws.nx >= nx:
        return ws
    return Workspace(nx, nz, device)


def _gradient(kernels, hessians, rho, *, precondition, sym, z_filt_algo, z_filt_pix, nk, floor,
              ws: Workspace | None = None) -> torch.Tensor:
    kernels = _dev(kernels, "cuda" if not torch.is_tensor(kernels) else kernels.device)
    dev = kernels.device
    if kernels.dim() == 2:
        kernels = kernels.unsqueeze(0)
    hessians = _dev(hessians, dev)
    if hessians.dim() == 2:
        hessians = hessians.unsqueeze(0)
    nsrc, nz, nx = kernels.shape
    if hessians.shape != kernels.shape:
        raise ValueError(f"hessians {tuple(hessians.shape)} != kernels {tuple(kernels.shape)}")
    cfg = capi.SparcGradConfig()
    cfg.nx, cfg.nz, cfg.nsrc = nx, nz, nsrc
    cfg.nk = float(nk)
    cfg.sym = SYM[sym]
    cfg.zfilt = ZFILT[z_filt_algo]
    cfg.zsigma = float(z_filt_pix)
    cfg.hess_floor = float(floor)
    cfg.precondition = 1 if precondition else 0
    rho_t = _dev(rho, dev) if rho is not None else None
    out = torch.empty((nz, nx), dtype=torch.float64, device=dev)
    w = _work(nx, nz, dev, ws)
    L = capi.lib()
    capi.check(L.sparc_gradient(ctypes.byref(cfg), _p(kernels), _p(hessians), _p(rho_t), _p(out), w.ptr, _stream()),
               "sparc_gradient")
    return out


def gradient_psi(kernels, hessians, rho, *, nk=30, sym="asym", z_filt_algo="gaussian", z_filt_pix=2.0,
                 floor=5e-3, ws: Workspace | None = None) -> torch.Tensor:
    """grad.py:188-200: kernels, hessians (nsrc, nz, nx) per source (or already summed, (nz, nx)),
    rho (nz,) the model file's density column.  Returns the gradient (nz, nx)."""
    return _gradient(kernels, hessians, rho, precondition=True, sym=sym, z_filt_algo=z_filt_algo,
                     z_filt_pix=z_filt_pix, nk=nk, floor=floor, ws=ws)


def filter_and_symmetrize(totkern, hess, sym=None, z_filt_algo="gaussian", z_filt_pix=0.3, nk=30,
                          ws: Workspace | None = None) -> torch.Tensor:
    """grad.py:109-117: filterz(sym(filterx(totkern / hess, nk)))."""
    return _gradient(totkern, hess, None, precondition=False, sym=sym, z_filt_algo=z_filt_algo,
                     z_filt_pix=z_filt_pix, nk=nk, floor=0.0, ws=ws)


def update_direction(algo: str, grad, grad_prev=None, update_prev=None, ws: Workspace | None = None):
    """grad.py:204-250.  Returns (update, beta); beta is 0 for steepest descent."""
    code = ALGOS[algo]
    if code == 3:
        raise ValueError("use lbfgs_direction for L-BFGS")
    g = _dev(grad, grad.device if torch.is_tensor(grad) else "cuda")
    n = g.numel()
    gp = _dev(grad_prev, g.device) if code else None
    pp = _dev(update_prev, g.device) if code else None
    p = torch.empty_like(g)
    beta = ctypes.c_double(0.0)
    w = _work(0, 0, g.device, ws)
    L = capi.lib()
    capi.check(L.sparc_update_direction(code, n, _p(g), _p(gp), _p(pp), _p(p), ctypes.byref(beta), w.ptr, _stream()),
               "sparc_update_direction")
    return p, beta.value


def lbfgs_direction(grad, s_hist: list, y_hist: list, ws: Workspace | None = None) -> torch.Tensor:
    """-H grad by the L-BFGS two-loop recursion over the pairs (oldest first)."""
    g = _dev(grad, grad.device if torch.is_tensor(grad) else "cuda")
    S = [_dev(s, g.device) for s in s_hist]
    Y = [_dev(y, g.device) for y in y_hist]
    if len(S) != len(Y):
        raise ValueError("s and y histories differ in length")
    sp = (ctypes.c_void_p * max(len(S), 1))(*[t.data_ptr() for t in S])
    yp = (ctypes.c_void_p * max(len(Y), 1))(*[t.data_ptr() for t in Y])
    p = torch.empty_like(g)
    w = _work(0, 0, g.device, ws)
    L = capi.lib()
    capi.check(L.sparc_lbfgs_direction(g.numel(), len(S), sp, yp, _p(g), _p(p), w.ptr, _stream()),
               "sparc_lbfgs_direction")
    return p


def linesearch_models(model, update, eps, ws: Workspace | None = None) -> torch.Tensor:
    """grad.py:351-364 for every eps: (neps, *model.shape)."""
    m = _dev(model, model.device if torch.is_tensor(model) else "cuda")
    u = _dev(update, m.device)
    eps = [float(e) for e in eps]
    out = torch.empty((len(eps),) + tuple(m.shape), dtype=torch.float64, device=m.device)
    arr = (ctypes.c_double * max(len(eps), 1))(*eps)
    w = _work(0, 0, m.device, ws)
    L = capi.lib()
    capi.check(L.sparc_linesearch_models(m.numel(), _p(m), _p(u), len(eps), arr, _p(out), w.ptr, _stream()),
               "sparc_linesearch_models")
    return out


# ---------------------------------------------------------------------------------------------
# File contract of grad.py's main
# ---------------------------------------------------------------------------------------------
def _isfloat(v: str) -> bool:
    try:
        float(v)
        return True
    except ValueError:
        return False


def _read2d(path: str) -> np.ndarray:
    a = fits.read(path)
    return a.reshape(a.shape[0], a.shape[-1])  # (nz, 1, nx) -> (nz, nx)


def _write2d(path: str, a) -> None:
    a = a.detach().cpu().numpy() if torch.is_tensor(a) else np.asarray(a)
    fits.write(path, a[:, None, :])


def main(argv=None) -> int:
    """``python grad.py algo=<cg|sd|LBFGS> eps...`` in the code directory (grad.py:122-432).

    Reads params.i (directory, model file), <dir>/master.pixels, <dir>/kernel/kernel_psi_NN.fits
    and hessian_NN.fits, <dir>/update/model_psi_II.fits (and the previous iteration's gradient
    and update for CG, the last four iterations' models and gradients for L-BFGS); writes
    <dir>/update/gradient_psi_II.fits, update_psi_II.fits, test_psi_<i>.fits and <dir>/epslist.npz.
    The reference's figures of the line-search models (matplotlib) are not drawn."""
    args = list(sys.argv[1:] if argv is None else argv)
    params = parse_params_i(open("params.i").read())
    datadir = params["directory"]
    updatedir = os.path.join(datadir, "update")
    iterno = len(fnmatch.filter(os.listdir(updatedir), "misfit_[0-9][0-9]")) - 1
    algo = next((a.split("=")[-1] for a in args if a.startswith("algo=")), "conjugate gradient")
    if algo not in ALGOS:
        print(f"grad: unknown algo {algo!r}", file=sys.stderr)
        return 2
    eps = [float(a) for a in args if _isfloat(a)]
    if not eps:
        nls = len(fnmatch.filter(os.listdir(datadir), "forward_src01_ls[0-9][1-9]"))
        eps = [0.01 * i for i in range(1, nls + 1)]
    back = np.loadtxt(params["file_data"])
    num_src = len(np.loadtxt(os.path.join(datadir, "master.pixels"), ndmin=1))
    it = lambda i: str(i).zfill(2)  # noqa: E731
    kern = np.stack([_read2d(os.path.join(datadir, "kernel", f"kernel_psi_{it(s)}.fits")) for s in range(1, num_src + 1)])
    hess = np.stack([_read2d(os.path.join(datadir, "kernel", f"hessian_{it(s)}.fits")) for s in range(1, num_src + 1)])
    nz, nx = kern.shape[1:]
    ws = Workspace(nx, nz)
    grad = gradient_psi(kern, hess, back[:, 2], ws=ws)
    _write2d(os.path.join(updatedir, f"gradient_psi_{it(iterno)}.fits"), grad)
    rd = lambda kind, i: torch.as_tensor(_read2d(os.path.join(updatedir, f"{kind}_psi_{it(i)}.fits")),  # noqa: E731
                                         dtype=torch.float64, device=grad.device)
    code = ALGOS[algo]
    if iterno == 0 or code == 0:
        update, _ = update_direction("sd", grad, ws=ws)
    elif code in (1, 2):
        update, _ = update_direction("cg" if code == 1 else "hs", grad, rd("gradient", iterno - 1),
                                     rd("update", iterno - 1), ws=ws)
    else:
        lo = max(0, iterno - LBFGS_M)
        models = [rd("model", i) for i in range(lo, iterno + 1)]
        grads = [rd("gradient", i) for i in range(lo, iterno)] + [grad]
        S = [models[j + 1] - models[j] for j in range(len(models) - 1)]
        Y = [grads[j + 1] - grads[j] for j in range(len(grads) - 1)]
        update = lbfgs_direction(grad, S, Y, ws=ws)
    _write2d(os.path.join(updatedir, f"update_psi_{it(iterno)}.fits"), update)
    tests = linesearch_models(rd("model", iterno), update, eps, ws=ws)
    for i in range(len(eps)):
        _write2d(os.path.join(updatedir, f"test_psi_{i + 1}.fits"), tests[i])
    _update_epslist(os.path.join(datadir, "epslist.npz"), iterno, eps)
    return 0


def _update_epslist(path: str, iterno: int, eps: list) -> None:
    """grad.py:401-428: row 0 the steps of this iteration, rows 2-3 the previous pass's rows 0-1."""
    key = str(iterno)
    try:
        with np.load(path) as f:
            old = {k: f[k] for k in f.files}
    except OSError:
        old = {}
    if key in old:
        ls = old[key].copy()
        ls[2:4] = ls[0:2]
        ls[0] = eps
        ls[1] = 0
        old[key] = ls
    else:
        arr = np.zeros((4, len(eps)))
        arr[0] = eps
        old[key] = arr
    np.savez(path, **old)


if __name__ == "__main__":
    sys.exit(main())
