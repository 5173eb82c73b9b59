"""Regenerate tests/golden/grad_small.npz by running the reference's own grad.py.

The reference's gradient post-processing (grad.py) is imported from the reference checkout
and its main() run twice in a scratch data directory: iteration 0 (steepest descent) and
iteration 1 (conjugate gradient, Polak-Ribiere), each with two line-search steps.  Only
what grad.py needs from outside the arithmetic is stubbed: its params.i reader (read_params:
directory, nx, nz, xlength, model file, flows), FITS I/O (astropy.io.fits, backed by
sparc_flows_gb300.fits) and plotting (matplotlib, a no-op).  The filter functions are also
called directly for the options main() does not use ('smooth' z filter, symmetrize).

Run in the build container only:
    python tests/golden/make_grad_golden.py /path/to/reference
The reference is not available where the tests run; the .npz is the committed fixture.
"""
import contextlib
import os
import sys
import tempfile
import types
from unittest import mock

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))
from sparc_flows_gb300 import fits as _fits  # noqa: E402

NX, NZ, NSRC = 64, 20, 2
XLENGTH = 400.0
EPS = (0.01, 0.02)


def _stub_modules(datadir: str, model_path: str):
    rp = types.ModuleType("read_params")
    rp.get_directory = lambda: datadir
    rp.get_nx = lambda: NX
    rp.get_nz = lambda: NZ
    rp.get_xlength = lambda: XLENGTH
    rp.get_solarmodel = lambda: model_path
    rp.if_flows = lambda: True

    class _HDUList(list):
        def __enter__(self):
            return self

        def __exit__(self, *a):
            return False

    fits = types.ModuleType("astropy.io.fits")
    fits.open = lambda f: _HDUList([types.SimpleNamespace(data=_fits.read(f))])

    def writeto(f, arr, overwrite=False):
        if os.path.exists(f) and not overwrite:
            raise OSError(f)
        _fits.write(f, np.asarray(arr))

    fits.writeto = writeto
    io = types.ModuleType("astropy.io")
    io.fits = fits
    astropy = types.ModuleType("astropy")
    astropy.io = io
    mpl = mock.MagicMock()
    return {"read_params": rp, "astropy": astropy, "astropy.io": io, "astropy.io.fits": fits,
            "matplotlib": mpl, "matplotlib.pyplot": mpl.pyplot}


def _field(rng, shape, scale):
    """Smooth-ish random field: white noise plus a few Gaussian blobs, times scale."""
    nz, nx = shape
    z, x = np.mgrid[0:nz, 0:nx]
    f = 0.3 * rng.standard_normal(shape)
    for _ in range(3):
        z0, x0 = rng.uniform(0, nz), rng.uniform(0, nx)
        f += rng.uniform(-1, 1) * np.exp(-((z - z0) / 4.0) ** 2 - ((x - x0) / 6.0) ** 2)
    return scale * f


def main(ref: str):
    rng = np.random.default_rng(20261203)
    out = {"nx": NX, "nz": NZ, "nsrc": NSRC, "eps": np.array(EPS)}
    with tempfile.TemporaryDirectory() as tmp:
        datadir = os.path.join(tmp, "data")
        for d in ("kernel", "update"):
            os.makedirs(os.path.join(datadir, d))
        np.savetxt(os.path.join(datadir, "master.pixels"), np.linspace(-20, 20, NSRC))
        # model file columns r/R, c, rho, p, g, Gamma1; only r and rho are read by grad.py
        zr = 1.0 + np.linspace(-25.0, 0.5, NZ) / 695.989467700
        rho = 2.78e-7 * np.exp(np.linspace(8.0, 0.0, NZ))
        back = np.column_stack([zr, np.ones(NZ), rho, np.ones(NZ), np.ones(NZ), np.ones(NZ)])
        model_path = os.path.join(tmp, "model")
        np.savetxt(model_path, back)
        out["rho"] = np.loadtxt(model_path)[:, 2]
        _fits.write(os.path.join(tmp, "true_psi.fits"), np.zeros((NZ, 1, NX)))
        sys.modules.update(_stub_modules(datadir, model_path))
        sys.path.insert(0, ref)
        import grad  # the reference's grad.py

        cwd = os.getcwd()
        os.chdir(tmp)
        try:
            for it in range(2):
                kern = np.stack([_field(rng, (NZ, NX), 1e-3 * (s + 1)) for s in range(NSRC)])
                hess = np.stack([np.abs(_field(rng, (NZ, NX), 1e2)) * (1 if s % 2 else -1) for s in range(NSRC)])
                psi = _field(rng, (NZ, NX), 1.0)
                for s in range(NSRC):
                    _fits.write(os.path.join(datadir, "kernel", f"kernel_psi_{s + 1:02d}.fits"), kern[s][:, None, :])
                    _fits.write(os.path.join(datadir, "kernel", f"hessian_{s + 1:02d}.fits"), hess[s][:, None, :])
                _fits.write(os.path.join(datadir, "update", f"model_psi_{it:02d}.fits"), psi[:, None, :])
                open(os.path.join(datadir, "update", f"misfit_{it:02d}"), "w").close()
                with contextlib.redirect_stdout(open(os.devnull, "w")):
                    sys.argv = ["grad.py", "algo=cg", *[str(e) for e in EPS]]
                    grad.main()
                u = lambda n: _fits.read(os.path.join(datadir, "update", n))[:, 0, :]  # noqa: E731
                out[f"it{it}_kernels"] = kern
                out[f"it{it}_hessians"] = hess
                out[f"it{it}_model"] = psi
                out[f"it{it}_gradient"] = u(f"gradient_psi_{it:02d}.fits")
                out[f"it{it}_update"] = u(f"update_psi_{it:02d}.fits")
                for i in range(len(EPS)):
                    out[f"it{it}_test_{i + 1}"] = u(f"test_psi_{i + 1}.fits")
            out["epslist_1"] = np.load(os.path.join(datadir, "epslist.npz"))["1"]
            # options main() does not exercise, through the module-level functions
            a = out["it0_kernels"][0].T[:, None, :].copy()  # grad.py's (nx, 1, nz) order
            s = a.copy()
            grad.filterz(s, algo="smooth")
            out["smooth_in"], out["smooth_out"] = out["it0_kernels"][0], s[:, 0, :].T
            y = a.copy()
            grad.symmetrize(y)
            out["sym_out"] = y[:, 0, :].T
            out["filterx_nk5"] = grad.filterx(a, 5)[:, 0, :].T
            g3 = a.copy()
            grad.filterz(g3, algo="gaussian", sp=3.0)
            out["gauss3_out"] = g3[:, 0, :].T
        finally:
            os.chdir(cwd)
    np.savez_compressed(os.path.join(HERE, "grad_small.npz"), **out)
    print({k: np.shape(v) for k, v in out.items()})


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.environ.get("SPARC_REFERENCE", ""))
