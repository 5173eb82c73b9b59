"""Compile the CUDA extension (sm_103a) into sparc_flows_gb300/_lib/libsparc_gb300.so.

nvcc is called directly (no torch extension machinery): the library is a plain C ABI
(include/sparc_gb300.h) loaded with ctypes.  Translation units compile in parallel.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
OUT_DIR = os.path.join(PKG, "_lib")
LIB_PATH = os.path.join(OUT_DIR, "libsparc_gb300.so")
SOURCES = ["sparc_row.cu", "sparc_col.cu", "sparc_col_tma.cu", "sparc_col_band.cu", "sparc_col_band_tma.cu", "sparc_end.cu", "sparc_capi.cu", "sparc_noalloc.cu", "sparc_grad.cu", "sparc_3d.cu", "sparc_tt.cu", "sparc_fits.cu", "sparc_sponge.cu", "sparc_adjoint.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
         "--expt-relaxed-constexpr", "-I", CSRC, "-I", os.path.join(ROOT, "include")]


def nvcc() -> str:
    for cand in (os.environ.get("NVCC"), shutil.which("nvcc"), "/usr/local/cuda/bin/nvcc"):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError("nvcc not found")


def _stale() -> bool:
    if not os.path.exists(LIB_PATH):
        return True
    t = os.path.getmtime(LIB_PATH)
    deps = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(ROOT, "include", "sparc_gb300.h"),
                                                                   __file__]
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False, extra: list[str] | None = None) -> str:
    """Build the shared library if any source is newer; returns its path."""
    if not force and not _stale():
        return LIB_PATH
    os.makedirs(OUT_DIR, exist_ok=True)
    cc = nvcc()
    objs = []

    def one(src):
        obj = os.path.join(OUT_DIR, src.replace(".cu", ".o"))
        cmd = [cc, *ARCH, *FLAGS, *(extra or []), "-c", os.path.join(CSRC, src), "-o", obj]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"nvcc failed for {src}:\n{r.stdout}\n{r.stderr}")
        if verbose and (r.stdout or r.stderr):
            print(r.stdout, r.stderr)
        return obj

    with cf.ThreadPoolExecutor(max_workers=len(SOURCES)) as ex:
        objs = list(ex.map(one, SOURCES))
    tmp = LIB_PATH + ".tmp"
    r = subprocess.run([cc, *ARCH, "-shared", "-o", tmp, *objs], capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError(f"link failed:\n{r.stdout}\n{r.stderr}")
    os.replace(tmp, LIB_PATH)
    return LIB_PATH


if __name__ == "__main__":
    import sys

    print(build(force="--force" in sys.argv, verbose=True,
                extra=["-Xptxas", "-v"] if "--ptxas" in sys.argv else None))
