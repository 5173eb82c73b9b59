"""Travel-time adjoint source and misfit (ADJOINT_SOURCE_FILT, driver.f90:1758-2238) on the GPU.

The host side: the ridge filters of the f, p1..p7 and all-p-mode ridges (driver.f90:1148-1718)
and FREQ_FILTER (driver.f90:1721-1733) as (nt, nx) masks, the measurement set-up (params.<pord>
and filter.params.* files, receiver distances, search ranges of the window pick,
driver.f90:1768-1800, 1946-2061), and the outputs the reference writes (ttdiff.<pord>,
windows.<pord>, adjoint_srcNN/source.fits and information, kernel/misfit_NN_MM,
driver.f90:1956-2230).  The transforms, window picks, travel times (Gizon-Birch) and the
adjoint-source assembly run in csrc/sparc_tt.cu through sparc_tt_*.

Single-precision literals of the reference (ridge polynomials, f_low, mode speeds, the
first-bounce window polynomial, 0.4 of FREQ_FILTER, 10.**(-8.)) are rounded to float32 as
the Fortran compiler rounds them.
"""
from __future__ import annotations

import ctypes
import math
import os

import numpy as np
import torch

from . import capi

PI = 3.141592653589793
_f = lambda v: float(np.float32(v))  # noqa: E731

# ridge edges f0 (lower) and f1 (upper) as quadratics in k (Polylow, Poly) and f_low
# (driver.f90:1160-1172, 1262-1272, 1320-1330, 1376-1386, 1432-1442, 1488-1498, 1547-1557, 1613-1623)
_RIDGE = {
    0: ((0.7, 1.7, -0.2), (1.1, 1.9, -0.2), 1.1),
    1: ((1.1, 2.4, -0.3), (1.4, 3.0, -0.5), 1.6),
    2: ("sqrt", (1.6, 3.8, -0.65), 1.6),
    3: ((2.0, 3.55, -0.7), (2.0, 4.1, -0.8), 1.6),
    4: ((2.15, 4.0, -0.7), (2.3, 4.4, -0.7), 1.6),
    5: ((2.2, 4.7, -1.0), (2.35, 5.6, -1.1), 1.6),
    6: ((1.80035417224, 7.42939105658, -2.84595764385), (1.98567115899, 8.09108986838, -3.20316331815), 1.6),
    7: ((1.98297334673, 7.94931076885, -3.00725356897), (2.18544600032, 8.68183289647, -3.84478880142), 1.6),
}
_P2_CONST = 4.1004  # driver.f90:1320
MODE_SPEED = [0.44, 0.60, 0.75, 0.9, 1.2, 1.4, 1.7, 1.9]  # vel(0:7), driver.f90:1936-1944


def signed_index(n: int) -> np.ndarray:
    """distmat(n, 1) (initialize.f90:1181-1198): q for q <= n - q, else -(n - q)."""
    q = np.arange(n)
    return np.where(q > n - q, -(n - q), q).astype(np.float64)


def _grid(nx, nt, xlength_cm, outputcad):
    k = np.abs(signed_index(nx)) * 2.0 * PI / (xlength_cm * _f(1e-8) * nx / (nx - 1.0))
    w = np.abs(signed_index(nt)) * 2.0 * PI / (nt * outputcad)
    return k, w / (2.0 * PI) * 1e3  # k in 1/Mm, f in mHz


def ridge_filters(nx: int, nt: int, xlength_cm: float, outputcad: float) -> np.ndarray:
    """(9, nt, nx): f, p1..p7 ridges and the all-p-mode filter (driver.f90:1148-1718)."""
    k, f = _grid(nx, nt, xlength_cm, outputcad)
    out = np.zeros((9, nt, nx))
    df = 0.5
    for p in range(9):
        if p == 8:
            m = np.ones((nt, nx))
            flow = _f(1.6)
        else:
            low, high, flow = _RIDGE[p]
            flow = _f(flow)
            ph = [_f(v) for v in high]
            f1 = ph[0] + ph[1] * k + ph[2] * k ** 2
            if low == "sqrt":
                f0 = _f(_P2_CONST) * np.sqrt(np.abs(k))
            else:
                pl = [_f(v) for v in low]
                f0 = pl[0] + pl[1] * k + pl[2] * k ** 2
            delta = (f1 - f0)[None, :]
            d = f[:, None] - f0[None, :]
            inside = (d < delta) & (d > 0)
            with np.errstate(invalid="ignore", divide="ignore"):
                if p == 0:
                    shape = 0.5 * (1.0 + np.cos(PI * (d - delta / 2.0) / (delta / 2.0)))
                else:
                    shape = 0.5 * (1.0 + np.cos(PI * (np.abs(d) - np.abs(delta) * 0.5) / (np.abs(delta) * 0.5)))
            m = np.where(inside, shape, 0.0)
        taper = np.where(f < flow + df, 0.5 * (1.0 + np.cos(PI * (f - (flow + df)) / df)), 1.0)
        m = m * taper[:, None]
        m[f < flow] = 0.0
        out[p] = m
    return out


def freq_filter(f1: float, f2: float, nt: int, outputcad: float) -> np.ndarray:
    """FREQ_FILTER (driver.f90:1721-1733), f1, f2 in mHz: (nt,)."""
    w = np.abs(signed_index(nt)) * 1e3 / (nt * outputcad)
    wid = _f(0.4) * (w[1] - w[0])
    return 1.0 / (1.0 + np.exp((f1 - w) / wid)) - 1.0 / (1.0 + np.exp((f2 - w) / wid))


def mode_filters(nx, nt, xlength_cm, outputcad, freq: dict) -> np.ndarray:
    """The ridge filters times their frequency filters (driver.f90:1849-1929).  freq holds the
    (f1, f2) of the filter.params.allmodes / .0 / .1 / .2 files present ('allmodes', 0, 1, 2);
    as in the reference, a mode whose own file is absent is multiplied by the last frequency
    filter read (the all-modes one, a second time, or 1)."""
    filt = ridge_filters(nx, nt, xlength_cm, outputcad)
    ff = np.ones(nt)
    if "allmodes" in freq:
        ff = freq_filter(*freq["allmodes"], nt, outputcad)
    filt *= ff[None, :, None]
    for p in (0, 1, 2):
        if p in freq:
            ff = freq_filter(*freq[p], nt, outputcad)
        filt[p] *= ff[:, None]
    return filt


def _read_floats(path: str, n: int) -> list[float]:
    vals = []
    with open(path) as fh:
        for line in fh:
            for tok in line.replace(",", " ").split():
                vals.append(float(tok.replace("d", "e").replace("D", "E")))
                if len(vals) == n:
                    return vals
    raise ValueError(f"{path}: expected {n} numbers")


def read_measurement_files(directory: str):
    """params.<pord> (mindist, maxdist, window) for pord 0..8 and filter.params.{allmodes,0,1,2}
    (left, right corner in mHz) present in the data directory (driver.f90:1853-1929, 1947-1956)."""
    modes, freq = {}, {}
    for p in range(9):
        f = os.path.join(directory, f"params.{p}")
        if os.path.exists(f):
            modes[p] = tuple(_read_floats(f, 3))
    for key, name in (("allmodes", "filter.params.allmodes"), (0, "filter.params.0"), (1, "filter.params.1"),
                      (2, "filter.params.2")):
        f = os.path.join(directory, name)
        if os.path.exists(f):
            freq[key] = tuple(_read_floats(f, 2))
    return modes, freq


BANDS = [(2.0, 3.5), (3.5, 4.5), (4.5, 6.0)]  # MISFIT_ALL's frequency bands, driver.f90:2376-2385


def misfit_search_range(pord: int, dist: float, dt_min: float) -> tuple[int, int]:
    """timest, timefin of MISFIT_ALL's window pick (driver.f90:2436-2446): the f/p modes as in
    ADJOINT_SOURCE_FILT, the first bounce (pord 8) with its own polynomials."""
    if pord != 8:
        return search_range(pord, dist, dt_min)
    ts = math.floor((_f(-1.45511095e-04) * dist ** 2 + _f(2.72140632e-01) * dist + _f(2.16331969e+01)) * (1.0 / dt_min))
    tf = math.floor((_f(3.85746516e-08) * dist ** 2 + _f(2.21324786e-01) * dist + _f(4.36702155e+01)) * (1.0 / dt_min))
    return ts, tf


def search_range(pord: int, dist: float, dt_min: float) -> tuple[int, int]:
    """timest, timefin of the window pick (driver.f90:2046-2053), 1-based."""
    if pord != 8:
        ts = math.floor(dist / _f(MODE_SPEED[pord]) * (1.0 / dt_min))
        return ts, ts + 40
    ts = math.floor((_f(-0.000417147774671) * dist ** 2 + _f(0.313350998096) * dist + _f(17.9609631186)) * (1.0 / dt_min))
    tf = math.floor((_f(-0.00028361249034) * dist ** 2 + _f(0.29270337114) * dist + _f(36.4398734578)) * (1.0 / dt_min))
    return ts, tf


class TTAdjoint:
    """Travel-time measurements and adjoint sources for a batch of sources on one grid."""

    def __init__(self, nx: int, nt: int, nbatch: int, xlength_cm: float, outputcad: float, device="cuda"):
        self.L = capi.lib()
        self.nx, self.nt, self.nb = nx, nt, nbatch
        self.xlength_cm, self.outputcad = xlength_cm, outputcad
        self.dev = torch.device(device)
        h = ctypes.c_void_p()
        capi.check(self.L.sparc_tt_plan_create(nx, nt, nbatch, nbatch * nx, ctypes.byref(h)), "sparc_tt_plan_create")
        self.plan = h

    def _stream(self):
        return ctypes.c_void_p(torch.cuda.current_stream(self.dev).cuda_stream)

    def distances(self, x00: float) -> np.ndarray:
        """|x - x00| in Mm of every column (driver.f90:1788)."""
        x = np.arange(self.nx) / self.nx
        return np.abs((x - 0.5) * self.xlength_cm * _f(1e-8) - x00)

    def run(self, synth, data, x00s, t_min: np.ndarray, modes: dict, freq: dict | None = None,
            windows: dict | None = None):
        """synth, data: (nb, nt, nx) records; x00s: source positions in Mm (master.pixels); t_min:
        record times in minutes as the reference forms them (t = -reversed(timeline) / 60);
        modes {pord: (mindist, maxdist, window)}; freq as in mode_filters; windows
        {pord: {b: [(lef, rig), ...]}} to reuse (line search) instead of picking.

        Returns dict(adj (nb, nt, nx) device tensor, misfit [nb] (0.5 sum tau^2), nmeas [nb],
        rows {pord: {b: [(i, tau*60, lef, rig, loc, timest, timefin)]}}, windows like the input)."""
        nb, nt, nx = self.nb, self.nt, self.nx
        s = torch.as_tensor(synth, dtype=torch.float64, device=self.dev).contiguous()
        d = torch.as_tensor(data, dtype=torch.float64, device=self.dev).contiguous()
        capi.check(self.L.sparc_tt_set_records(self.plan, s.data_ptr(), d.data_ptr(), self._stream()),
                   "sparc_tt_set_records")
        dt = float(t_min[1] - t_min[0])
        filt = torch.as_tensor(mode_filters(nx, nt, self.xlength_cm, self.outputcad, freq or {}),
                               dtype=torch.float64, device=self.dev).contiguous()
        misfit = np.zeros(nb)
        nmeas = np.zeros(nb, dtype=int)
        rows_out, wins_out = {}, {}
        for pord in sorted(modes):
            mindist, maxdist, window = modes[pord]
            halftime = int(math.floor(window / (2.0 * dt) + 0.5))
            given = windows is not None and pord in windows
            rows = []
            for b in range(nb):
                dist = self.distances(x00s[b])
                it = iter(windows[pord].get(b, [])) if given else None
                for i in range(nx):
                    if not (dist[i] > mindist and dist[i] < maxdist):
                        continue
                    ts, tf = search_range(pord, dist[i], dt)
                    lef, rig = next(it) if given else (0, 0)
                    if not given and max(ts, 1) > min(tf, nt):
                        continue  # search range outside the record: the reference reads out of bounds
                    rows.append((b, i, ts, tf, lef, rig, 0))
            arr = np.ascontiguousarray(np.array(rows, dtype=np.int32).reshape(-1, 7))
            tau = np.zeros(max(len(rows), 1))
            capi.check(self.L.sparc_tt_mode(self.plan, filt[pord].data_ptr(), len(rows),
                                            arr.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), halftime, int(given),
                                            dt, tau.ctypes.data_as(ctypes.POINTER(ctypes.c_double)), self._stream()),
                       "sparc_tt_mode")
            per_b, per_w = {}, {}
            for r, (b, i, ts, tf, lef, rig, loc) in enumerate(arr.tolist()):
                if given:
                    loc = ts = tf = 0
                per_b.setdefault(b, []).append((i + 1, tau[r] * 60.0, lef, rig, loc, ts, tf))
                per_w.setdefault(b, []).append((lef, rig))
                misfit[b] += tau[r] ** 2
                nmeas[b] += 1
            rows_out[pord], wins_out[pord] = per_b, per_w
        adj = torch.empty((nb, nt, nx), dtype=torch.float64, device=self.dev)
        capi.check(self.L.sparc_tt_adjoint(self.plan, adj.data_ptr(), self._stream()), "sparc_tt_adjoint")
        torch.cuda.current_stream(self.dev).synchronize()
        return {"adj": adj, "misfit": 0.5 * misfit, "nmeas": nmeas, "rows": rows_out, "windows": wins_out}

    def misfit_all(self, synth, data, x00s, t_min: np.ndarray, modes: dict, windows: dict | None = None):
        """MISFIT_ALL (driver.f90:2294-2651): cross-correlation travel times of every ridge filter
        in three frequency bands.  windows {band (1..3): {pord: {b: [(lef, rig), ...]}}} to reuse.
        Returns a list over the bands of dict(band, nmeas (nb, 11), misfit (nb, 11) halved,
        windows {pord: {b: [(lef, rig)]}} as picked (unclipped))."""
        nb, nt, nx = self.nb, self.nt, self.nx
        s = torch.as_tensor(synth, dtype=torch.float64, device=self.dev).contiguous()
        d = torch.as_tensor(data, dtype=torch.float64, device=self.dev).contiguous()
        capi.check(self.L.sparc_tt_set_records(self.plan, s.data_ptr(), d.data_ptr(), self._stream()),
                   "sparc_tt_set_records")
        dt = float(t_min[1] - t_min[0])
        ridges = ridge_filters(nx, nt, self.xlength_cm, self.outputcad)
        out = []
        for fb, (left, right) in enumerate(BANDS, start=1):
            ff = freq_filter(left, right, nt, self.outputcad)
            nmeas = np.zeros((nb, 11), dtype=int)
            mis = np.zeros((nb, 11))
            wins = {}
            for pord in sorted(modes):
                mindist, maxdist, window = modes[pord]
                halftime = int(math.floor(window / (2.0 * dt) + 0.5))
                given = windows is not None and fb in windows and pord in windows[fb]
                rows = []
                for b in range(nb):
                    dist = self.distances(x00s[b])
                    it = iter(windows[fb][pord].get(b, [])) if given else None
                    for i in range(nx):
                        if not (dist[i] > mindist and dist[i] < maxdist):
                            continue
                        ts, tf = misfit_search_range(pord, dist[i], dt)
                        lef, rig = next(it) if given else (0, 0)
                        if not given and max(ts, 1) > min(tf, nt):
                            continue
                        rows.append((b, i, ts, tf, lef, rig, 0))
                arr = np.ascontiguousarray(np.array(rows, dtype=np.int32).reshape(-1, 7))
                tau = np.zeros(max(len(rows), 1))
                filt = torch.as_tensor(ridges[pord] * ff[:, None], dtype=torch.float64, device=self.dev).contiguous()
                capi.check(self.L.sparc_tt_misfit_mode(self.plan, filt.data_ptr(), len(rows),
                                                       arr.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), halftime,
                                                       int(given), dt, tau.ctypes.data_as(ctypes.POINTER(ctypes.c_double)),
                                                       self._stream()), "sparc_tt_misfit_mode")
                per_w = {}
                for r, (b, i, ts, tf, lef, rig, loc) in enumerate(arr.tolist()):
                    per_w.setdefault(b, []).append((lef, rig))
                    if np.isfinite(tau[r]):
                        mis[b, pord] += tau[r] ** 2
                        nmeas[b, pord] += 1
                wins[pord] = per_w
            out.append({"band": (left, right), "nmeas": nmeas, "misfit": 0.5 * mis, "windows": wins})
        return out

    def close(self):
        if getattr(self, "plan", None):
            self.L.sparc_tt_plan_destroy(self.plan)
            self.plan = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def write_outputs(directory: str, contrib: str, jobno: str, res: dict, b: int, t_min: np.ndarray,
                  linesearch: bool, compute_synth: bool, test_in_2d: bool = True):
    """The files ADJOINT_SOURCE_FILT writes for source b (driver.f90:1956-2230)."""
    from . import fits

    fdir = os.path.join(directory, f"forward_src{contrib}_ls{jobno}")
    os.makedirs(fdir, exist_ok=True)
    for pord, per_b in res["rows"].items():
        with open(os.path.join(fdir, f"ttdiff.{pord}"), "w") as fh:
            for (i, tau60, lef, rig, loc, ts, tf) in per_b.get(b, []):
                fh.write(f"{i:3d} {tau60:14.8f} {lef:4d} {rig:4d} {loc:4d} {ts:4d} {tf:4d}\n")
        if not linesearch:
            wdir = os.path.join(directory, f"forward_src{contrib}_ls00")
            os.makedirs(wdir, exist_ok=True)
            with open(os.path.join(wdir, f"windows.{pord}"), "w") as fh:
                for (lef, rig) in res["windows"][pord].get(b, []):
                    fh.write(f"{lef:12d}{rig:12d}\n")
    adir = os.path.join(directory, f"adjoint_src{contrib}")
    if not (linesearch or compute_synth):
        os.makedirs(adir, exist_ok=True)
        adj = res["adj"][b].cpu().numpy()
        fits.write(os.path.join(adir, "source.fits"), adj[:, None, :])
    if not linesearch:
        os.makedirs(adir, exist_ok=True)
        with open(os.path.join(adir, "information"), "w") as fh:
            fh.write(f"{len(t_min)}\n{float(t_min[0]) * 60.0!r}\n{float(t_min[-1]) * 60.0!r}\n")
            if test_in_2d:
                fh.write("2D\n")
    kdir = os.path.join(directory, "kernel")
    os.makedirs(kdir, exist_ok=True)
    with open(os.path.join(kdir, f"misfit_{contrib}_{jobno}"), "w") as fh:
        fh.write(f"{int(contrib):12d}{int(res['nmeas'][b]):12d}  {float(res['misfit'][b])!r}\n")


def write_misfit_all(directory: str, contrib: str, jobno: str, bands: list, b: int, linesearch: bool):
    """kernel/misfit_all_NN_MM (three blocks of '# NN left right', '# nmeas(0:10)', misfit(0:10)/2)
    and, outside line searches, forward_srcNN_ls00/windows.all.<pord 2 digits>.<band>
    (driver.f90:2361-2362, 2420-2432, 2470-2476)."""
    kdir = os.path.join(directory, "kernel")
    os.makedirs(kdir, exist_ok=True)
    with open(os.path.join(kdir, f"misfit_all_{contrib}_{jobno}"), "w") as fh:
        for bd in bands:
            left, right = bd["band"]
            fh.write(f" # {int(contrib):12d} {left!r} {right!r}\n")
            fh.write(" # " + " ".join(f"{int(v):12d}" for v in bd["nmeas"][b]) + "\n")
            fh.write(" " + " ".join(repr(float(v)) for v in bd["misfit"][b]) + "\n")
    if not linesearch:
        wdir = os.path.join(directory, f"forward_src{contrib}_ls00")
        os.makedirs(wdir, exist_ok=True)
        for fb, bd in enumerate(bands, start=1):
            for pord, per_b in bd["windows"].items():
                with open(os.path.join(wdir, f"windows.all.{pord:02d}.{fb}"), "w") as fh:
                    for (lef, rig) in per_b.get(b, []):
                        fh.write(f"{lef:12d}{rig:12d}\n")


def read_windows_all(directory: str, contrib: str, modes: dict) -> dict:
    """windows.all.<pord>.<band> of the ls00 forward run (read back in line searches)."""
    out = {}
    for fb in (1, 2, 3):
        for pord in modes:
            f = os.path.join(directory, f"forward_src{contrib}_ls00", f"windows.all.{pord:02d}.{fb}")
            if os.path.exists(f):
                vals = np.loadtxt(f, dtype=int, ndmin=2)
                out.setdefault(fb, {})[pord] = {0: [tuple(map(int, v)) for v in vals]}
    return out


def read_windows(directory: str, contrib: str, modes: dict) -> dict:
    """windows.<pord> of the ls00 forward run (driver.f90:2022-2027, read back in line searches)."""
    out = {}
    for pord in modes:
        f = os.path.join(directory, f"forward_src{contrib}_ls00", f"windows.{pord}")
        if os.path.exists(f):
            vals = np.loadtxt(f, dtype=int, ndmin=2)
            out[pord] = {0: [tuple(map(int, v)) for v in vals]}
    return out
