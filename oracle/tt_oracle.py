"""CPU oracle of the travel-time adjoint source (test infrastructure only).

A NumPy restatement of the reference's ADJOINT_SOURCE_FILT (driver.f90:1758-2238) that keeps
its structure -- one inverse 2-D transform of the filtered, windowed, weighted time derivative
per measured receiver, accumulated time-reversed into the adjoint source -- so that it checks
the GPU path (csrc/sparc_tt.cu), which folds all receivers of a mode into one transform.
Nothing in the product imports it.  Arrays are (nt, nx): time slow, x fast (the Fortran
(nx, 1, nt) order of vz_cc.fits read in NumPy order).

numpy.fft stands in for FFTW 3 (un-vendored; "fftw-3.2" by path only): FFTW's unnormalised
forward / backward transforms are np.fft.fft2 and np.fft.ifft2 * (nx nt).  Parity unpinned:
the reference cannot run here (Fortran, MPI, FFTW, CFITSIO) and ships no fixtures for this path.

Followed lines:
  distmat                       initialize.f90:1181-1198
  ridge filters                 driver.f90:1148-1198 (f), 1251-1305 (p1), 1308-1361 (p2),
                                1364-1664 (p3-p7), 1667-1718 (all p modes, all ones in the ridge)
  FREQ_FILTER                   driver.f90:1721-1733
  COMPUTE_TT_GIZONBIRCH         driver.f90:894-940 with SIMPSON_REGULAR (integrals.f90:107-130,
                                accumulator taken as starting from zero)
  ADJOINT_SOURCE_FILT           driver.f90:1758-2238
Single-precision literals of those routines (ridge polynomials, f_low, the mode speeds vel,
the first-bounce polynomial, 0.4 of FREQ_FILTER, 10.**(-8.)) are rounded to float32 as the
Fortran compiler rounds them.
"""
from __future__ import annotations

import math

import numpy as np

F32 = lambda v: float(np.float32(v))  # noqa: E731
PI = 3.141592653589793

# (Polylow, Poly, f_low) of the ridge filters; p2's lower edge is 4.1004 sqrt(k) instead
RIDGES = {
    0: ((0.7, 1.7, -0.2), (1.1, 1.9, -0.2), 1.1),
    1: ((1.1, 2.4, -0.3), (1.4, 3.0, -0.5), 1.6),
    2: (None, (1.6, 3.8, -0.65), 1.6),
    3: ((2.0, 3.55, -0.7), (2.0, 4.1, -0.8), 1.6),
    4: ((2.15, 4.0, -0.7), (2.3, 4.4, -0.7), 1.6),
    5: ((2.2, 4.7, -1.0), (2.35, 5.6, -1.1), 1.6),
    6: ((1.80035417224, 7.42939105658, -2.84595764385), (1.98567115899, 8.09108986838, -3.20316331815), 1.6),
    7: ((1.98297334673, 7.94931076885, -3.00725356897), (2.18544600032, 8.68183289647, -3.84478880142), 1.6),
}
VEL = [0.44, 0.60, 0.75, 0.9, 1.2, 1.4, 1.7, 1.9]  # driver.f90:1936-1944 (vel(8:10) = 0)


def distmat(n: int) -> np.ndarray:
    """initialize.f90:1181-1198 with m = 1: signed distance to index 0 on a ring."""
    f = np.zeros(n)
    for i in range(1, n + 1):
        sig = 1.0
        i2 = min(i - 1, n - i + 1)
        if (i - 1) > (n - i + 1):
            sig = -1.0
        f[i - 1] = math.sqrt(i2 * i2) * sig
    return f


def _kw(nx, nt, xlength_cm, outputcad):
    k = np.abs(distmat(nx)) * 2.0 * PI / (xlength_cm * F32(1e-8) * nx / (nx - 1.0))
    w = np.abs(distmat(nt)) * 2.0 * PI / (nt * outputcad)
    return k, w


def ridge_filter(pord: int, nx: int, nt: int, xlength_cm: float, outputcad: float) -> np.ndarray:
    """FMODE_FILTER, P1..P7MODE_FILTER, ALL_PMODE_FILTER: (nt, nx)."""
    k, w = _kw(nx, nt, xlength_cm, outputcad)
    f = w / (2.0 * PI) * 1e3
    out = np.zeros((nt, nx))
    if pord == 8:
        out[:] = 1.0  # ALL_PMODE_FILTER: pmode = 1.0 and the ridge sets 1 (driver.f90:1694-1703)
        flow = F32(1.6)
    else:
        low, high, flow = RIDGES[pord]
        flow = F32(flow)
        pl = [F32(v) for v in low] if low is not None else None
        ph = [F32(v) for v in high]
        for i in range(nx):
            if pord == 2:
                f0 = F32(4.1004) * math.sqrt(abs(k[i]))
            else:
                f0 = pl[0] + pl[1] * k[i] + pl[2] * k[i] ** 2
            f1 = ph[0] + ph[1] * k[i] + ph[2] * k[i] ** 2
            delta = f1 - f0
            for j in range(nt):
                d = f[j] - f0
                if d < delta and d > 0:
                    if pord == 0:
                        out[j, i] = 0.5 * (1.0 + math.cos(PI * (d - delta / 2.0) / (delta / 2.0)))
                    else:
                        out[j, i] = 0.5 * (1.0 + math.cos(PI * (abs(d) - abs(delta) * 0.5) / (abs(delta) * 0.5)))
    df = 0.5
    for j in range(nt):
        if pord == 0:
            if f[j] < flow + df:
                out[j] *= 0.5 * (1.0 + math.cos(PI * (f[j] - (flow + df)) / df))
            if f[j] < flow:
                out[j] = 0.0
        else:
            if f[j] < flow:
                out[j] = 0.0
            if f[j] < flow + df:
                out[j] *= 0.5 * (1.0 + math.cos(PI * (f[j] - (flow + df)) / df))
    return out


def freq_filter(f1: float, f2: float, nt: int, outputcad: float) -> np.ndarray:
    """FREQ_FILTER (f1, f2 in mHz): (nt,)."""
    w = np.abs(distmat(nt)) * 1e3 / (nt * outputcad)
    wid = F32(0.4) * (w[1] - w[0])
    return 1.0 / (1.0 + np.exp((f1 - w) / wid)) - 1.0 / (1.0 + np.exp((f2 - w) / wid))


def simpson(f: np.ndarray, dv: float) -> float:
    """SIMPSON_REGULAR (integrals.f90:107-130), 1-based weights 1, 4, 2, 4, ..., 1."""
    n = len(f)
    s = 0.0
    for k in range(1, n + 1):
        if k == 1 or k == n:
            s += f[k - 1]
        elif k % 2 == 0:
            s += 4 * f[k - 1]
        else:
            s += 2 * f[k - 1]
    return s * dv / 3.0


def tt_gizon_birch(u0: np.ndarray, u: np.ndarray, dt: float, lef: int, rig: int) -> float:
    """COMPUTE_TT_GIZONBIRCH; lef, rig 1-based inclusive."""
    nt = len(u0)
    win = np.zeros(nt)
    win[lef - 1:rig] = 1.0
    u0w = np.fft.rfft(u0)
    for k in range(1, nt // 2 + 1):
        u0w[k - 1] = u0w[k - 1] * (1j * 2 * PI * (k - 1.0) / (nt * dt))
    u0w[nt // 2] = 0
    u0dot = np.fft.irfft(u0w, n=nt)  # FFTW c2r then /nt
    num = simpson(win * u0dot * (u0 - u), dt)
    den = simpson(win * u0dot ** 2, dt)
    return num / den


def window_bounds(pord: int, dist: float, dt: float, acc_row: np.ndarray, halftime: int):
    """driver.f90:2046-2061: (lef, rig, loc, timest, timefin), 1-based; the search range is
    clipped to [1, nt] (the reference reads out of bounds there), None when nothing is left."""
    nt = len(acc_row)
    if pord != 8:
        timest = math.floor(dist / F32(VEL[pord]) * (1.0 / dt))
        timefin = timest + 40
    else:
        timest = math.floor((F32(-0.000417147774671) * dist ** 2 + F32(0.313350998096) * dist
                             + F32(17.9609631186)) * (1.0 / dt))
        timefin = math.floor((F32(-0.00028361249034) * dist ** 2 + F32(0.29270337114) * dist
                              + F32(36.4398734578)) * (1.0 / dt))
    a, b = max(timest, 1), min(timefin, nt)
    if a > b:
        return None  # search range outside the record (the reference reads out of bounds): no measurement
    seg = np.abs(acc_row[a - 1:b])
    loc = int(np.argmax(seg)) + a
    return max(loc - halftime, 1), min(loc + halftime, nt), loc, timest, timefin


def adjoint_source(synth: np.ndarray, data: np.ndarray, x00: float, xlength_cm: float, t_min: np.ndarray,
                   outputcad: float, modes: dict, freq: dict | None = None, windows: dict | None = None):
    """ADJOINT_SOURCE_FILT for one source.

    synth, data: (nt, nx) vz_cc and data; t_min: the record times in minutes as the reference
    forms them (t = -reversed(timeline)/60); modes: {pord: (mindist, maxdist, window)} for the
    params.<pord> files present; freq: {'allmodes' | 0 | 1 | 2: (f1, f2)} for the filter.params
    files present; windows: {pord: [(lef, rig), ...]} to reuse (line search) instead of picking.
    Returns dict(adj (nt, nx), misfit (sum tau^2, not halved), nmeas, rows {pord: [(i, tau*60,
    lef, rig, loc, timest, timefin)]}, windows {pord: [(lef, rig)]})."""
    nt, nx = synth.shape
    freq = freq or {}
    dt = t_min[1] - t_min[0]
    x = np.arange(nx) / nx
    dmat = distmat(nx)
    eyekh = 1j * dmat * 2.0 * PI
    distances = np.abs((x - 0.5) * xlength_cm * F32(1e-8) - x00)
    freqnu = distmat(nt) / (nt * dt * 60.0)
    tempout = np.fft.fft2(synth)     # FFTW forward over (x, t)
    tempdat = np.fft.fft2(data)
    filt = np.ones(nt)
    filters = {p: ridge_filter(p, nx, nt, xlength_cm, outputcad) for p in range(9)}
    if "allmodes" in freq:
        filt = freq_filter(*freq["allmodes"], nt, outputcad)
    for p in range(9):
        filters[p] = filters[p] * filt[:, None]
    for p in (0, 1, 2):  # driver.f90:1880-1929: filt carries over when a file is absent
        if p in freq:
            filt = freq_filter(*freq[p], nt, outputcad)
        filters[p] = filters[p] * filt[:, None]
    adj = np.zeros((nt, nx))
    misfit, nmeas = 0.0, 0
    rows_out, win_out = {}, {}
    for pord in range(9):
        if pord not in modes:
            continue
        mindist, maxdist, window = modes[pord]
        halftime = int(math.floor(window / (2.0 * dt) + 0.5))
        filt2 = filters[pord]
        fo = tempout * filt2
        fd = tempdat * filt2
        acc = np.fft.ifft2(fo) * (nx * nt)
        dat = np.fft.ifft2(fd) * (nx * nt)
        fo = fo * (1j * freqnu[:, None] * (2.0 * PI))
        ccdot = np.fft.ifft2(fo) * (nx * nt)
        rows, wins = [], []
        it = iter(windows[pord]) if windows and pord in windows else None
        for i in range(nx):
            if not (distances[i] > mindist and distances[i] < maxdist):
                continue
            if it is None:
                wb = window_bounds(pord, distances[i], dt, acc[:, i].real, halftime)
                if wb is None:
                    continue
                lef, rig, loc, timest, timefin = wb
            else:
                lef, rig = next(it)
                loc = timest = timefin = 0
            wins.append((lef, rig))
            tau = tt_gizon_birch(acc[:, i].real, dat[:, i].real, dt, lef, rig)
            rows.append((i + 1, tau * 60.0, lef, rig, loc, timest, timefin))
            win = np.zeros(nt)
            win[lef - 1:rig] = 1.0
            ccdotone = np.fft.fft(ccdot[:, i] * win)
            filtemp = filt2 * ccdotone[:, None] * np.exp(-eyekh * x[i])[None, :]
            filtex = np.fft.ifft2(filtemp) * (nx * nt)
            misfit += tau ** 2
            nmeas += 1
            con = (-tau / (np.sum(ccdot[lef - 1:rig, i] ** 2) * dt)).real
            adj[::-1] += (filtex * con).real
        rows_out[pord], win_out[pord] = rows, wins
    adj = adj * nt / 60.0
    return {"adj": adj, "misfit": misfit, "nmeas": nmeas, "rows": rows_out, "windows": win_out}


# ---------------------------------------------------------------------------------------------
# MISFIT_ALL (driver.f90:2294-2651): travel times by cross-correlation in three frequency bands
# ---------------------------------------------------------------------------------------------
BANDS = [(2.0, 3.5), (3.5, 4.5), (4.5, 6.0)]  # driver.f90:2376-2385


def compute_tt(u0: np.ndarray, u: np.ndarray, dt: float):
    """COMPUTE_TT (driver.f90:855-890): peak of the cross-correlation refined by the parabola
    through its three samples (the 3 x 3 system solved by inversion).  None when the peak sits
    at the end of the lag range (the reference reads past the array there)."""
    n = len(u0)
    lags = np.arange(-n + 1, n)
    cc = np.zeros(2 * n - 1)
    for j, i in enumerate(lags):
        if i <= 0:
            l1 = -i + 1
            cc[j] = np.sum(u0[l1 - 1:n] * u[0:n - l1 + 1]) * dt
        else:
            l2 = n - i
            cc[j] = np.sum(u0[0:l2] * u[i:n]) * dt
    jm = int(np.argmax(cc))
    if jm == 0 or jm == 2 * n - 2:
        return None
    loc = lags[jm]
    times = np.array([(loc - 1) * dt, loc * dt, (loc + 1) * dt])
    mat = np.stack([np.ones(3), times, times ** 2], axis=1)
    inv = np.linalg.inv(mat)
    c3 = cc[jm - 1:jm + 2]
    p1 = inv[1] @ c3
    p2 = inv[2] @ c3
    return -p1 * 0.5 / p2


def misfit_search_range(pord: int, dist: float, dt: float):
    """timest, timefin of MISFIT_ALL's window pick (driver.f90:2436-2446): the f/p modes as in
    ADJOINT_SOURCE_FILT, the first bounce with its own polynomials."""
    if pord != 8:
        ts = math.floor(dist / F32(VEL[pord]) * (1.0 / dt))
        return ts, ts + 40
    ts = math.floor((F32(-1.45511095e-04) * dist ** 2 + F32(2.72140632e-01) * dist + F32(2.16331969e+01)) * (1.0 / dt))
    tf = math.floor((F32(3.85746516e-08) * dist ** 2 + F32(2.21324786e-01) * dist + F32(4.36702155e+01)) * (1.0 / dt))
    return ts, tf


def misfit_all(synth: np.ndarray, data: np.ndarray, x00: float, xlength_cm: float, t_min: np.ndarray,
               outputcad: float, modes: dict, windows: dict | None = None):
    """MISFIT_ALL for one source.  Returns a list over the three bands of dict(band, nmeas (11,),
    misfit (11,) halved, windows {pord: [(lef, rig)]}) -- windows as picked, unclipped; a window
    that leaves the record, or a correlation peak at the end of its lag range, is not measured."""
    nt, nx = synth.shape
    dt = t_min[1] - t_min[0]
    x = np.arange(nx) / nx
    distances = np.abs((x - 0.5) * xlength_cm * F32(1e-8) - x00)
    tempout = np.fft.fft2(synth)
    tempdat = np.fft.fft2(data)
    out = []
    for fb, (left, right) in enumerate(BANDS, start=1):
        filt = freq_filter(left, right, nt, outputcad)
        nmeas = np.zeros(11, dtype=int)
        mis = np.zeros(11)
        wins = {}
        for pord in range(9):
            if pord not in modes:
                continue
            mindist, maxdist, window = modes[pord]
            halftime = int(math.floor(window / (2.0 * dt) + 0.5))
            filt2 = ridge_filter(pord, nx, nt, xlength_cm, outputcad) * filt[:, None]
            acc = (np.fft.ifft2(tempout * filt2) * (nx * nt)).real
            dat = (np.fft.ifft2(tempdat * filt2) * (nx * nt)).real
            given = iter(windows[fb][pord]) if windows and fb in windows and pord in windows[fb] else None
            wl = []
            for i in range(nx):
                if not (distances[i] > mindist and distances[i] < maxdist):
                    continue
                if given is None:
                    ts, tf = misfit_search_range(pord, distances[i], dt)
                    a, b = max(ts, 1), min(tf, nt)
                    if a > b:
                        continue
                    loc = int(np.argmax(np.abs(acc[a - 1:b, i]))) + a
                    lef, rig = loc - halftime, loc + halftime
                else:
                    lef, rig = next(given)
                wl.append((lef, rig))
                if lef < 1 or rig > nt:
                    continue
                tau = compute_tt(acc[lef - 1:rig, i], dat[lef - 1:rig, i], dt)
                if tau is None:
                    continue
                mis[pord] += tau ** 2
                nmeas[pord] += 1
            wins[pord] = wl
        out.append({"band": (left, right), "nmeas": nmeas, "misfit": 0.5 * mis, "windows": wins})
    return out
