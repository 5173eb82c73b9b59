"""Run configuration and the ``params.i`` contract of the reference ``sparc`` executable.

``RunConfig`` carries the compile-time parameters of params.i (params.i:26-165) as run-time
values, so one build serves every grid.  ``parse_params_i`` reads a params.i the way the
reference's read_params.py does (read_params.py:3-228) plus the Fortran literal rules that
matter for the arithmetic (``800.0 * 10**(8)`` etc.).
"""
from __future__ import annotations

import dataclasses
import math
import re

RSUN_CM = 6.95989467700e10  # initialize.f90:42
DIMC = 1.0e6                # initialize.f90:746 (cm/s)
DIMRHO = 1.0e-3             # initialize.f90:750 (g/cc)


@dataclasses.dataclass
class RunConfig:
    """One solve's grid, timing and boundary parameters (params.i:26-165)."""

    nx: int = 512
    nz: int = 300
    xlength_cm: float = 400.0e8      # params.i:28 (cm)
    timestep: float = 2.0            # params.i:28 (s)
    npmlbot: int = 10                # params.i:121
    npmltop: int = 10
    npmlhor: int = 9                 # params.i:91
    excitdep_cm: float = -1.5e7      # params.i:148
    obsheight_cm: float = 2.0e7      # params.i:137
    flows: bool = True               # BACKGROUND_FLOWS_EXIST, params.i:70
    adjoint: bool = False            # COMPUTE_ADJOINT
    outputcad: float = 30.0          # params.i:141 (s)
    cadforcing: float = 30.0         # params.i:46 (s)
    nsteps: int = 3600               # number of time steps to run
    solartime_h: float = 4.0         # params.i:132
    filter_kst: int = 6              # first row (1-based) FILTER_VARS_2D writes (physics2d.f90:544-545)
    filter_all_x: bool = False       # filter the horizontal-PML columns too (physics2d.f90:548-556)

    @property
    def steps_out(self) -> int:
        """``steps = floor(outputcad/timestep)`` (driver.f90:209)."""
        return int(math.floor(self.outputcad / self.timestep))

    @property
    def cadforcing_step(self) -> int:
        return int(math.floor(self.cadforcing / self.timestep))

    @property
    def forcing_length(self) -> int:
        """``floor(maxtime/cadforcing_step) + 1`` with maxtime = nsteps - 1 (initialize.f90:1001)."""
        return (self.nsteps - 1) // self.cadforcing_step + 1

    @property
    def src_until(self) -> int:
        """Sources are injected while ``time <= forcing_length*cadforcing_step`` (physics2d.f90:1049)."""
        return self.forcing_length * self.cadforcing_step

    @property
    def nrec(self) -> int:
        """Seismogram records: steps 0, steps_out, ... <= nsteps-1 (driver.f90:386)."""
        return (self.nsteps - 1) // self.steps_out + 1

    @property
    def num_steps(self) -> int:
        """Adjoint-source length bound used by LAGRANGE_INTERP (driver.f90:223-224)."""
        maxtime = self.nsteps - 1
        n = int(math.floor(float(maxtime) * self.timestep / self.cadforcing)) + 2
        return 2 * (n // 2) + 2

    def replace(self, **kw) -> "RunConfig":
        return dataclasses.replace(self, **kw)


def reference_maxtime(solartime_h: float, timestep: float, cadforcing: float, nupeak: float) -> int:
    """``maxtime`` of READ_PARAMETERS (initialize.f90:998-1000); the run has maxtime+1 steps."""
    cadforcing_step = int(math.floor(cadforcing / timestep))
    maxtime = int(math.floor((solartime_h * 3600.0 + 2.0 / nupeak) / timestep)) + 2
    return cadforcing_step * int(math.floor(maxtime / cadforcing_step))


_NUM = r"[-+]?(?:\d+\.?\d*|\.\d+)(?:[eEdD][-+]?\d+)?"


def _fortran_real(expr: str) -> float:
    """Evaluate the simple constant expressions params.i uses (``800.0 * 10**(8)``)."""
    e = expr.strip().lower().replace("d", "e")
    e = re.sub(r"\*\*", "^", e)
    if not re.fullmatch(r"[0-9eE+\-*/^(). ]+", e):
        raise ValueError(f"unsupported params.i expression: {expr!r}")
    return float(eval(e.replace("^", "**"), {"__builtins__": {}}, {}))  # noqa: S307 - digits only


def parse_params_i(text: str) -> dict:
    """Return the parameters of a params.i file as a dict of Python values.

    Keys (lower case): nx, ny, nz, xlength, timestep, file_data, directory, cadforcing,
    npmlbot, npmltop, npmlhor, solartime, obsheight, outputcad, excitdep, flows, magnetic,
    use_pml, horizontal_pmls, displ, periodic, use_fft, compact_finite_diff.
    """
    out: dict = {}
    body = []
    for line in text.splitlines():
        line = line.split("!")[0].strip()
        if line:
            body.append(line)
    joined = "\n".join(body)
    for m in re.finditer(r"parameter\s*\((.*?)\)\s*$", joined, flags=re.I | re.M):
        for item in _split_top(m.group(1)):
            if "=" in item:
                k, v = item.split("=", 1)
                out[k.strip().lower()] = v.strip()
    for m in re.finditer(r"::\s*(\w+)\s*=\s*(.+)$", joined, flags=re.M):
        out[m.group(1).strip().lower()] = m.group(2).strip()
    res: dict = {}
    for k, v in out.items():
        vl = v.lower()
        if vl.startswith("'") or vl.startswith('"'):
            res[k] = v.strip("'\"")
        elif vl.strip(".") in ("true", "false"):
            res[k] = vl.strip(".") == "true"
        else:
            try:
                res[k] = int(v) if re.fullmatch(r"[-+]?\d+", v) else _fortran_real(v)
            except (ValueError, SyntaxError):
                res[k] = v
    return res


def _split_top(s: str):
    depth, cur, parts = 0, "", []
    for ch in s:
        if ch == "(":
            depth += 1
        elif ch == ")":
            depth -= 1
        if ch == "," and depth == 0:
            parts.append(cur)
            cur = ""
        else:
            cur += ch
    if cur:
        parts.append(cur)
    return parts


def run_config_from_params(p: dict, nsteps: int | None = None, adjoint: bool = False) -> RunConfig:
    """RunConfig from parsed params.i values; nsteps defaults to the reference maxtime+1."""
    nupeak = float(__import__("numpy").float32(0.0017))
    rc = RunConfig(
        nx=int(p.get("nx", 512)), nz=int(p.get("nz", 300)),
        xlength_cm=float(p.get("xlength", 800e8)), timestep=float(p.get("timestep", 2.0)),
        npmlbot=int(p.get("npmlbot", 10)), npmltop=int(p.get("npmltop", 10)),
        npmlhor=int(p.get("npmlhor", 9)), excitdep_cm=float(p.get("excitdep", -1.5e7)),
        obsheight_cm=float(p.get("obsheight", 2e7)), flows=bool(p.get("flows", True)),
        adjoint=adjoint, outputcad=float(p.get("outputcad", 30.0)),
        cadforcing=float(p.get("cadforcing", 30.0)), solartime_h=float(p.get("solartime", 4.0)),
    )
    if nsteps is None:
        nsteps = reference_maxtime(rc.solartime_h, rc.timestep, rc.cadforcing, nupeak) + 1
    return rc.replace(nsteps=nsteps)
