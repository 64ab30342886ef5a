"""Scheme options: the flags of the reference's input module.

:class:`Options` carries the values ``input_read`` (src/input.f90:64-413) reads
from ``fvs2d.input`` and ``mms_init`` (src/mms.f90:45-63) reads from
``fvs2d.vortex``, under the same meaning, plus the extensions this library
adds.  :func:`read_input` parses the reference's positional text files, so the
reference's own inputs drive the device path.
"""
from __future__ import annotations

import dataclasses
import os

from . import capi

GRAD = {"ggcb": 1, "ggnb": 2, "lsq": 3}
LIMITER = {"none": 0, "venk": 1, "barth": 2, "albada": 3}
RECON = {"upwind1": 1, "upwind2": 2, "umuscl": 3}


@dataclasses.dataclass
class Options:
    gamma: float = 1.4
    mach_inf: float = 0.5
    aoa_inf_deg: float = 0.0
    dt: float = 0.01
    cfl: float = 1.0
    steady: bool = False
    vortex: bool = False
    ntstart: int = 1
    grad_method: int = 3          # 1 GGCB, 2 GGNB, 3 LSQ
    lsq_stencil: str = "fn"       # 'fn' / 'nn'
    lsq_pow: float = 0.0
    limiter: int = 0              # 0 none, 1 venk, 2 barth, 3 albada
    reconst: int = 2              # 1 upwind-1st, 2 upwind-2nd, 3 UMUSCL
    umuscl: float = 0.0
    flux: int = 1                 # Roe
    rk_nstages: int = 4
    rk_order: int = 4
    ssprk: bool = False
    vortex_x: float = 5.0
    vortex_y: float = 5.0
    vortex_kappa: float = 1.0
    vortex_inf: tuple = (1.0, 0.2, 0.0, 1.0)
    # extensions
    dt_from_cfl: bool = False
    precision: int = capi.PREC_FP64
    diverge_factor: float = 0.0
    # input-file items outside the hot path, kept for completeness
    grid_base: str = ""
    ntimes: int = 0
    nsaves: int = 1

    def to_struct(self) -> capi.FvsOptions:
        s = capi.FvsOptions()
        s.gamma = self.gamma
        s.mach_inf = self.mach_inf
        s.aoa_inf_deg = self.aoa_inf_deg
        s.dt = self.dt
        s.cfl = self.cfl
        s.steady = int(bool(self.steady))
        s.vortex = int(bool(self.vortex))
        s.ntstart = int(self.ntstart)
        s.grad_method = int(self.grad_method)
        s.lsq_stencil = 1 if str(self.lsq_stencil).lower() == "nn" else 0
        s.lsq_pow = self.lsq_pow
        s.limiter = int(self.limiter)
        s.reconst = int(self.reconst)
        s.umuscl = self.umuscl if int(self.reconst) == 3 else 0.0
        s.flux = int(self.flux)
        s.rk_nstages = int(self.rk_nstages)
        s.rk_order = int(self.rk_order)
        s.ssprk = int(bool(self.ssprk))
        s.vortex_x = self.vortex_x
        s.vortex_y = self.vortex_y
        s.vortex_kappa = self.vortex_kappa
        for k in range(4):
            s.vortex_inf[k] = self.vortex_inf[k]
        s.dt_from_cfl = int(bool(self.dt_from_cfl))
        s.precision = int(self.precision)
        s.diverge_factor = self.diverge_factor
        return s

    def replace(self, **kw) -> "Options":
        return dataclasses.replace(self, **kw)


def _num(tok: str) -> float:
    return float(tok.replace("d", "e").replace("D", "e"))


def _logical(tok: str) -> bool:
    t = tok.strip().strip(".").upper()
    if t.startswith("T"):
        return True
    if t.startswith("F"):
        return False
    raise ValueError(f"not a Fortran logical: {tok!r}")


def _fields(line: str, n: int) -> list:
    """First n list-directed values of a line (comma or blank separated;
    the '---' annotations of the reference's files are ignored)."""
    body = line.split("---")[0].split("!")[0]
    toks = [t for t in body.replace(",", " ").split() if t]
    if len(toks) < n:
        raise ValueError(f"expected {n} values in {line!r}")
    return toks[:n]


def read_input(path: str, vortex_path: str | None = None) -> Options:
    """Parse an fvs2d.input file (positional, src/input.f90:86-118) and, when
    the vortex flag is set, its fvs2d.vortex companion (src/mms.f90:55-62).

    Errors mirror the reference's checks (which stop the program there) as
    ValueError."""
    with open(path) as f:
        lines = f.read().splitlines()
    L = iter(lines)
    for _ in range(3):
        next(L)
    dchar_grid = next(L)
    o = Options()
    next(L)  # Reynolds number (viscous terms are not implemented by the reference)
    o.mach_inf = _num(_fields(next(L), 1)[0])
    o.aoa_inf_deg = _num(_fields(next(L), 1)[0])
    o.gamma = _num(_fields(next(L), 1)[0])
    next(L)
    o.dt = _num(_fields(next(L), 1)[0])
    o.ntimes = int(_fields(next(L), 1)[0])
    o.nsaves = int(_fields(next(L), 1)[0])
    o.ntstart = int(_fields(next(L), 1)[0])
    st, cfl = _fields(next(L), 2)
    o.steady, o.cfl = _logical(st), _num(cfl)
    o.vortex = _logical(_fields(next(L), 1)[0])
    next(L)
    next(L)  # output variables
    next(L)  # s4 / s8
    for _ in range(3):
        next(L)
    g = _fields(next(L), 3)
    method, nghbr, pw = int(g[0]), g[1].lower(), _num(g[2])
    lim = int(_fields(next(L), 1)[0])
    rc = _fields(next(L), 2)
    recon, kappa = int(rc[0]), _num(rc[1])
    fl = int(_fields(next(L), 1)[0])
    next(L)
    o.rk_nstages = int(_fields(next(L), 1)[0])
    o.rk_order = int(_fields(next(L), 1)[0])
    o.ssprk = _logical(_fields(next(L), 1)[0])
    # src/input.f90:140: MMS start disables the vortex
    if o.ntstart == 0:
        o.vortex = False
    # grid base name: text before the first '-' (src/input.f90:166-175)
    o.grid_base = dchar_grid.split("-")[0].strip()
    if method not in (1, 2, 3):
        raise ValueError("check cell-center gradient scheme in input file")
    if method == 3 and nghbr not in ("fn", "nn"):
        raise ValueError("check Least-Squares gradient scheme in input file")
    o.grad_method, o.lsq_stencil, o.lsq_pow = method, nghbr if method == 3 else "fn", pw
    if lim not in (0, 1, 2, 3):
        raise ValueError("check gradient limiter scheme in input file")
    o.limiter = lim
    if recon not in (1, 2, 3):
        raise ValueError("check face reconstruction scheme in input file")
    o.reconst, o.umuscl = recon, (kappa if recon == 3 else 0.0)
    if fl != 1:
        raise ValueError("check inviscid flux discretization scheme in input file")
    o.flux = 1
    if o.vortex:
        vp = vortex_path or os.path.join(os.path.dirname(path), "fvs2d.vortex")
        with open(vp) as f:
            vl = f.read().splitlines()
        cx, cy = _fields(vl[0], 2)
        o.vortex_x, o.vortex_y = _num(cx), _num(cy)
        o.vortex_kappa = _num(_fields(vl[1], 1)[0])
        o.vortex_inf = tuple(_num(_fields(vl[2 + k], 1)[0]) for k in range(4))
    return o
