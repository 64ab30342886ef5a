"""Checkpoint files in the reference's IOS format (restart interchange).

The reference writes its final state as a pair of files (src/io.f90:93-114,
156-178 through src/ios_unstrc.f90:141-297):

  <base>.cd   text control data: the array length, the numbers of parameters
              and time steps, info lines, parameter names, time-step numbers
  <base>.s8   unformatted direct-access records of big-endian FP64 (the build
              uses ifort -convert big_endian, CMakeLists.txt:28-32); record
              r = (nt-1)*mp + np holds parameter np of time step nt, one value
              per cell, with no record markers.  <base>.s4 is the FP32 variant.

The save file holds the four conservative variables at cell centres.  Its
first header field ("number of nodes") carries ncells and the second carries
nnodes (src/io.f90:112-113, "#ncells and #nodes are replaced"), which is what
the restart reader expects (src/initialize.f90:60-71 passes ncells_r in that
slot).  A restart (ntstart > 1) reads the same layout from <base> "cont".

Only the layout is shared with the reference; the code is this project's own.
"""
from __future__ import annotations

import dataclasses
import os

import numpy as np

MAXLEN = 72  # character length of an info line (src/ios_unstrc.f90:37)
FEXT = {1: ".s4", 2: ".s8"}
DTYPE = {1: ">f4", 2: ">f8"}
SAVE_PARAMS = ("rho", "rhou", "rhov", "rhoE")


class IosError(ValueError):
    """A control or data file that does not match what the reader needs
    (the reference stops the program in these cases)."""


@dataclasses.dataclass
class ControlData:
    """Contents of a .cd file.  `m1` is the record length (values per
    record); `m2` the second size field."""

    m1: int
    m2: int
    params: list[str]
    info: list[str]
    itimes: list[int]

    @property
    def mp(self) -> int:
        return len(self.params)

    @property
    def mt(self) -> int:
        return len(self.itimes)


def _line72(s: str) -> str:
    return "   " + s[:MAXLEN].ljust(MAXLEN)


def format_cd(cd: ControlData) -> str:
    """Text of a .cd file, the layout of writecd (src/ios_unstrc.f90:229-247)."""
    out = [f"     number of nodes = {cd.m1}",
           f"     number of cells = {cd.m2}",
           f"     number of parameters = {cd.mp:5d}",
           f"     number of timesteps  = {cd.mt:5d}",
           "",
           f"     Information about file :   ({len(cd.info):3d}  info lines )"]
    out += [_line72(s) for s in cd.info]
    # list-directed write: the record starts with one blank
    out.append("      Information about parameters :")
    out += [_line72(s) for s in cd.params]
    out.append("  Numbers of timesteps :")
    it = list(cd.itimes)[:5000]
    for k in range(0, len(it), 6):
        out.append("".join(f"  {t:10d}" for t in it[k:k + 6]))
    return "\n".join(out) + "\n"


def _int_at(line: str, col: int, width: int | None, what: str) -> int:
    field = line[col:] if width is None else line[col:col + width]
    try:
        return int(field.split()[0])
    except (ValueError, IndexError):
        raise IosError(f"control file: cannot read {what} from {line!r}") from None


def parse_cd(text: str) -> ControlData:
    """Reads a .cd file by the column layout readcd uses
    (src/ios_unstrc.f90:489-501: 23x,i / 23x,i / 28x,i5 / 28x,i5 / blank /
    33x,i3, then the info lines, a skipped line, the parameter lines, a
    skipped line and the time-step numbers read list-directed)."""
    L = text.split("\n")
    if len(L) < 6:
        raise IosError("control file: truncated header")
    m1 = _int_at(L[0], 23, None, "the first size")
    m2 = _int_at(L[1], 23, None, "the second size")
    mp = _int_at(L[2], 28, 5, "the number of parameters")
    mt = _int_at(L[3], 28, 5, "the number of time steps")
    minf = _int_at(L[5], 33, 3, "the number of info lines")
    k = 6
    need = k + minf + 1 + mp + 1
    if len(L) < need:
        raise IosError("control file: truncated info or parameter lines")
    info = [s[3:3 + MAXLEN].rstrip() for s in L[k:k + minf]]
    k += minf + 1
    params = [s[3:3 + MAXLEN].rstrip() for s in L[k:k + mp]]
    k += mp + 1
    vals = " ".join(L[k:]).split()
    nt = min(mt, 5000)
    if len(vals) < nt:
        raise IosError("control file: fewer time-step numbers than declared")
    itimes = [int(v) for v in vals[:nt]]
    return ControlData(m1, m2, params, info, itimes)


def write_records(path: str, records, imach: int = 2) -> None:
    """Data file: records one after the other, each one array of m1 values."""
    with open(path, "wb") as f:
        for r in records:
            f.write(np.ascontiguousarray(r, dtype=np.float64).astype(DTYPE[imach]).tobytes())


def read_record(path: str, m1: int, mp: int, nt: int, np_: int, imach: int = 2) -> np.ndarray:
    """Record (nt, np) of a data file (1-based, src/ios_unstrc.f90:640-651)."""
    if nt < 1 or np_ < 1 or np_ > mp:
        raise IosError(f"record index out of range: nt={nt}, np={np_}, mp={mp}")
    size = np.dtype(DTYPE[imach]).itemsize
    rec = (nt - 1) * mp + (np_ - 1)
    with open(path, "rb") as f:
        f.seek(rec * m1 * size)
        buf = f.read(m1 * size)
    if len(buf) != m1 * size:
        raise IosError(f"{path}: record {rec + 1} is beyond the end of the file")
    return np.frombuffer(buf, dtype=DTYPE[imach]).astype(np.float64)


def save_control(ncells: int, nnodes: int, ntstart: int, ntimes: int) -> ControlData:
    """Control data of the save file (src/io.f90:93-113)."""
    return ControlData(m1=ncells, m2=nnodes, params=list(SAVE_PARAMS),
                       info=["number of time-step computed = " + f"{ntimes:6d}".rstrip(),
                             "conservatve variables are saved in cell centers",
                             "#ncells and #nodes are replaced",
                             " "],
                       itimes=[ntstart - 1 + ntimes])


def write_save(directory: str, cvar: np.ndarray, nnodes: int, ntstart: int, ntimes: int, base: str = "save",
               imach: int = 2) -> tuple[str, str]:
    """Writes <base>.cd and <base>.s8 (or .s4) for a state cvar [ncells][4]
    (write_save_ios, src/io.f90:156-178).  Returns the two paths."""
    cvar = np.asarray(cvar, dtype=np.float64)
    if cvar.ndim != 2 or cvar.shape[1] != 4:
        raise IosError("cvar must have shape (ncells, 4)")
    cd = save_control(cvar.shape[0], nnodes, ntstart, ntimes)
    p_cd = os.path.join(directory, base + ".cd")
    p_s = os.path.join(directory, base + FEXT[imach])
    with open(p_cd, "w") as f:
        f.write(format_cd(cd))
    write_records(p_s, [cvar[:, k] for k in range(4)], imach)
    return p_cd, p_s


def read_cont(directory: str, ncells: int, nnodes: int, base: str = "cont", imach: int = 2) -> np.ndarray:
    """Restart state cvar [ncells][4] from <base>.cd / <base>.s8, with the
    reference's checks (src/initialize.f90:56-77): the grid sizes must match
    and the file must hold one time step of four parameters."""
    p_cd = os.path.join(directory, base + ".cd")
    p_s = os.path.join(directory, base + FEXT[imach])
    if not os.path.exists(p_cd) or not os.path.exists(p_s):
        raise IosError(f"continuation files {p_cd} / {p_s} not found")
    with open(p_cd) as f:
        cd = parse_cd(f.read())
    ncells_r, nnodes_r = cd.m1, cd.m2
    if ncells_r != ncells or nnodes_r != nnodes:
        raise IosError(f"dimension between grid and cont files does not match: file ncells={ncells_r} "
                       f"nnodes={nnodes_r}, grid ncells={ncells} nnodes={nnodes}")
    if cd.mt > 1 or cd.mp != 4:
        raise IosError(f"nt>1 or #parameters/=nvar: nt={cd.mt}, parameters={cd.mp}")
    out = np.empty((ncells, 4), np.float64)
    for k in range(4):
        out[:, k] = read_record(p_s, cd.m1, cd.mp, 1, k + 1, imach)
    return out
