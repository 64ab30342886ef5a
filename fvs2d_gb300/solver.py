"""Host-side mirror of the reference's hot-path module API.

The reference exposes its residual-and-update loop as Fortran module
procedures over module-global arrays:

  compute_residual(time)          src/residual.f90:23      -> Solver.compute_residual
  time_integration(t1, nsub)      src/runge_kutta.f90:94   -> Solver.time_integration
  initialize_solution             src/initialize.f90:19    -> Solver.initialize_solution
  error_isentropic_vortex(time)   src/mms.f90:271          -> Solver.error_isentropic_vortex
  cvar / resid / grad / phi_lim / ws_nrml   src/data_solution.f90:16-21 -> properties

Every call goes through the C-ABI of libfvs2d_gb300.so; the arithmetic runs in
the sm_103a kernels.  Errors raise :class:`FvsError` carrying the FVS_* code.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import capi
from .meshgen import Mesh
from .options import Options


class FvsError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{capi.ERROR_NAMES.get(code, code)}: {msg}")
        self.code = code


class Solver:
    """One mesh + one scheme on the GPU (one CUDA stream)."""

    def __init__(self, mesh: Mesh, options: Options):
        self._lib = capi.load()
        self.mesh = mesh
        self.options = options
        self._m = capi.MeshArrays(mesh)
        self._o = options.to_struct()
        h = C.c_void_p()
        rc = self._lib.fvs_create(C.byref(self._m.struct), C.byref(self._o), C.byref(h))
        if rc != capi.FVS_OK:
            raise FvsError(rc, self._lib.fvs_last_error(None).decode())
        self._h = h
        s = capi.FvsSizes()
        self._check(self._lib.fvs_get_sizes(self._h, C.byref(s)))
        self.sizes = s
        self.ncells = s.ncells

    # -- plumbing -----------------------------------------------------------
    def _check(self, rc: int) -> None:
        if rc != capi.FVS_OK:
            raise FvsError(rc, self._lib.fvs_last_error(self._h).decode())

    def close(self) -> None:
        if getattr(self, "_h", None):
            self._lib.fvs_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # -- state --------------------------------------------------------------
    def initialize_solution(self, cont_dir: str = ".") -> None:
        """Free stream / vortex / MMS start (ntstart <= 1), or a restart from
        cont.cd + cont.s8 in `cont_dir` (ntstart > 1, src/initialize.f90:56-77)."""
        if self.options.ntstart > 1:
            from . import ios
            self.cvar = ios.read_cont(cont_dir, self.ncells, self.mesh.nnodes)
            return
        self._check(self._lib.fvs_init_state(self._h))

    def write_save(self, directory: str, ntimes: int, imach: int = 2) -> tuple[str, str]:
        """save.cd + save.s8 of the current state (write_save_ios,
        src/io.f90:93-114,156-178); ntimes = steps computed in this run."""
        from . import ios
        return ios.write_save(directory, self.cvar, self.mesh.nnodes, self.options.ntstart, ntimes, imach=imach)

    @property
    def cvar(self) -> np.ndarray:
        """Conservative state, shape (ncells, 4), reference cell order."""
        out = np.empty((self.ncells, 4), np.float64)
        self._check(self._lib.fvs_get_state(self._h, capi.ptr(out)))
        return out

    @cvar.setter
    def cvar(self, value) -> None:
        a = np.ascontiguousarray(value, np.float64).reshape(self.ncells, 4)
        self._check(self._lib.fvs_set_state(self._h, capi.ptr(a)))

    def set_state_ptr(self, host_ptr: int) -> None:
        """Upload from a caller-owned (e.g. pinned) host buffer of ncells*4 doubles."""
        self._check(self._lib.fvs_set_state(self._h, C.c_void_p(host_ptr)))

    def get_state_ptr(self, host_ptr: int) -> None:
        self._check(self._lib.fvs_get_state(self._h, C.c_void_p(host_ptr)))

    # -- hot path -----------------------------------------------------------
    def compute_residual(self, time: float = 0.0):
        """resid (= dU/dt = -R/vol) and ws_nrml of the current state."""
        r = np.empty((self.ncells, 4), np.float64)
        w = np.empty(self.ncells, np.float64)
        self._check(self._lib.fvs_residual(self._h, float(time), capi.ptr(r), capi.ptr(w)))
        return r, w

    def gradient(self):
        """grad (2, ncells, 4) and phi_lim (ncells) of the last residual."""
        g = np.empty((2, self.ncells, 4), np.float64)
        p = np.empty(self.ncells, np.float64)
        self._check(self._lib.fvs_get_gradient(self._h, capi.ptr(g), capi.ptr(p)))
        return g, p

    def time_integration(self, t1: float, nsteps: int) -> np.ndarray:
        """nsteps RK steps from t1; returns the (nsteps, 4) RMS(|U-U0|) log."""
        out = np.empty((max(nsteps, 1), 4), np.float64)
        self._check(self._lib.fvs_time_integration(self._h, float(t1), int(nsteps), capi.ptr(out)))
        return out[:nsteps]

    def run_to_drop(self, t1: float, max_steps: int, drop: float = 1e-10, check_every: int = 100):
        """Steps until RMS(dU_rho) falls to drop x its first value; returns (steps, norms)."""
        out = np.empty((max_steps, 4), np.float64)
        n = C.c_int32(0)
        rc = self._lib.fvs_run_to_drop(self._h, float(t1), int(max_steps), float(drop), int(check_every),
                                       C.byref(n), capi.ptr(out))
        self._check(rc)
        return n.value, out[: n.value]

    def steps_device(self, nsteps: int) -> float:
        """Device-resident steps; returns CUDA-event milliseconds."""
        ms = C.c_float(0)
        self._check(self._lib.fvs_steps_device(self._h, int(nsteps), C.byref(ms)))
        return ms.value

    def profile_step(self) -> list:
        cap = 64
        names = C.create_string_buffer(32 * cap)
        ms = (C.c_float * cap)()
        n = C.c_int32(0)
        self._check(self._lib.fvs_profile_step(self._h, cap, C.byref(n), names, ms))
        raw = names.raw
        return [(raw[32 * i:32 * i + 32].split(b"\0")[0].decode(), ms[i]) for i in range(n.value)]

    def current_dt(self) -> float:
        """The global dt in use (derived from the CFL at the first step when
        dt_from_cfl is set)."""
        s = capi.FvsSizes()
        self._check(self._lib.fvs_get_sizes(self._h, C.byref(s)))
        return float(s.dt)

    def launches_per_step(self) -> int:
        n = C.c_int32(0)
        self._check(self._lib.fvs_launches_per_step(self._h, C.byref(n)))
        return n.value

    # -- diagnostics --------------------------------------------------------
    def error_isentropic_vortex(self, time: float) -> np.ndarray:
        e = np.empty(13, np.float64)
        self._check(self._lib.fvs_vortex_error(self._h, float(time), capi.ptr(e)))
        return e

    def wall_loads(self, ib: int = 1) -> tuple[np.ndarray, dict]:
        """Wall pressure and loads of slip-wall boundary ib (1-based), the
        numbers of write_inst_cp_un (src/io.f90:340-446): the edge table
        [nedges][4] = (x_face, cp_wall, cp_cell, un) and a dict of cl, cd,
        cl1, cd1, un_max, un_l2, un_l1, cn, ca, cn1, ca1."""
        n = int(self.mesh.bndry_cells[ib - 1].size) if 1 <= ib <= len(self.mesh.bndry_cells) else 0
        e = np.empty((max(n, 1), 4), np.float64)
        loads = np.empty(11, np.float64)
        self._check(self._lib.fvs_wall_loads(self._h, int(ib), capi.ptr(e), capi.ptr(loads)))
        return e[:n], dict(zip(WALL_LOAD_NAMES, loads.tolist()))

    def write_cp(self, path: str, ib: int = 1, sol_time: float = 0.0) -> dict:
        """One zone of the reference's Tecplot cp file (x, cp_w, cp_cell per
        wall edge, src/io.f90:387-409); returns the loads."""
        e, loads = self.wall_loads(ib)
        with open(path, "w") as f:
            f.write('TITLE     = "cp"\n')
            f.write('VARIABLES = "x" "cp_w" "cp_cell"\n')
            f.write(f"ZONE I={e.shape[0]} J=1\n")
            f.write(f"STRANDID=1, SOLUTIONTIME={_e16(sol_time)}\n")
            for xf, cp, cp1, _ in e:
                f.write(f"{_e16(xf)} {_e16(cp)} {_e16(cp1)} \n")
        return loads

    def mms_source(self) -> np.ndarray:
        s = np.empty((self.ncells, 4), np.float64)
        self._check(self._lib.fvs_mms_source(self._h, capi.ptr(s)))
        return s

    def export(self, name: str) -> np.ndarray:
        """Setup array by name (reference numbering), see capi export names."""
        n = C.c_int64(0)
        self._check(self._lib.fvs_export_size(self._h, name.encode(), C.byref(n)))
        dtype = np.int32 if name in INT_EXPORTS else np.float64
        out = np.empty(max(n.value // np.dtype(dtype).itemsize, 1), dtype)
        if n.value:
            self._check(self._lib.fvs_export(self._h, name.encode(), capi.ptr(out), n.value))
        return out[: n.value // np.dtype(dtype).itemsize]


WALL_LOAD_NAMES = ("cl", "cd", "cl1", "cd1", "un_max", "un_l2", "un_l1", "cn", "ca", "cn1", "ca1")


def _e16(x: float) -> str:
    """Fortran e16.8: 0.dddddddd E+xx, right-justified in 16 columns."""
    if not np.isfinite(x):
        return f"{x!s:>16}"
    if x == 0.0:
        return "0.00000000E+00".rjust(16)
    mant, ex = f"{abs(x):.7E}".split("E")
    return (("-" if x < 0 else "") + f"0.{mant.replace('.', '')}E{int(ex) + 1:+03d}").rjust(16)


INT_EXPORTS = {"cell_nghbr", "cell_nghbre", "cell_edge", "edge_nodes", "edge_cells", "edge_intr", "edge_bndr",
               "bedge_cell", "cell_intr", "cell_bndr", "bndry_edges", "stencil_ptr", "stencil_cell"}
FLOAT_EXPORTS = {"cell_xy", "cell_vol", "cell_nrmlsign", "edge_geom", "stencil_coef", "stencil_w", "coef0",
                 "coefedg", "eps2"}
