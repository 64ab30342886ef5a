"""ctypes driver of the CPU oracle (oracle/fvs_oracle.c) for the tests.

The oracle is test infrastructure: it is the checker the device results are
compared with, never a code path of the product.
"""
from __future__ import annotations

import ctypes as C
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from fvs2d_gb300 import capi  # noqa: E402
from fvs2d_gb300.solver import INT_EXPORTS, WALL_LOAD_NAMES  # noqa: E402

import build_oracle  # noqa: E402

_LIBS = {}


def load(timed: bool = False) -> C.CDLL:
    """The checker's build, or (timed) the -O3 -ffast-math build that only
    times the CPU baseline."""
    if timed not in _LIBS:
        try:
            path = build_oracle.build(timed=timed)
        except RuntimeError:
            if not timed:
                raise
            # the baseline falls back to the checker's build (Oracle.timed says which ran)
            _LIBS[True] = load(False)
            return _LIBS[True]
        lib = C.CDLL(path)
        vp = C.c_void_p
        sig = {
            "orc_create": (C.c_int, [C.POINTER(capi.FvsMesh), C.POINTER(capi.FvsOptions), C.POINTER(vp), C.c_char_p, C.c_int]),
            "orc_destroy": (None, [vp]),
            "orc_sizes": (C.c_int, [vp, C.POINTER(capi.FvsSizes)]),
            "orc_export_size": (C.c_int, [vp, C.c_char_p, C.POINTER(C.c_int64)]),
            "orc_export": (C.c_int, [vp, C.c_char_p, vp, C.c_int64]),
            "orc_init_state": (C.c_int, [vp]),
            "orc_set_state": (C.c_int, [vp, vp]),
            "orc_get_state": (C.c_int, [vp, vp]),
            "orc_residual": (C.c_int, [vp, C.c_double, vp, vp, C.c_int]),
            "orc_get_gradient": (C.c_int, [vp, vp, vp]),
            "orc_wall_loads": (C.c_int, [vp, C.c_int, vp, vp]),
            "orc_time_integration": (C.c_int, [vp, C.c_double, C.c_int, vp, C.c_int]),
            "orc_vortex_error": (C.c_int, [vp, C.c_double, vp]),
            "orc_mms_source": (C.c_int, [vp, vp]),
            "orc_dt": (C.c_double, [vp]),
        }
        for k, (r, a) in sig.items():
            f = getattr(lib, k)
            f.restype = r
            f.argtypes = a
        _LIBS[timed] = lib
    return _LIBS[timed]


class OracleError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{capi.ERROR_NAMES.get(code, code)}: {msg}")
        self.code = code


class Oracle:
    """Same surface as fvs2d_gb300.Solver, computed by the CPU restatement."""

    def __init__(self, mesh, options, nthreads: int = 1, timed: bool = False):
        self._lib = load(timed)
        self.timed = timed and self._lib is not load(False)  # the -O3 -ffast-math build is the one running
        self._m = capi.MeshArrays(mesh)
        self._o = options.to_struct()
        self.nthreads = nthreads
        h = C.c_void_p()
        err = C.create_string_buffer(512)
        rc = self._lib.orc_create(C.byref(self._m.struct), C.byref(self._o), C.byref(h), err, 512)
        if rc:
            raise OracleError(rc, err.value.decode())
        self._h = h
        s = capi.FvsSizes()
        self._lib.orc_sizes(self._h, C.byref(s))
        self.sizes = s
        self.ncells = s.ncells

    def close(self):
        if getattr(self, "_h", None):
            self._lib.orc_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def initialize_solution(self):
        self._lib.orc_init_state(self._h)

    @property
    def cvar(self):
        out = np.empty((self.ncells, 4))
        self._lib.orc_get_state(self._h, capi.ptr(out))
        return out

    @cvar.setter
    def cvar(self, v):
        a = np.ascontiguousarray(v, np.float64).reshape(self.ncells, 4)
        self._lib.orc_set_state(self._h, capi.ptr(a))

    def compute_residual(self, time=0.0):
        r = np.empty((self.ncells, 4))
        w = np.empty(self.ncells)
        self._lib.orc_residual(self._h, float(time), capi.ptr(r), capi.ptr(w), self.nthreads)
        return r, w

    def gradient(self):
        g = np.empty((2, self.ncells, 4))
        p = np.empty(self.ncells)
        self._lib.orc_get_gradient(self._h, capi.ptr(g), capi.ptr(p))
        return g, p

    def wall_loads(self, ib=1, n_edges=None):
        """(edge table [n][4] = xf, cp, cp_cell, un; loads dict) of boundary ib."""
        loads = np.empty(11)
        n = n_edges if n_edges is not None else 0
        e = np.empty((max(n, 1), 4))
        rc = self._lib.orc_wall_loads(self._h, int(ib), capi.ptr(e) if n else None, capi.ptr(loads))
        if rc:
            raise OracleError(rc, "wall_loads")
        return e[:n], dict(zip(WALL_LOAD_NAMES, loads))

    def time_integration(self, t1, nsteps):
        out = np.empty((max(nsteps, 1), 4))
        self._lib.orc_time_integration(self._h, float(t1), int(nsteps), capi.ptr(out), self.nthreads)
        return out[:nsteps]

    def error_isentropic_vortex(self, time):
        e = np.empty(13)
        self._lib.orc_vortex_error(self._h, float(time), capi.ptr(e))
        return e

    def mms_source(self):
        s = np.empty((self.ncells, 4))
        self._lib.orc_mms_source(self._h, capi.ptr(s))
        return s

    @property
    def dt(self):
        return self._lib.orc_dt(self._h)

    def export(self, name):
        n = C.c_int64(0)
        rc = self._lib.orc_export_size(self._h, name.encode(), C.byref(n))
        if rc:
            raise OracleError(rc, f"no export named {name}")
        dtype = np.int32 if name in INT_EXPORTS else np.float64
        out = np.empty(max(n.value // np.dtype(dtype).itemsize, 1), dtype)
        if n.value:
            self._lib.orc_export(self._h, name.encode(), capi.ptr(out), n.value)
        return out[: n.value // np.dtype(dtype).itemsize]
