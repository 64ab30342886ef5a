"""Batched independent cases through the C-ABI (fvs_batch_*).

All cases share the scheme; each has its own mesh, Mach number and angle of
attack.  One launch advances every active case per chunk of steps (a
cooperative persistent kernel, or a CUDA graph of tile launches per step);
converged cases leave the work lists.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import capi
from .solver import FvsError


class Batch:
    def __init__(self, meshes, options, host_threads: int = 0):
        if len(meshes) != len(options) or not meshes:
            raise ValueError("one Options per mesh")
        self._lib = capi.load()
        self._arrays = [capi.MeshArrays(m) for m in meshes]
        self._meshes = (capi.FvsMesh * len(meshes))(*[a.struct for a in self._arrays])
        self._opts = (capi.FvsOptions * len(options))(*[o.to_struct() for o in options])
        h = C.c_void_p()
        rc = self._lib.fvs_batch_create(self._meshes, self._opts, len(meshes), int(host_threads), C.byref(h))
        if rc != capi.FVS_OK:
            raise FvsError(rc, self._lib.fvs_batch_last_error(None).decode())
        self._h = h
        self.ncases = len(meshes)
        self.case_cells = [m.ncells for m in meshes]

    def _check(self, rc):
        if rc != capi.FVS_OK:
            raise FvsError(rc, self._lib.fvs_batch_last_error(self._h).decode())

    def close(self):
        if getattr(self, "_h", None):
            self._lib.fvs_batch_destroy(self._h)
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

    def info(self) -> dict:
        nc, ne = C.c_int32(0), C.c_int32(0)
        launch = (C.c_int32 * 4)()
        self._check(self._lib.fvs_batch_info(self._h, C.byref(nc), C.byref(ne), launch))
        return {"ncells": nc.value, "nedges": ne.value, "block": launch[0], "tile": launch[1],
                "blocks_per_sm": launch[2], "graph": bool(launch[3] & 1), "tiled": bool(launch[3] & 2),
                "fused": bool(launch[3] & 4)}

    def initialize_solution(self):
        self._check(self._lib.fvs_batch_init_state(self._h))

    def set_state(self, icase: int, cvar) -> None:
        a = np.ascontiguousarray(cvar, np.float64).reshape(self.case_cells[icase], 4)
        self._check(self._lib.fvs_batch_set_state(self._h, int(icase), capi.ptr(a)))

    def get_state(self, icase: int) -> np.ndarray:
        out = np.empty((self.case_cells[icase], 4), np.float64)
        self._check(self._lib.fvs_batch_get_state(self._h, int(icase), capi.ptr(out)))
        return out

    def steps(self, nsteps: int):
        """nsteps steps of all cases; returns (norms [ncases][nsteps][4], ms)."""
        norms = np.empty((self.ncases, nsteps, 4), np.float64)
        ms = C.c_float(0)
        self._check(self._lib.fvs_batch_steps(self._h, int(nsteps), capi.ptr(norms), C.byref(ms)))
        return norms, ms.value

    def autotune(self, trial_steps: int = 3) -> float:
        ms = C.c_float(0)
        self._check(self._lib.fvs_batch_autotune(self._h, int(trial_steps), C.byref(ms)))
        return ms.value

    def set_launch(self, block: int, tile: int, blocks_per_sm: int):
        self._check(self._lib.fvs_batch_set_launch(self._h, block, tile, blocks_per_sm))

    def set_precision(self, precision: int):
        """Switch all cases to another arithmetic (FP64 state kept)."""
        self._check(self._lib.fvs_batch_set_precision(self._h, int(precision)))

    def set_barrier_budget(self, seconds: float):
        self._check(self._lib.fvs_batch_set_barrier_budget(self._h, float(seconds)))

    def run_to_drop(self, max_steps: int, drop: float = 1e-10, chunk: int = 50):
        """Returns (steps_done [ncases], first [ncases,4], last [ncases,4], ms)."""
        done = np.zeros(self.ncases, np.int32)
        first = np.zeros((self.ncases, 4))
        last = np.zeros((self.ncases, 4))
        ms = C.c_float(0)
        self._check(self._lib.fvs_batch_run_to_drop(self._h, int(max_steps), float(drop), int(chunk), capi.ptr(done),
                                                    capi.ptr(first), capi.ptr(last), C.byref(ms)))
        return done, first, last, ms.value

    def set_mode(self, tiled: bool, fused: bool = True, dc_fused: bool = False, fixed: bool = False) -> None:
        """Launch mode: a persistent cooperative kernel per chunk (tiled False)
        or a graph of per-phase tile launches per step (True).  fused: first-
        order mixed stages evaluate the flux per cell in one phase per stage
        (where the stage count is even); dc_fused: the same for the
        defect-correction stages; fixed: run_to_level keeps this shape instead
        of trying others as the active set shrinks."""
        mode = (1 if tiled else 0) | (0 if fused else 2) | (4 if dc_fused else 0) | (8 if fixed else 0)
        self._check(self._lib.fvs_batch_set_mode(self._h, mode))

    def set_groups(self, group=None) -> None:
        """Cases with the same group id stop together when the first of them
        meets its target (None: every case alone)."""
        if group is None:
            self._check(self._lib.fvs_batch_set_groups(self._h, None))
            return
        g = np.ascontiguousarray(group, np.int32)
        if g.shape != (self.ncases,):
            raise ValueError("one group id per case")
        self._check(self._lib.fvs_batch_set_groups(self._h, capi.ptr(g)))

    def run_to_level(self, max_steps: int, levels, chunk: int = 50, dc: bool = False):
        """Steps until each case's RMS(dU_k) <= levels[c, k] for all k; same
        returns as run_to_drop.  dc: defect-correction iteration (first-order
        steady batches; leaves the batch in FP64)."""
        lv = np.ascontiguousarray(np.broadcast_to(np.asarray(levels, np.float64).reshape(self.ncases, -1),
                                                  (self.ncases, 4)), np.float64)
        done = np.zeros(self.ncases, np.int32)
        first = np.zeros((self.ncases, 4))
        last = np.zeros((self.ncases, 4))
        ms = C.c_float(0)
        fn = self._lib.fvs_batch_run_to_level_dc if dc else self._lib.fvs_batch_run_to_level
        self._check(fn(self._h, int(max_steps), capi.ptr(lv), int(chunk), capi.ptr(done), capi.ptr(first),
                       capi.ptr(last), C.byref(ms)))
        return done, first, last, ms.value
