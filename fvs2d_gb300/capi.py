"""ctypes declarations of include/fvs2d.h and the library loader.

The structures below mirror the C header field for field; tests use the same
declarations to drive the CPU oracle, whose entry points take the same
structures.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

FVS_OK = 0
FVS_ERR_INVALID = 1
FVS_ERR_MESH = 2
FVS_ERR_CUDA = 3
FVS_ERR_NONFINITE = 4
FVS_ERR_DIVERGED = 5
FVS_ERR_TIMEOUT = 6
FVS_ERR_NOMEM = 7
FVS_ERR_BOUNDS = 8
ERROR_NAMES = {0: "FVS_OK", 1: "FVS_ERR_INVALID", 2: "FVS_ERR_MESH", 3: "FVS_ERR_CUDA", 4: "FVS_ERR_NONFINITE",
               5: "FVS_ERR_DIVERGED", 6: "FVS_ERR_TIMEOUT", 7: "FVS_ERR_NOMEM", 8: "FVS_ERR_BOUNDS"}

PREC_FP64_STRICT = 0
PREC_FP64 = 1
PREC_MIXED = 2
PREC_FP64_DF = 3

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int32)


class FvsMesh(C.Structure):
    _fields_ = [
        ("nnodes", C.c_int32), ("ncells_tri", C.c_int32), ("ncells_quad", C.c_int32),
        ("node_xy", _dp), ("tri_nodes", _ip), ("quad_nodes", _ip),
        ("nbndries", C.c_int32), ("bndry_ncells", _ip), ("bndry_type", _ip), ("bndry_cells", _ip),
        ("period_x", C.c_double), ("period_y", C.c_double),
    ]


class FvsOptions(C.Structure):
    _fields_ = [
        ("gamma", C.c_double), ("mach_inf", C.c_double), ("aoa_inf_deg", C.c_double), ("dt", C.c_double),
        ("cfl", C.c_double), ("steady", C.c_int32), ("vortex", C.c_int32), ("ntstart", C.c_int32),
        ("grad_method", C.c_int32), ("lsq_stencil", C.c_int32), ("lsq_pow", C.c_double), ("limiter", C.c_int32),
        ("reconst", C.c_int32), ("umuscl", C.c_double), ("flux", C.c_int32), ("rk_nstages", C.c_int32),
        ("rk_order", C.c_int32), ("ssprk", C.c_int32), ("vortex_x", C.c_double), ("vortex_y", C.c_double),
        ("vortex_kappa", C.c_double), ("vortex_inf", C.c_double * 4), ("dt_from_cfl", C.c_int32),
        ("precision", C.c_int32), ("diverge_factor", C.c_double),
    ]


class FvsSizes(C.Structure):
    _fields_ = [
        ("nnodes", C.c_int32), ("ncells", C.c_int32), ("ncells_tri", C.c_int32), ("ncells_quad", C.c_int32),
        ("nedges", C.c_int32), ("nedges_intr", C.c_int32), ("nedges_bndr", C.c_int32),
        ("ncells_intr", C.c_int32), ("ncells_bndr", C.c_int32), ("nbndries", C.c_int32),
        ("stencil_len", C.c_int32), ("nstages", C.c_int32), ("heff1", C.c_double), ("heff2", C.c_double),
        ("vol_sum", C.c_double), ("vol_green", C.c_double), ("dt", C.c_double),
    ]


# every symbol the header declares, with its ctypes signature
SIGNATURES = {
    "fvs_options_default": (C.c_int, [C.POINTER(FvsOptions)]),
    "fvs_create": (C.c_int, [C.POINTER(FvsMesh), C.POINTER(FvsOptions), C.POINTER(C.c_void_p)]),
    "fvs_create_host": (C.c_int, [C.POINTER(FvsMesh), C.POINTER(FvsOptions), C.POINTER(C.c_void_p)]),
    "fvs_destroy": (None, [C.c_void_p]),
    "fvs_last_error": (C.c_char_p, [C.c_void_p]),
    "fvs_get_sizes": (C.c_int, [C.c_void_p, C.POINTER(FvsSizes)]),
    "fvs_export_size": (C.c_int, [C.c_void_p, C.c_char_p, C.POINTER(C.c_int64)]),
    "fvs_export": (C.c_int, [C.c_void_p, C.c_char_p, C.c_void_p, C.c_int64]),
    "fvs_init_state": (C.c_int, [C.c_void_p]),
    "fvs_set_state": (C.c_int, [C.c_void_p, C.c_void_p]),
    "fvs_get_state": (C.c_int, [C.c_void_p, C.c_void_p]),
    "fvs_residual": (C.c_int, [C.c_void_p, C.c_double, C.c_void_p, C.c_void_p]),
    "fvs_get_gradient": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p]),
    "fvs_time_integration": (C.c_int, [C.c_void_p, C.c_double, C.c_int32, C.c_void_p]),
    "fvs_run_to_drop": (C.c_int, [C.c_void_p, C.c_double, C.c_int32, C.c_double, C.c_int32, C.POINTER(C.c_int32),
                                  C.c_void_p]),
    "fvs_vortex_error": (C.c_int, [C.c_void_p, C.c_double, C.c_void_p]),
    "fvs_wall_loads": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p]),
    "fvs_mms_source": (C.c_int, [C.c_void_p, C.c_void_p]),
    "fvs_steps_device": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_float)]),
    "fvs_profile_step": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_int32), C.c_char_p, C.POINTER(C.c_float)]),
    "fvs_launches_per_step": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32)]),
    "fvs_device_state": (C.c_int, [C.c_void_p, C.POINTER(C.c_void_p)]),
    "fvs_check_fp64_math": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p]),
    "fvs_tile_plan_info": (C.c_int, [C.POINTER(FvsMesh), C.POINTER(FvsOptions), C.c_void_p]),
    "fvs_debug_set_gather": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32]),
    "fvs_batch_create": (C.c_int, [C.POINTER(FvsMesh), C.POINTER(FvsOptions), C.c_int32, C.c_int32, C.POINTER(C.c_void_p)]),
    "fvs_batch_destroy": (None, [C.c_void_p]),
    "fvs_batch_last_error": (C.c_char_p, [C.c_void_p]),
    "fvs_batch_info": (C.c_int, [C.c_void_p, C.POINTER(C.c_int32), C.POINTER(C.c_int32), C.c_void_p]),
    "fvs_batch_init_state": (C.c_int, [C.c_void_p]),
    "fvs_batch_set_state": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p]),
    "fvs_batch_get_state": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p]),
    "fvs_batch_autotune": (C.c_int, [C.c_void_p, C.c_int32, C.POINTER(C.c_float)]),
    "fvs_batch_set_launch": (C.c_int, [C.c_void_p, C.c_int32, C.c_int32, C.c_int32]),
    "fvs_batch_set_precision": (C.c_int, [C.c_void_p, C.c_int32]),
    "fvs_batch_set_barrier_budget": (C.c_int, [C.c_void_p, C.c_double]),
    "fvs_batch_steps": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.POINTER(C.c_float)]),
    "fvs_batch_run_to_drop": (C.c_int, [C.c_void_p, C.c_int32, C.c_double, C.c_int32, C.c_void_p, C.c_void_p,
                                        C.c_void_p, C.POINTER(C.c_float)]),
    "fvs_batch_set_mode": (C.c_int, [C.c_void_p, C.c_int32]),
    "fvs_batch_set_groups": (C.c_int, [C.c_void_p, C.c_void_p]),
    "fvs_batch_run_to_level": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p,
                                         C.c_void_p, C.POINTER(C.c_float)]),
    "fvs_batch_run_to_level_dc": (C.c_int, [C.c_void_p, C.c_int32, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p,
                                         C.c_void_p, C.POINTER(C.c_float)]),
    "fvs_mlp_create": (C.c_int, [C.c_int32, C.c_int32, C.c_int32, C.c_int32, C.c_uint64, C.POINTER(C.c_void_p)]),
    "fvs_mlp_destroy": (None, [C.c_void_p]),
    "fvs_mlp_set_engine": (C.c_int, [C.c_void_p, C.c_int32]),
    "fvs_mlp_last_error": (C.c_char_p, [C.c_void_p]),
    "fvs_mlp_num_params": (C.c_int, [C.c_void_p, C.POINTER(C.c_int64)]),
    "fvs_mlp_get_params": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64]),
    "fvs_mlp_set_params": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64]),
    "fvs_mlp_loss_grad": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int32, C.POINTER(C.c_float), C.c_void_p]),
    "fvs_mlp_train": (C.c_int, [C.c_void_p, C.c_void_p, C.c_void_p, C.c_int64, C.c_int32, C.c_int32, C.c_float,
                                C.c_uint64, C.c_void_p]),
    "fvs_mlp_predict": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int64, C.c_void_p]),
    "fvs_rms_delta_noalloc": (C.c_int, [C.c_void_p, C.c_void_p, C.c_int32, C.c_void_p, C.c_void_p]),
}

_LIB = None


def library_path() -> str:
    return os.path.join(os.path.dirname(os.path.abspath(__file__)), "libfvs2d_gb300.so")


def load(build_if_missing: bool = True) -> C.CDLL:
    """Load libfvs2d_gb300.so (building it in-tree if it is missing).

    There is no fallback: without the CUDA library nothing in this package
    runs."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = library_path()
    if not os.path.exists(path):
        if not build_if_missing:
            raise RuntimeError(f"{path} is missing: run fvs2d_gb300._build.build()")
        from . import _build
        _build.build()
    lib = C.CDLL(path)
    for name, (res, args) in SIGNATURES.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    _LIB = lib
    return lib


def ptr(a: np.ndarray) -> C.c_void_p:
    return C.c_void_p(a.ctypes.data)


class MeshArrays:
    """Keeps the numpy arrays behind an FvsMesh alive."""

    def __init__(self, mesh):
        from .meshgen import BC_CODES
        self.node_xy = np.ascontiguousarray(mesh.node_xy, np.float64)
        self.tri = np.ascontiguousarray(mesh.tri_nodes, np.int32).reshape(-1, 3)
        self.quad = np.ascontiguousarray(mesh.quad_nodes, np.int32).reshape(-1, 4)
        self.bn = np.array([len(c) for c in mesh.bndry_cells], np.int32)
        self.bt = np.array([BC_CODES[t] if isinstance(t, str) else int(t) for t in mesh.bndry_types], np.int32)
        cells = [np.asarray(c, np.int32) for c in mesh.bndry_cells]
        self.bc = np.ascontiguousarray(np.concatenate(cells) if cells else np.zeros(1, np.int32), np.int32)
        if self.bn.size == 0:
            self.bn = np.zeros(1, np.int32)
            self.bt = np.zeros(1, np.int32)
        self.struct = FvsMesh(
            self.node_xy.shape[0], self.tri.shape[0], self.quad.shape[0],
            self.node_xy.ctypes.data_as(_dp), self.tri.ctypes.data_as(_ip),
            self.quad.ctypes.data_as(_ip) if self.quad.shape[0] else C.cast(None, _ip),
            len(mesh.bndry_cells), self.bn.ctypes.data_as(_ip), self.bt.ctypes.data_as(_ip),
            self.bc.ctypes.data_as(_ip), float(mesh.period_x), float(mesh.period_y))
