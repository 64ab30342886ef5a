"""fvs2d_gb300 — GB300-native residual-and-update loop of the fvs2d solver.

The arithmetic runs in hand-written sm_103a kernels behind the C-ABI of
include/fvs2d.h (libfvs2d_gb300.so, built in-tree).  This package is the
host-side mirror of the reference's module API (:mod:`.solver`), its input
options (:mod:`.options`) and the synthetic meshes of the benchmark cases
(:mod:`.meshgen`).  There is no CPU fallback: a missing library raises.
"""
from . import capi, meshgen
from .capi import PREC_FP64, PREC_FP64_DF, PREC_FP64_STRICT, PREC_MIXED
from .meshgen import Mesh
from .options import Options, read_input
from .solver import FvsError, Solver

__all__ = ["capi", "meshgen", "Mesh", "Options", "read_input", "Solver", "FvsError", "PREC_FP64", "PREC_FP64_DF", "PREC_FP64_STRICT",
           "PREC_MIXED"]
