"""Checkpoint / restart through the reference's IOS files on the GPU path:
a run interrupted by save -> cont files -> restart (ntstart > 1) continues
bit-identically to the uninterrupted run (strict FP64, steady local time
stepping)."""
from __future__ import annotations

import os
import shutil

import numpy as np
import pytest

from cases import airfoil

pytestmark = pytest.mark.gpu


def test_restart_continues_bit_identically(tmp_path):
    from fvs2d_gb300 import PREC_FP64_STRICT, FvsError, Solver
    mesh, o = airfoil(nw=64, nr=20, precision=PREC_FP64_STRICT)
    with Solver(mesh, o) as s:
        s.initialize_solution()
        n_all = s.time_integration(0.0, 6)
        u_all = s.cvar
    with Solver(mesh, o) as s:
        s.initialize_solution()
        n_a = s.time_integration(0.0, 3)
        s.write_save(str(tmp_path), ntimes=3)
    for ext in (".cd", ".s8"):
        shutil.copy(os.path.join(tmp_path, "save" + ext), os.path.join(tmp_path, "cont" + ext))
    o2 = o.replace(ntstart=4)
    with Solver(mesh, o2) as s:
        s.initialize_solution(str(tmp_path))
        n_b = s.time_integration(0.0, 3)
        u_b = s.cvar
        # the C-ABI's own initialize_solution refuses a restart start
        with pytest.raises(FvsError):
            s._check(s._lib.fvs_init_state(s._h))
    assert np.array_equal(u_all, u_b)
    assert np.array_equal(n_all[:3], n_a) and np.array_equal(n_all[3:], n_b)
