"""Benchmark config 1: the 8,192-cell periodic vortex (64x64 quads, seeded
diagonals), LSQ-fn, SSP-RK3, CFL 0.8, 200 steps, against the CPU oracle over
the whole run: strict FP64 bit-identical, FP64 and double-float within
1e-11, mixed within 1e-5 of max|U|; all four with the same error against the
exact vortex to within their own tolerance."""
import numpy as np
import pytest

import cases
from fvs2d_gb300 import PREC_FP64, PREC_FP64_DF, PREC_FP64_STRICT, PREC_MIXED, Solver, meshgen
from oracle_lib import Oracle

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.abs(a - b).max() / np.abs(b).max())


@pytest.mark.parametrize("grad", [3, 1, 2])
def test_config1_200_steps(grad):
    mesh = meshgen.periodic_square(64, 64, seed=1)
    _, opt = cases.periodic_vortex(4, grad_method=grad)
    assert mesh.ncells == 8192
    orc = Oracle(mesh, opt)
    orc.initialize_solution()
    orc.time_integration(0.0, 200)
    u_ref = orc.cvar
    t_end = 200 * orc.dt
    e_ref = orc.error_isentropic_vortex(t_end)
    for prec, tol in ((PREC_FP64_STRICT, 0.0), (PREC_FP64, 1e-11), (PREC_FP64_DF, 1e-11), (PREC_MIXED, 1e-5)):
        with Solver(mesh, opt.replace(precision=prec)) as s:
            s.initialize_solution()
            s.time_integration(0.0, 200)
            u = s.cvar
            e = s.error_isentropic_vortex(t_end)
        if tol == 0.0:
            assert np.array_equal(u, u_ref)
        else:
            assert rel(u, u_ref) <= tol, (prec, rel(u, u_ref))
        # the vortex error itself agrees to the same relative level
        assert abs(e[12] - e_ref[12]) <= max(tol, 1e-14) * 10 * abs(e_ref[12]) + tol, (prec, e[12], e_ref[12])
