"""RMS(dU) norms of the last stage's reduction against the states themselves.

The last RK stage's update runs as one wave of resident blocks that stride
over the cells, and sums |U - U0|^2 per block (FP32 pairs in the mixed and
double-float builds, FP64 otherwise) before the last block sums the
partials (src/runge_kutta.f90:395-410 defines the norm).  On a mesh larger
than one wave (411,426 cells, not a multiple of the block size) the norm of
one step must equal sqrt(mean((U1 - U0)^2)) of the downloaded states: every
cell counted once.  The states are FP64 in every mode; the mixed increment is
an FP32 number added to the FP64 state, so its norm agrees to the FP32
rounding of the squares."""
import math

import numpy as np
import pytest

import cases
from fvs2d_gb300 import PREC_FP64, PREC_FP64_DF, PREC_FP64_STRICT, PREC_MIXED, Solver, meshgen

pytestmark = pytest.mark.gpu

TOL = {PREC_FP64_STRICT: 1e-13, PREC_FP64: 1e-13, PREC_FP64_DF: 1e-12, PREC_MIXED: 1e-6}


@pytest.mark.parametrize("prec", [PREC_FP64_STRICT, PREC_FP64, PREC_FP64_DF, PREC_MIXED])
def test_one_wave_norm_counts_every_cell_once(prec):
    mesh = meshgen.periodic_square(513, 401, jitter=0.2)
    _, opt = cases.periodic_vortex(4)
    with Solver(mesh, opt.replace(precision=prec)) as s:
        assert s.ncells == 2 * 513 * 401 and s.ncells % 256 != 0
        s.initialize_solution()
        u0 = s.cvar
        norms = s.time_integration(0.0, 2)
        u2 = s.cvar
        s.cvar = u0
        s.time_integration(0.0, 1)
        u1 = s.cvar
    # exactly rounded sums (numpy's sum along the long axis is sequential,
    # ~1e-13 relative at this size)
    def rms(a, b):
        d2 = (a - b) ** 2
        return np.array([math.sqrt(math.fsum(d2[:, k]) / d2.shape[0]) for k in range(4)])

    ref1, ref2 = rms(u1, u0), rms(u2, u1)
    assert np.all(ref1 > 0) and np.all(ref2 > 0)
    assert np.allclose(norms[0], ref1, rtol=TOL[prec], atol=0), (norms[0], ref1)
    assert np.allclose(norms[1], ref2, rtol=TOL[prec], atol=0), (norms[1], ref2)
