"""The FP64 kernels' reciprocal and square root (fp64_fast.cuh: the
hardware approximations refined by one Newton-Raphson step of cubic order)
against CUDA's IEEE-rounded 1/x and sqrt(x), through fvs_check_fp64_math.

Arguments: seeded log-uniform values over [1e-30, 1e30] plus the range the
Roe flux sees (densities, 1 + sqrt(density ratio), squared sound speeds,
0.01-100) and powers of two with their neighbours.  Bar: at most 2 units in
the last place from the correctly rounded result (relative 2^-52)."""
import numpy as np
import pytest

from fvs2d_gb300 import capi

pytestmark = pytest.mark.gpu


def ulps(a, b):
    """|a - b| in units in the last place of b."""
    return np.abs(a - b) / np.spacing(np.abs(b))


def test_fp64_reciprocal_and_sqrt_within_2_ulp():
    lib = capi.load()
    rng = np.random.default_rng(11)
    x = np.concatenate([10.0 ** rng.uniform(-30, 30, 200_000), rng.uniform(0.01, 100.0, 200_000),
                        np.ldexp(1.0, np.arange(-60, 61)), np.nextafter(np.ldexp(1.0, np.arange(-60, 61)), 0),
                        np.nextafter(np.ldexp(1.0, np.arange(-60, 61)), np.inf)]).astype(np.float64)
    out = np.empty((x.size, 5))
    assert lib.fvs_check_fp64_math(capi.ptr(x), x.size, capi.ptr(out)) == capi.FVS_OK
    rcp, rcp_ieee, rsq, sq, sq_ieee = out.T
    assert np.array_equal(rcp_ieee, 1.0 / x)  # the device's IEEE results equal numpy's
    assert np.array_equal(sq_ieee, np.sqrt(x))
    assert ulps(rcp, rcp_ieee).max() <= 2.0
    assert ulps(sq, sq_ieee).max() <= 2.0
    exact_rsq = (1.0 / np.sqrt(x.astype(np.longdouble))).astype(np.float64)
    assert ulps(rsq, exact_rsq).max() <= 2.0
