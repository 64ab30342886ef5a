"""The index-checking kernels (FVS2D_BOUNDS=1 handles, the FVS_BOUNDS build):
every indirect index checked against its array, the first violation
recorded in a device word and reported as FVS_ERR_BOUNDS; nothing traps or
faults.

On valid meshes the checked kernels give results bit-identical to the FP64
handle's (same arithmetic).  A gather entry set out of range through
fvs_debug_set_gather (refused on other handles) is caught by the kernel's
own check, which substitutes a valid index, and reported with its site."""
import numpy as np
import pytest

import cases
from fvs2d_gb300 import PREC_FP64, FvsError, Solver, capi

pytestmark = pytest.mark.gpu


def states(mesh, opt, bounds, monkeypatch, steps=4):
    if bounds:
        monkeypatch.setenv("FVS2D_BOUNDS", "1")
    else:
        monkeypatch.delenv("FVS2D_BOUNDS", raising=False)
    with Solver(mesh, opt.replace(precision=PREC_FP64)) as s:
        s.initialize_solution()
        n = s.time_integration(0.0, steps)
        r, w = s.compute_residual(0.0 if opt.steady else steps * s.current_dt())
        return n, s.cvar, r, w


@pytest.mark.parametrize("make", [lambda: cases.periodic_vortex(24, jitter=0.2),
                                  lambda: cases.airfoil(64, 24, cfl=0.5),
                                  lambda: cases.periodic_vortex(24, jitter=0.2, grad_method=2)])
def test_checked_kernels_bit_identical_on_valid_meshes(make, monkeypatch):
    mesh, opt = make()
    a = states(mesh, opt, True, monkeypatch)
    b = states(mesh, opt, False, monkeypatch)
    for x, y in zip(a, b):
        assert np.array_equal(x, y)


def test_out_of_range_gather_slot_reported(monkeypatch):
    mesh, opt = cases.periodic_vortex(16, jitter=0.2)
    monkeypatch.delenv("FVS2D_BOUNDS", raising=False)
    with Solver(mesh, opt) as s:
        # refused on a handle whose kernels do not check
        assert s._lib.fvs_debug_set_gather(s._h, 1, 0, 10 ** 6) == capi.FVS_ERR_INVALID
    monkeypatch.setenv("FVS2D_BOUNDS", "1")
    with Solver(mesh, opt) as s:
        s.initialize_solution()
        s.time_integration(0.0, 1)
        nedge = s.sizes.nedges
        assert s._lib.fvs_debug_set_gather(s._h, 5, 1, nedge + 7) == capi.FVS_OK
        with pytest.raises(FvsError) as e:
            s.time_integration(0.0, 1)
        assert e.value.code == capi.FVS_ERR_BOUNDS
        assert "gather slot" in str(e.value) and str(nedge + 6) in str(e.value)
