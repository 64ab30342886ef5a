"""fvs_rms_delta_noalloc: the allocation-free residual norm.

For callers that cannot allocate device memory where they need the per-step
residual norm (their device memory is reserved up front by another
allocator, or their loop must not pay cudaMalloc's implicit synchronisation):
the entry point takes caller-owned device arrays and keeps its partial sums
in a fixed device array of the library.  This test checks it, through the
C-ABI, against the norm the existing fvs_time_integration entry point logs
for the same step, on two calls in a row (the second call reuses the fixed
array the first one left filled).  The file is named to be collected last.
"""
import ctypes as C

import numpy as np
import pytest

import cases
from fvs2d_gb300 import PREC_FP64, Solver, capi

pytestmark = pytest.mark.gpu


def test_noalloc_norm_matches_time_integration_log():
    torch = pytest.importorskip("torch")
    lib = capi.load()
    mesh, opt = cases.periodic_vortex(64, jitter=0.2)  # 8,192 cells
    with Solver(mesh, opt.replace(precision=PREC_FP64)) as s:
        s.initialize_solution()
        n = s.ncells
        out = torch.zeros(4, dtype=torch.float64, device="cuda")
        for call in range(2):
            u0 = s.cvar
            ref = s.time_integration(0.0, 1)[0]  # existing entry point: RMS(|U-U0|) of this step
            u1 = s.cvar
            du0 = torch.from_numpy(u0).to("cuda")
            du1 = torch.from_numpy(u1).to("cuda")
            out.fill_(-1.0)
            torch.cuda.synchronize()
            rc = lib.fvs_rms_delta_noalloc(C.c_void_p(du1.data_ptr()), C.c_void_p(du0.data_ptr()), n,
                                           C.c_void_p(out.data_ptr()), None)
            assert rc == capi.FVS_OK, f"call {call}: rc {rc}"
            torch.cuda.synchronize()
            got = out.cpu().numpy()
            # same tolerance as the other norm checks (blocked reductions in a
            # different cell order)
            assert np.allclose(got, ref, rtol=1e-13, atol=0), (call, got, ref)
        # a prefix that ends inside a block of 256 cells (the partial last
        # block), on a stream other than the default one, against numpy
        m = n - 37
        side = torch.cuda.Stream()
        with torch.cuda.stream(side):
            out.fill_(-1.0)
            rc = lib.fvs_rms_delta_noalloc(C.c_void_p(du1.data_ptr()), C.c_void_p(du0.data_ptr()), m,
                                           C.c_void_p(out.data_ptr()), C.c_void_p(side.cuda_stream))
            assert rc == capi.FVS_OK, f"prefix call: rc {rc}"
        side.synchronize()
        got = out.cpu().numpy()
        ref = np.sqrt(np.mean((u1[:m] - u0[:m]) ** 2, axis=0))
        assert np.allclose(got, ref, rtol=1e-13, atol=0), (got, ref)
        # exactly the accepted maximum (every block of the fixed array in use)
        cap = 2_097_152
        g = torch.Generator(device="cuda").manual_seed(3)
        a = torch.rand((cap, 4), dtype=torch.float64, device="cuda", generator=g)
        b = torch.rand((cap, 4), dtype=torch.float64, device="cuda", generator=g)
        out.fill_(-1.0)
        torch.cuda.synchronize()
        assert lib.fvs_rms_delta_noalloc(C.c_void_p(a.data_ptr()), C.c_void_p(b.data_ptr()), cap,
                                         C.c_void_p(out.data_ptr()), None) == capi.FVS_OK
        torch.cuda.synchronize()
        ref = np.sqrt(np.mean((a.cpu().numpy() - b.cpu().numpy()) ** 2, axis=0))
        assert np.allclose(out.cpu().numpy(), ref, rtol=1e-13, atol=0)
        del a, b
        # beyond the fixed scratch: rejected before any device work
        big = 2_097_152 + 1
        assert lib.fvs_rms_delta_noalloc(C.c_void_p(du1.data_ptr()), C.c_void_p(du0.data_ptr()), big,
                                         C.c_void_p(out.data_ptr()), None) == capi.FVS_ERR_INVALID
