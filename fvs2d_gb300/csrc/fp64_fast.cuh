// fp64_fast.cuh — FP64 reciprocal and reciprocal square root for the FP64
// (non-strict) kernels, built from the hardware's approximations.
//
// GB300 executes 2 FP64 operations per clock per SM, and the FP64 Roe flux
// is bound by that pipe.  A reciprocal or square root rounded as IEEE
// division and sqrt require costs several FP64 operations plus special-case
// handling; the flux needs three reciprocals and two square roots per edge.
// Here each starts from PTX's approximate instructions (rcp.approx.ftz.f64,
// rsqrt.approx.ftz.f64: issued on the special-function unit, not on the FP64
// pipe) and is refined by ONE Newton-Raphson step carried to second order
// in the residual (cubic convergence; the series form of the iteration, e.g.
// P. Markstein, "IA-64 and Elementary Functions", 2000, ch. 8-9):
//
//   1/x:      e = 1 - x y0            y = y0 + y0 (e + e^2)
//   1/sqrt x: u = 1 - x y0^2          y = y0 + y0 u (1/2 + 3/8 u)
//
// If y0 has relative error d, the result has relative error ~d^3 (rcp) and
// ~(5/16)(2d)^3 (rsqrt) before the final roundings: below 2^-60 for any
// d <= 2^-20, so the results are within a few units in the last place of the
// correctly rounded ones (tests/test_gpu_fast_math.py measures the maximum
// over many arguments through fvs_check_fp64_math).  Three FP64 operations
// for 1/x, five for 1/sqrt x.
//
// Domain: positive normal numbers (densities, pressures, squared sound
// speeds of physical states).  Zero, negative, infinite and NaN arguments
// give NaN or infinity, which the residual-norm checks report as
// FVS_ERR_NONFINITE; subnormal arguments are flushed to zero.
#pragma once

namespace fvs {

__device__ __forceinline__ double rcp_nr(double x) {
  double y;
  asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
  const double e = fma(-x, y, 1.0);
  return fma(fma(e, e, e), y, y);
}

__device__ __forceinline__ double rsqrt_nr(double x) {
  double y;
  asm("rsqrt.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(x));
  const double u = fma(-x * y, y, 1.0);
  return fma(y * u, fma(0.375, u, 0.5), y);
}

// sqrt(x) = x / sqrt(x): one product after the reciprocal square root
__device__ __forceinline__ double sqrt_nr(double x) { return x * rsqrt_nr(x); }

}  // namespace fvs
