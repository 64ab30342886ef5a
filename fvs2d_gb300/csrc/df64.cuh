// df64.cuh — FP64-accuracy arithmetic on the FP32 pipe ("double-float").
//
// A value is the unevaluated sum hi + lo of two FP32 numbers with
// |lo| <= ulp(hi)/2: 48 significant bits, relative precision u^2 = 2^-48
// (3.6e-15) against FP64's 2^-53.  GB300 executes 2 FP64 FMA per clock per SM
// but 128 FP32 FMA, so a df64 operation of 3-20 FP32 instructions is still
// several times cheaper than one FP64 instruction.
//
// Building blocks (published algorithms, written here from the mathematics):
//  - TwoSum (Knuth, TAOCP vol. 2, 4.2.2) and Fast2Sum (Dekker 1971): the
//    exact rounding error of a sum;
//  - TwoProd by FMA: the exact rounding error of a product;
//  - the double-word algorithms of Joldes, Muller and Popescu, "Tight and
//    rigorous error bounds for basic building blocks of double-word
//    arithmetic", ACM TOMS 44(2), 2017: accurate DW+DW (their Algorithm 6,
//    relative error <= 3u^2), DW x DW with FMA (Algorithm 12, <= 5u^2),
//    DW x FP (Algorithm 9) and DW / DW (Algorithm 17, <= 15u^2);
//  - square root: the FP32 root refined by one Newton step on the residual
//    x - s*s computed exactly with TwoProd;
//  - two cheaper forms for the Roe flux and the stage arithmetic, whose error
//    is bounded by ~2^-47 of the operands' magnitude rather than of the
//    result's: the sloppy DW+DW sum (Dekker 1971), ~11 instructions against
//    ~20, and a fused a*b + c that adds c to the exact product of the high
//    parts (TwoProd, then TwoSum with c's high part) and collects the cross
//    terms and both low parts in one FP32 sum, ~12 instructions against ~29
//    for a product and an accurate sum.
// Comparisons order by hi, then lo.  Conversions from FP64 split the
// significand on the integer pipe (no FP64 instruction); conversion back to
// FP64 is one exact FP64 addition.
#pragma once

#include <cuda_runtime.h>

namespace fvs {

struct df64 {
  float hi, lo;
  df64() = default;
  __host__ __device__ constexpr df64(float h, float l) : hi(h), lo(l) {}
  __host__ __device__ constexpr df64(int x) : hi(float(x)), lo(0.0f) {}
  // compile-time constants and host values: round to nearest FP32, then the
  // remainder (exact in FP64)
  __host__ __device__ constexpr df64(double x) : hi(float(x)), lo(float(x - double(float(x)))) {}
  __host__ __device__ explicit operator double() const { return double(hi) + double(lo); }
};

__host__ __device__ __forceinline__ df64 fast_two_sum(float a, float b) {
  const float s = a + b;
  return df64(s, b - (s - a));
}
__host__ __device__ __forceinline__ df64 two_sum(float a, float b) {
  const float s = a + b;
  const float bp = s - a;
  return df64(s, (a - (s - bp)) + (b - bp));
}
__device__ __forceinline__ df64 two_prod(float a, float b) {
  const float p = a * b;
  return df64(p, __fmaf_rn(a, b, -p));
}

__device__ __forceinline__ df64 operator+(df64 x, df64 y) {
  const df64 s = two_sum(x.hi, y.hi);
  const df64 t = two_sum(x.lo, y.lo);
  const df64 v = fast_two_sum(s.hi, s.lo + t.hi);
  return fast_two_sum(v.hi, t.lo + v.lo);
}
__device__ __forceinline__ df64 operator-(df64 x) { return df64(-x.hi, -x.lo); }
__device__ __forceinline__ df64 operator-(df64 x, df64 y) { return x + (-y); }
__device__ __forceinline__ df64 operator*(df64 x, df64 y) {
  const df64 c = two_prod(x.hi, y.hi);
  const float t = __fmaf_rn(x.hi, y.lo, x.lo * y.lo);
  const float cl = c.lo + __fmaf_rn(x.lo, y.hi, t);
  return fast_two_sum(c.hi, cl);
}
__device__ __forceinline__ df64 mul_fp(df64 x, float y) {
  const df64 c = two_prod(x.hi, y);
  return fast_two_sum(c.hi, __fmaf_rn(x.lo, y, c.lo));
}
__device__ __forceinline__ df64 operator/(df64 x, df64 y) {
  const float th = __fdiv_rn(x.hi, y.hi);
  const df64 r = mul_fp(y, th);
  const float ph = x.hi - r.hi;  // exact (Sterbenz)
  const float dl = x.lo - r.lo;
  const float d = ph + dl;
  return fast_two_sum(th, __fdiv_rn(d, y.hi));
}
__device__ __forceinline__ df64 dsqrt_(df64 x) {
  if (!(x.hi > 0.0f)) return df64(sqrtf(x.hi), 0.0f);
  const float s = __fsqrt_rn(x.hi);
  const df64 p = two_prod(s, s);
  const float r = ((x.hi - p.hi) - p.lo) + x.lo;
  return fast_two_sum(s, __fdiv_rn(r, 2.0f * s));
}
// a + b, sloppy: one TwoSum of the high parts, the low parts added to its
// error, renormalised
__device__ __forceinline__ df64 dadd_s(df64 a, df64 b) {
  const df64 s = two_sum(a.hi, b.hi);
  return fast_two_sum(s.hi, s.lo + (a.lo + b.lo));
}
// a * b + c: TwoProd of the high parts, TwoSum with c's high part, the
// cross terms and both low parts in one FP32 sum, renormalised
__device__ __forceinline__ df64 dfma(df64 a, df64 b, df64 c) {
  const df64 p = two_prod(a.hi, b.hi);
  const float cross = __fmaf_rn(a.hi, b.lo, a.lo * b.hi);
  const df64 s = two_sum(p.hi, c.hi);
  return fast_two_sum(s.hi, s.lo + ((p.lo + cross) + c.lo));
}
__device__ __forceinline__ df64 dabs_(df64 x) { return x.hi < 0.0f ? -x : x; }
__device__ __forceinline__ df64 half(df64 x) { return df64(0.5f * x.hi, 0.5f * x.lo); }
__device__ __forceinline__ bool operator<(df64 a, df64 b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
__device__ __forceinline__ bool operator>(df64 a, df64 b) { return b < a; }

// FP64 -> df64 on the integer pipe: hi keeps the top 24 bits of the
// significand (truncated, exact), lo the remaining 29 bits scaled by
// 2^(e-1075) (exact integer -> float conversion, rounded); one Fast2Sum
// renormalises.  |x| outside ~[2^-74, 2^127] loses lo (zeros, Inf, NaN pass).
__device__ __forceinline__ df64 df_from_double(double x) {
  const unsigned int hi = (unsigned int)__double2hiint(x), lo = (unsigned int)__double2loint(x);
  const unsigned int sign = hi & 0x80000000u;
  const int e = (int)((hi >> 20) & 0x7ffu);
  const int fe = e - 896;  // FP32 biased exponent of x
  if (e == 0x7ff || fe <= 0 || fe >= 255) return df64(float(x), 0.0f);
  const unsigned int mant23 = ((hi & 0xfffffu) << 3) | (lo >> 29);
  const float h = __uint_as_float(sign | ((unsigned int)fe << 23) | mant23);
  const unsigned int rest = lo & 0x1fffffffu;  // 29 bits below h's last bit
  const int se = e - 1075 + 127;                // biased exponent of 2^(e-1075)
  if (rest == 0u || se <= 0) return df64(h, 0.0f);
  float l = __uint2float_rn(rest) * __uint_as_float((unsigned int)se << 23);
  if (sign) l = -l;
  return fast_two_sum(h, l);
}

}  // namespace fvs
