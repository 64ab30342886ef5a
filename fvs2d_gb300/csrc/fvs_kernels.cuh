// fvs_kernels.cuh — device code of the residual-and-update loop.
//
// Included by three translation units that differ only in arithmetic:
//   fvs_kern_strict.cu  FP64, -fmad=false: every product and sum rounded as
//                       the reference writes it (bit-identical to the oracle)
//   fvs_kern_fast.cu    FP64, -fmad=true (FMA contraction allowed)
//   fvs_kern_mixed.cu   T = float for gradient, limiter, reconstruction and
//                       flux; FP64 residual accumulation, update and norms
//   fvs_kern_df.cu      T = df64 (FP64 accuracy from FP32 pairs, df64.cuh)
//                       for gradient, limiter, reconstruction, flux and the
//                       slot gather; FP64 state update and norms
// FVS_NS names the namespace, FVS_T the compute type.
//
// One RK stage is three launches, all coalesced one-thread-per-item gathers:
//   k_gradient  cell-parallel: gradient of the primitives (LSQ / GG-cell /
//               GG-node) fused with the limiter (src/gradient_*.f90,
//               src/gradient_limiter.f90)
//   k_flux      edge-parallel: MUSCL reconstruction + Roe flux on interior
//               edges, ghost state + Roe on boundary edges; writes flux*area
//               and ws*area per edge slot (src/residual.f90:66-157,
//               src/flux_invscid.f90:37-136)
//   k_update    cell-parallel: sums the cell's edge slots in the reference's
//               summation order (deterministic, no atomics), -R/vol, local
//               time step, RK stage update, primitives for the next stage and
//               per-block partial norms (src/runge_kutta.f90)
#pragma once

#include <cuda_runtime.h>

#include <cstdlib>

#include "df64.cuh"
#include "fp64_fast.cuh"
#include "fvs_internal.hpp"

#ifndef FVS_DF
#define FVS_DF 0
#endif
// the FP64 build with multiply-add contraction (FVS_PREC_FP64)
#define FVS_FP64_FAST (!FVS_STRICT && !FVS_MIXED && !FVS_DF)
// the index-checking build (FVS2D_BOUNDS=1 handles): FP64 arithmetic with
// every indirect index checked
#ifndef FVS_BOUNDS
#define FVS_BOUNDS 0
#endif

namespace fvs {
namespace FVS_NS {

using T = FVS_T;
struct T2 { T x, y; };

// Index check of the index-checking build: i must lie in [lo, hi).  On a
// violation the first one is recorded in d.bounds_err (flag, site, index,
// extent) and index 0 (a valid cell and edge slot) is used instead, so the
// kernel carries on without touching memory outside the array.  Other builds
// return i unchecked.
enum : int { SITE_STENCIL = 1, SITE_EDGE_L = 2, SITE_EDGE_R = 3, SITE_GATHER = 4 };
__device__ __forceinline__ int chk_idx(int* err, int i, int lo, int hi, int site) {
#if FVS_BOUNDS
  if (i < lo || i >= hi) {
    if (atomicCAS(err, 0, 1) == 0) {
      err[1] = site;
      err[2] = i;
      err[3] = hi;
    }
    return 0;
  }
#else
  (void)err; (void)lo; (void)hi; (void)site;
#endif
  return i;
}

// Programmatic dependent launch.  The single-mesh step kernels are launched
// with the programmatic stream serialization attribute (launch_k below), so
// a kernel's blocks may be scheduled while its predecessor in the stream
// finishes.  pdl_wait() blocks until the predecessor grid has completed and
// its memory writes are visible; every kernel calls it before its first
// global memory access, so results are unchanged.  pdl_trigger() right after
// lets this grid's successor be launched once every block of this grid has
// started.  Launched without the attribute, both return at once.
__device__ __forceinline__ void pdl_wait() { asm volatile("griddepcontrol.wait;" ::: "memory"); }
__device__ __forceinline__ void pdl_trigger() { asm volatile("griddepcontrol.launch_dependents;" ::: "memory"); }

// programmatic dependent launch of the single-mesh step kernels (see
// pdl_wait); FVS2D_PDL=0 in the environment launches them plainly
static bool pdl_enabled() {
  static const bool on = [] {
    const char* e = std::getenv("FVS2D_PDL");
    return !(e && e[0] == '0' && e[1] == 0);
  }();
  return on;
}

template <typename... KArgs, typename... Args>
static void launch_k(void (*kern)(KArgs...), unsigned grid, unsigned block, size_t smem, cudaStream_t s,
                     Args... args) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3(grid);
  cfg.blockDim = dim3(block);
  cfg.dynamicSmemBytes = smem;
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
  attr[0].val.programmaticStreamSerializationAllowed = pdl_enabled() ? 1 : 0;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  cudaLaunchKernelEx(&cfg, kern, args...);
}

__device__ __forceinline__ void ld4(const double* __restrict__ p, int i, double* o) {
  const double2* q = reinterpret_cast<const double2*>(p) + 2 * (size_t)i;
  double2 a = q[0], b = q[1];
  o[0] = a.x; o[1] = a.y; o[2] = b.x; o[3] = b.y;
}
__device__ __forceinline__ void st4(double* __restrict__ p, int i, const double* v) {
  double2* q = reinterpret_cast<double2*>(p) + 2 * (size_t)i;
  q[0] = make_double2(v[0], v[1]);
  q[1] = make_double2(v[2], v[3]);
}
__device__ __forceinline__ void ld4(const float* __restrict__ p, int i, float* o) {
  float4 a = reinterpret_cast<const float4*>(p)[i];
  o[0] = a.x; o[1] = a.y; o[2] = a.z; o[3] = a.w;
}
__device__ __forceinline__ void st4(float* __restrict__ p, int i, const float* v) {
  reinterpret_cast<float4*>(p)[i] = make_float4(v[0], v[1], v[2], v[3]);
}
__device__ __forceinline__ void ld4(const df64* __restrict__ p, int i, df64* o) {
  const float4* q = reinterpret_cast<const float4*>(p) + 2 * (size_t)i;
  const float4 a = q[0], b = q[1];
  o[0] = df64(a.x, a.y); o[1] = df64(a.z, a.w); o[2] = df64(b.x, b.y); o[3] = df64(b.z, b.w);
}
__device__ __forceinline__ void st4(df64* __restrict__ p, int i, const df64* v) {
  float4* q = reinterpret_cast<float4*>(p) + 2 * (size_t)i;
  q[0] = make_float4(v[0].hi, v[0].lo, v[1].hi, v[1].lo);
  q[1] = make_float4(v[2].hi, v[2].lo, v[3].hi, v[3].lo);
}
__device__ __forceinline__ T2 ld2(const void* p, int i) {
  return reinterpret_cast<const T2*>(p)[i];
}

// Loads of arrays that another block wrote earlier in the same launch (the
// persistent kernel): COH selects ld.global.cg, which reads through L2 and
// never returns a stale L1 line or a non-coherent read-only-path value.
template <bool COH>
__device__ __forceinline__ void ldc4(const double* p, int i, double* o) {
  const double2* q = reinterpret_cast<const double2*>(p) + 2 * (size_t)i;
  double2 a, b;
  if (COH) { a = __ldcg(q); b = __ldcg(q + 1); }
  else { a = q[0]; b = q[1]; }
  o[0] = a.x; o[1] = a.y; o[2] = b.x; o[3] = b.y;
}
template <bool COH>
__device__ __forceinline__ void ldc4(const float* p, int i, float* o) {
  const float4* q = reinterpret_cast<const float4*>(p) + i;
  const float4 a = COH ? __ldcg(q) : *q;
  o[0] = a.x; o[1] = a.y; o[2] = a.z; o[3] = a.w;
}
template <bool COH>
__device__ __forceinline__ void ldc4(const df64* p, int i, df64* o) {
  const float4* q = reinterpret_cast<const float4*>(p) + 2 * (size_t)i;
  float4 a, b;
  if (COH) { a = __ldcg(q); b = __ldcg(q + 1); }
  else { a = q[0]; b = q[1]; }
  o[0] = df64(a.x, a.y); o[1] = df64(a.z, a.w); o[2] = df64(b.x, b.y); o[3] = df64(b.z, b.w);
}
template <bool COH, typename V>
__device__ __forceinline__ V ldc1(const V* p, int i) {
  return COH ? __ldcg(p + i) : p[i];
}
template <bool COH>
__device__ __forceinline__ df64 ldc1(const df64* p, int i) {
  const float2 a = COH ? __ldcg(reinterpret_cast<const float2*>(p) + i) : reinterpret_cast<const float2*>(p)[i];
  return df64(a.x, a.y);
}

// scheme constants in the compute type, rounded once on the host
#if FVS_MIXED
#define TP(name) (d.f##name)
#elif FVS_DF
#define TP(name) (df64(d.d##name[0], d.d##name[1]))
#else
#define TP(name) (d.name)
#endif

// Exact FP32 -> FP64 conversion on the integer pipe (the FP64 pipe, 2 ops per
// clock per SM on GB300, is the scarce resource of the update kernel).
// FP32 subnormals (|x| < 1.2e-38) become signed zero; Inf/NaN are kept.
__device__ __forceinline__ double f2d_bits(float f) {
  const unsigned int b = __float_as_uint(f);
  const unsigned int e = (b >> 23) & 0xffu;
  const unsigned int sign = b & 0x80000000u;
  const unsigned int de = e == 0u ? 0u : (e == 0xffu ? 0x7ffu : e + 896u);
  const unsigned int m = e == 0u ? 0u : (b & 0x7fffffu);
  const unsigned int hi = sign | (de << 20) | (m >> 3);
  const unsigned int lo = m << 29;
  return __hiloint2double((int)hi, (int)lo);
}

// FP64 -> FP32 rounded to nearest even, on the integer pipe.  Results below
// the FP32 normal range flush to signed zero, above it become Inf.
__device__ __forceinline__ float d2f_bits(double x) {
  const unsigned int hi = (unsigned int)__double2hiint(x), lo = (unsigned int)__double2loint(x);
  const unsigned int sign = hi & 0x80000000u;
  const int e = (int)((hi >> 20) & 0x7ffu);
  if (e == 0x7ff) return __uint_as_float(sign | 0x7f800000u | ((hi & 0xfffffu) ? 0x400000u : 0u));
  const int fe = e - 896;
  if (fe <= 0) return __uint_as_float(sign);
  // 23 kept mantissa bits: 20 from hi, 3 from the top of lo; 29 dropped bits
  unsigned int mant = ((hi & 0xfffffu) << 3) | (lo >> 29);
  const unsigned int rem = lo & 0x1fffffffu;
  unsigned int r = ((unsigned int)fe << 23) + mant;
  if (rem > 0x10000000u || (rem == 0x10000000u && (mant & 1u))) r += 1u;  // carry may bump the exponent
  if (r >= 0x7f800000u) return __uint_as_float(sign | 0x7f800000u);
  return __uint_as_float(sign | r);
}

__device__ __forceinline__ double dsqrt_(double x) { return sqrt(x); }
__device__ __forceinline__ float dsqrt_(float x) { return sqrtf(x); }
__device__ __forceinline__ double dabs_(double x) { return fabs(x); }
__device__ __forceinline__ float dabs_(float x) { return fabsf(x); }
// x / 2 (exact): 0.5 * x in FP64 / FP32, a scaling of both words in df64
__device__ __forceinline__ double half(double x) { return 0.5 * x; }
__device__ __forceinline__ float half(float x) { return 0.5f * x; }

#if FVS_MIXED
// FP32 limiter with every product and sum pinned (explicit multiply-adds),
// so that the compiler's contraction choices cannot differ between the
// kernels that inline it (the separate gradient kernel and the fused tile
// stage give bit-identical limiter values)
__device__ __forceinline__ float limiter_fn(int type, float a, float b, float eps2) {
  if (type == FVS_LIM_VENK) {
    const float num = __fmaf_rn(__fmul_rn(2.0f, b), a, __fmaf_rn(a, a, eps2));
    const float den = __fadd_rn(__fmaf_rn(a, b, __fmaf_rn(a, a, __fmul_rn(2.0f, __fmul_rn(b, b)))), eps2);
    return num / den;
  }
  if (type == FVS_LIM_BARTH) { const float q = a / b; return q < 1.0f ? q : 1.0f; }
  const float num = __fmaf_rn(__fmaf_rn(a, a, eps2), b, __fmul_rn(__fmaf_rn(b, b, eps2), a));
  const float den = __fmaf_rn(2.0f, eps2, __fmaf_rn(a, a, __fmul_rn(b, b)));
  return (num / den) / __fadd_rn(b, eps2);
}
// a face value p + cx gx + cy gy with the same pinned sequence
__device__ __forceinline__ float face_value(float p, float cx, float gx, float cy, float gy) {
  return __fmaf_rn(cy, gy, __fmaf_rn(cx, gx, p));
}
#else
// limiter, src/gradient_limiter.f90:103-134 (eps2 precomputed per cell)
__device__ __forceinline__ T limiter_fn(int type, T a, T b, T eps2) {
  if (type == FVS_LIM_VENK) return ((a * a + eps2) + T(2) * b * a) / (a * a + T(2) * (b * b) + a * b + eps2);
  if (type == FVS_LIM_BARTH) { T q = a / b; return q < T(1) ? q : T(1); }
  T l = ((b * b + eps2) * a + (a * a + eps2) * b) / (a * a + b * b + T(2) * eps2);
  return l / (b + eps2);
}
__device__ __forceinline__ T face_value(T p, T cx, T gx, T cy, T gy) { return p + cx * gx + cy * gy; }
#endif

// flux_invscid_roe, src/flux_invscid.f90:37-136 (same operation order)
__device__ __forceinline__ void roe_flux(T gamma, const T* pl, const T* pr, T nx, T ny, T* flux, T& ws_max) {
  const T tx = -ny, ty = nx;
  const T rhoL = pl[0], uL = pl[1], vL = pl[2], pL = pl[3];
  const T rhoR = pr[0], uR = pr[1], vR = pr[2], pR = pr[3];
  const T unL = uL * nx + vL * ny, unR = uR * nx + vR * ny;
  const T utL = uL * tx + vL * ty, utR = uR * tx + vR * ty;
  const T aL = dsqrt_(gamma * pL / rhoL), aR = dsqrt_(gamma * pR / rhoR);
  const T kL = T(0.5) * (uL * uL + vL * vL), kR = T(0.5) * (uR * uR + vR * vR);
  const T HL = aL * aL / (gamma - T(1)) + kL, HR = aR * aR / (gamma - T(1)) + kR;
  const T RT = dsqrt_(rhoR / rhoL);
  const T rho = RT * rhoL;
  const T u = (uL + RT * uR) / (T(1) + RT);
  const T v = (vL + RT * vR) / (T(1) + RT);
  const T H = (HL + RT * HR) / (T(1) + RT);
  const T a = dsqrt_((gamma - T(1)) * (H - T(0.5) * (u * u + v * v)));
  const T un = u * nx + v * ny;
  const T ut = u * tx + v * ty;
  const T drho = rhoR - rhoL, dp = pR - pL, dun = unR - unL, dut = utR - utL;
  T LdU[4], ws[4];
  LdU[0] = (dp - rho * a * dun) / (T(2) * a * a);
  LdU[1] = rho * dut;
  LdU[2] = drho - dp / (a * a);
  LdU[3] = (dp + rho * a * dun) / (T(2) * a * a);
  ws[0] = dabs_(un - a); ws[1] = dabs_(un); ws[2] = dabs_(un); ws[3] = dabs_(un + a);
  const T dws = T(1) / T(5);
  if (ws[0] < dws) ws[0] = T(0.5) * (ws[0] * ws[0] / dws + dws);
  if (ws[3] < dws) ws[3] = T(0.5) * (ws[3] * ws[3] / dws + dws);
  const T tke = T(0.5) * (u * u + v * v);
  const T Rv[4][4] = {{T(1), T(0), T(1), T(1)},
                      {u - a * nx, tx, u, u + a * nx},
                      {v - a * ny, ty, v, v + a * ny},
                      {H - un * a, ut, tke, H + un * a}};
  T diss[4];
#pragma unroll
  for (int i = 0; i < 4; i++) {
    T s = T(0);
#pragma unroll
    for (int j = 0; j < 4; j++) s = s + ws[j] * LdU[j] * Rv[i][j];
    diss[i] = s;
  }
  T fL[4], fR[4];
  fL[0] = rhoL * unL;
  fL[1] = rhoL * unL * uL + pL * nx;
  fL[2] = rhoL * unL * vL + pL * ny;
  fL[3] = rhoL * unL * HL;
  fR[0] = rhoR * unR;
  fR[1] = rhoR * unR * uR + pR * nx;
  fR[2] = rhoR * unR * vR + pR * ny;
  fR[3] = rhoR * unR * HR;
#pragma unroll
  for (int i = 0; i < 4; i++) flux[i] = T(0.5) * (fL[i] + fR[i] - T(1) * diss[i]);
  ws_max = T(0.5) * (dabs_(un) + a);
}

// The same Roe flux, algebraically rearranged for fewer FP64 instructions
// (FP64 and MIXED builds; the strict build keeps the source form above):
//  - aL, aR enter only through aL*aL/(gamma-1) in HL, HR: no square roots
//  - one reciprocal each for rhoL, rhoR, 1+RT and a*a replaces 8 divisions
//  - the eigenvector sum drops the products with the constants 0 and 1
// Differences to the source form are rounding-level (relative ~1e-16 per
// operation), checked against the oracle at 1e-12.
// R: the scalar type (T, or the FP32 dual number of the linearised residual)
template <typename R>
__device__ __forceinline__ void roe_flux_fast_t(R gamma, R gm1, R igm1, const R* pl, const R* pr, R nx, R ny, R* flux,
                                                R& ws_max) {
  const R tx = -ny, ty = nx;
  const R rhoL = pl[0], uL = pl[1], vL = pl[2], pL = pl[3];
  const R rhoR = pr[0], uR = pr[1], vR = pr[2], pR = pr[3];
  const R riL = R(1) / rhoL, riR = R(1) / rhoR;
  const R unL = uL * nx + vL * ny, unR = uR * nx + vR * ny;
  const R utL = uL * tx + vL * ty, utR = uR * tx + vR * ty;
  const R HL = gamma * pL * riL * igm1 + half(uL * uL + vL * vL);
  const R HR = gamma * pR * riR * igm1 + half(uR * uR + vR * vR);
  const R RT = dsqrt_(rhoR * riL);
  const R rho = RT * rhoL;
  const R i1 = R(1) / (R(1) + RT);
  const R u = (uL + RT * uR) * i1;
  const R v = (vL + RT * vR) * i1;
  const R H = (HL + RT * HR) * i1;
  const R q2 = half(u * u + v * v);
  const R a2 = gm1 * (H - q2);
  const R a = dsqrt_(a2);
  const R ia2 = R(1) / a2;
  const R un = u * nx + v * ny;
  const R ut = u * tx + v * ty;
  const R drho = rhoR - rhoL, dp = pR - pL, dun = unR - unL, dut = utR - utL;
  const R rad = rho * a * dun;
  const R L0 = half(dp - rad) * ia2;
  const R L1 = rho * dut;
  const R L2 = drho - dp * ia2;
  const R L3 = half(dp + rad) * ia2;
  R ws0 = dabs_(un - a), ws3 = dabs_(un + a);
  const R ws1 = dabs_(un);
  if (ws0 < R(0.2)) ws0 = half(ws0 * ws0 * R(5) + R(0.2));
  if (ws3 < R(0.2)) ws3 = half(ws3 * ws3 * R(5) + R(0.2));
  const R w0 = ws0 * L0, w1 = ws1 * L1, w2 = ws1 * L2, w3 = ws3 * L3;
  const R s03 = w0 + w3, s = s03 + w2, dw = (w3 - w0) * a;
  const R diss0 = s;
  const R diss1 = u * s + dw * nx + w1 * tx;
  const R diss2 = v * s + dw * ny + w1 * ty;
  const R diss3 = H * s03 + un * dw + w1 * ut + w2 * q2;
  const R mL = rhoL * unL, mR = rhoR * unR;
  flux[0] = half(mL + mR - diss0);
  flux[1] = half(mL * uL + mR * uR + (pL + pR) * nx - diss1);
  flux[2] = half(mL * vL + mR * vR + (pL + pR) * ny - diss2);
  flux[3] = half(mL * HL + mR * HR - diss3);
  ws_max = half(ws1 + a);
}

__device__ __forceinline__ void roe_flux_fast(T gamma, T gm1, T igm1, const T* pl, const T* pr, T nx, T ny, T* flux,
                                              T& ws_max) {
  roe_flux_fast_t<T>(gamma, gm1, igm1, pl, pr, nx, ny, flux, ws_max);
}

#if FVS_FP64_FAST
// The Roe flux of roe_flux_fast_t arranged for the FP64 pipe (FVS_PREC_FP64;
// GB300 issues 2 FP64 operations per clock per SM, and this function is most
// of the FP64 step):
//  - reciprocals and square roots from the hardware approximations refined
//    by one Newton-Raphson step (fp64_fast.cuh): 1/rhoL, 1/rhoR, 1/(1+RT),
//    and 1/sqrt(a^2), which gives both a = a^2 / sqrt(a^2) and 1/a^2
//  - gamma/(gamma-1) and the factor 1/2 of the flux and of the wave speed
//    folded into constants and into the face length (haf = af / 2); the
//    result is already flux * af and ws_max * af
//  - every product-sum a fused multiply-add; Harten's fix of the acoustic
//    waves written as 0.5 (l^2 / 0.2 + 0.2) = 2.5 l^2 + 0.1
// About 120 FP64 operations per edge against ~175 for roe_flux_fast_t with
// IEEE division and sqrt.  Rounding-level differences to the source form,
// checked against the oracle at 1e-12.
__device__ __forceinline__ void roe_flux_area_fp64(double gm1, double ggm1, const double* pl, const double* pr,
                                                   double nx, double ny, double af, double* flux, double& wsa) {
  const double rhoL = pl[0], uL = pl[1], vL = pl[2], pL = pl[3];
  const double rhoR = pr[0], uR = pr[1], vR = pr[2], pR = pr[3];
  const double riL = rcp_nr(rhoL), riR = rcp_nr(rhoR);
  const double unL = fma(uL, nx, vL * ny), unR = fma(uR, nx, vR * ny);
  const double utL = fma(vL, nx, -(uL * ny)), utR = fma(vR, nx, -(uR * ny));
  const double HL = fma(ggm1 * pL, riL, 0.5 * fma(uL, uL, vL * vL));
  const double HR = fma(ggm1 * pR, riR, 0.5 * fma(uR, uR, vR * vR));
  const double RT = sqrt_nr(rhoR * riL);
  const double rho = RT * rhoL;
  const double i1 = rcp_nr(1.0 + RT);
  const double u = fma(RT, uR, uL) * i1;
  const double v = fma(RT, vR, vL) * i1;
  const double H = fma(RT, HR, HL) * i1;
  const double q2 = 0.5 * fma(u, u, v * v);
  const double a2 = gm1 * (H - q2);
  const double ra = rsqrt_nr(a2);
  const double a = a2 * ra, ia2 = ra * ra;
  const double un = fma(u, nx, v * ny);
  const double ut = fma(v, nx, -(u * ny));
  const double drho = rhoR - rhoL, dp = pR - pL, dun = unR - unL, dut = utR - utL;
  const double rad = rho * a * dun;
  const double hia2 = 0.5 * ia2;
  const double L0 = (dp - rad) * hia2;
  const double L1 = rho * dut;
  const double L2 = fma(-dp, ia2, drho);
  const double L3 = (dp + rad) * hia2;
  double ws0 = fabs(un - a), ws3 = fabs(un + a);
  const double ws1 = fabs(un);
  if (ws0 < 0.2) ws0 = fma(2.5 * ws0, ws0, 0.1);
  if (ws3 < 0.2) ws3 = fma(2.5 * ws3, ws3, 0.1);
  const double w0 = ws0 * L0, w1 = ws1 * L1, w2 = ws1 * L2, w3 = ws3 * L3;
  const double s03 = w0 + w3, sd = s03 + w2, dw = (w3 - w0) * a;
  // eigenvector sum with tx = -ny, ty = nx
  const double diss1 = fma(u, sd, fma(dw, nx, -(w1 * ny)));
  const double diss2 = fma(v, sd, fma(dw, ny, w1 * nx));
  const double diss3 = fma(H, s03, fma(un, dw, fma(w1, ut, w2 * q2)));
  const double mL = rhoL * unL, mR = rhoR * unR;
  const double pLR = pL + pR;
  const double haf = 0.5 * af;
  flux[0] = ((mL + mR) - sd) * haf;
  flux[1] = (fma(mL, uL, mR * uR) + fma(pLR, nx, -diss1)) * haf;
  flux[2] = (fma(mL, vL, mR * vR) + fma(pLR, ny, -diss2)) * haf;
  flux[3] = (fma(mL, HL, mR * HR) - diss3) * haf;
  wsa = (ws1 + a) * haf;
}
#endif

// ---------------------------------------------------------------------------
// gradient (+ limiter) : one thread per cell
// ---------------------------------------------------------------------------
// Gradient (and limiter) of cell ic from its primitives pc; load(k, pj)
// fills pj with the primitives of stencil entry k (global CSR index).
// Shared by the separate gradient kernel (loads from global memory) and the
// fused tile stage (loads from shared memory): the same arithmetic.
// gradient_core over the stencil entries [b, e) with coef(k) the (LSQ or
// GG-cell) coefficient pair of entry k
template <int METHOD, int LIM, class Load, class Coef>
__device__ __forceinline__ void gradient_core_r(const DevView& d, int ic, const T* pc, int b, int e, Load load,
                                                Coef coef, T* gx, T* gy, T& phi_out) {
  T pmin[4], pmax[4];
#pragma unroll
  for (int v = 0; v < 4; v++) { pmin[v] = pc[v]; pmax[v] = pc[v]; }
  if (METHOD == FVS_GRAD_LSQ) {
    // grad_lsq, src/gradient_lsq.f90:393-401: sum over the stencil of
    // (coef * (p_j - p_i)) * w, stencil outer, variable inner
#pragma unroll
    for (int v = 0; v < 4; v++) { gx[v] = T(0); gy[v] = T(0); }
#if FVS_STRICT
    const T* __restrict__ W = static_cast<const T*>(d.st_w);
#endif
    for (int k = b; k < e; k++) {
      T pj[4];
      load(k, pj);
      const T2 c = coef(k);
#if FVS_STRICT
      const T w = W[k];
#endif
#pragma unroll
      for (int v = 0; v < 4; v++) {
        const T diff = pj[v] - pc[v];
#if FVS_STRICT
        gx[v] = gx[v] + c.x * diff * w;
        gy[v] = gy[v] + c.y * diff * w;
#elif FVS_DF
        // coefficients premultiplied by the weight on the host
        gx[v] = dfma(c.x, diff, gx[v]);
        gy[v] = dfma(c.y, diff, gy[v]);
#else
        // coefficients premultiplied by the weight on the host
        gx[v] = gx[v] + c.x * diff;
        gy[v] = gy[v] + c.y * diff;
#endif
        if (LIM) {
          pmin[v] = pj[v] < pmin[v] ? pj[v] : pmin[v];
          pmax[v] = pj[v] > pmax[v] ? pj[v] : pmax[v];
        }
      }
    }
  } else if (METHOD == FVS_GRAD_GGCB) {
    // grad_ggcb, src/gradient_ggcb.f90:123-135
    const T2 c0 = ld2(d.coef0, ic);
#pragma unroll
    for (int v = 0; v < 4; v++) { gx[v] = c0.x * pc[v]; gy[v] = c0.y * pc[v]; }
    for (int k = b; k < e; k++) {
      T pj[4];
      load(k, pj);
      const T2 c = coef(k);
#pragma unroll
      for (int v = 0; v < 4; v++) {
#if FVS_DF
        gx[v] = dfma(c.x, pj[v], gx[v]);
        gy[v] = dfma(c.y, pj[v], gy[v]);
#else
        gx[v] = gx[v] + c.x * pj[v];
        gy[v] = gy[v] + c.y * pj[v];
#endif
      }
    }
#if FVS_STRICT
    const T vol = d.vol[ic];
#pragma unroll
    for (int v = 0; v < 4; v++) { gx[v] = gx[v] / vol; gy[v] = gy[v] / vol; }
#else
    const T rv = static_cast<const T*>(d.volT)[ic];
#pragma unroll
    for (int v = 0; v < 4; v++) { gx[v] = gx[v] * rv; gy[v] = gy[v] * rv; }
#endif
  } else {
    // grad_ggnb, src/gradient_ggnb.f90:190-207
    const T2 c0 = ld2(d.coef0, ic);
#pragma unroll
    for (int v = 0; v < 4; v++) { gx[v] = c0.x * pc[v]; gy[v] = c0.y * pc[v]; }
    const T* __restrict__ CN = static_cast<const T*>(d.st_coef);
    for (int k = b; k < e; k++) {
      T pj[4];
      load(k, pj);
      const T cn = CN[k];
      const T2 ce = ld2(d.coefedg, 4 * ic + d.st_node[k]);
#pragma unroll
      for (int v = 0; v < 4; v++) { gx[v] = gx[v] + ce.x * cn * pj[v]; gy[v] = gy[v] + ce.y * cn * pj[v]; }
    }
#if FVS_STRICT
    const T vol = d.vol[ic];
#pragma unroll
    for (int v = 0; v < 4; v++) { gx[v] = gx[v] / vol; gy[v] = gy[v] / vol; }
#else
    const T rv = static_cast<const T*>(d.volT)[ic];
#pragma unroll
    for (int v = 0; v < 4; v++) { gx[v] = gx[v] * rv; gy[v] = gy[v] * rv; }
#endif
  }
  if (LIM) {
    // compute_gradient_limiter, src/gradient_limiter.f90:47-88
    const int nv = d.nvrt[ic];
    const T eps2 = static_cast<const T*>(d.eps2)[ic];
    T2 cp[4];
#pragma unroll
    for (int f = 0; f < 4; f++) cp[f] = ld2(d.cpos, 4 * ic + f);
    T phimin = T(1);
#pragma unroll
    for (int v = 0; v < 4; v++) {
      T pe[4] = {T(100), T(100), T(100), T(100)};
#pragma unroll
      for (int f = 0; f < 4; f++) {
        if (f >= nv) break;
        const T pf = face_value(pc[v], cp[f].x, gx[v], cp[f].y, gy[v]);
        const T dmax = pmax[v] - pc[v], dmin = pmin[v] - pc[v], diff = pf - pc[v];
        if (diff > T(0)) pe[f] = limiter_fn(d.limiter, dmax, diff, eps2);
        else if (diff < T(0)) pe[f] = limiter_fn(d.limiter, dmin, diff, eps2);
        else pe[f] = T(1);
      }
      T mv = pe[0];
#pragma unroll
      for (int f = 1; f < 4; f++) mv = pe[f] < mv ? pe[f] : mv;
      const T ph = mv < T(1) ? mv : T(1);
      phimin = (v == 0 || ph < phimin) ? ph : phimin;
    }
    phi_out = phimin;
  }
}

template <int METHOD, int LIM, class Load>
__device__ __forceinline__ void gradient_core(const DevView& d, int ic, const T* pc, Load load, T* gx, T* gy,
                                              T& phi_out) {
  gradient_core_r<METHOD, LIM>(d, ic, pc, d.st_ptr[ic], d.st_ptr[ic + 1], load,
                               [&](int k) { return ld2(d.st_coef, k); }, gx, gy, phi_out);
}

template <int METHOD, int LIM, bool COH>
__device__ __forceinline__ void gradient_item(const DevView& d, int ic) {
  const T* P = static_cast<const T*>(d.Pv);
  T pc[4], gx[4], gy[4], ph;
  ldc4<COH>(P, ic, pc);
  gradient_core<METHOD, LIM>(
      d, ic, pc, [&](int k, T* pj) { ldc4<COH>(P, chk_idx(d.bounds_err, d.st_cell[k], 0, d.nc, SITE_STENCIL), pj); },
      gx, gy, ph);
  st4(static_cast<T*>(d.Gx), ic, gx);
  st4(static_cast<T*>(d.Gy), ic, gy);
  if (LIM) static_cast<T*>(d.phi)[ic] = ph;
}

template <int METHOD, int LIM>
__global__ void __launch_bounds__(256) k_gradient(const DevView d) {
  pdl_wait();
  pdl_trigger();
  const int ic = blockIdx.x * blockDim.x + threadIdx.x;
  if (ic < d.nc) gradient_item<METHOD, LIM, false>(d, ic);
}

// ---------------------------------------------------------------------------
// boundary ghost state, bc_flux src/residual.f90:183-255
// ---------------------------------------------------------------------------
__device__ __forceinline__ double texp_(double x) { return exp(x); }
__device__ __forceinline__ float texp_(float x) { return expf(x); }
__device__ __forceinline__ double tpow_(double x, double y) { return pow(x, y); }
__device__ __forceinline__ float tpow_(float x, float y) { return powf(x, y); }
__device__ __forceinline__ double tsin_(double x) { return sin(x); }
__device__ __forceinline__ float tsin_(float x) { return sinf(x); }
__device__ __forceinline__ double tcos_(double x) { return cos(x); }
__device__ __forceinline__ float tcos_(float x) { return cosf(x); }
// double-float: boundary values of the Dirichlet states, evaluated in FP64
__device__ __forceinline__ df64 texp_(df64 x) { return df_from_double(exp(double(x))); }
__device__ __forceinline__ df64 tpow_(df64 x, df64 y) { return df_from_double(pow(double(x), double(y))); }
__device__ __forceinline__ df64 tsin_(df64 x) { return df_from_double(sin(double(x))); }
__device__ __forceinline__ df64 tcos_(df64 x) { return df_from_double(cos(double(x))); }
// an FP64 value in the compute type
__device__ __forceinline__ T to_t(double x) {
#if FVS_DF
  return df_from_double(x);
#else
  return T(x);
#endif
}

__device__ __forceinline__ void ghost_state(const DevView& d, int rec, double time, T x, T y, T nx, T ny,
                                            const T* pfL, T* pfR) {
  const int type = rec & 15;
  if (type == FVS_BC_FREESTREAM) {
    // the free stream of the slot's case (batched meshes), else the handle's
    const double* pi = d.case_pinf ? d.case_pinf + 4 * (rec >> 4) : d.pinf;
#pragma unroll
    for (int k = 0; k < 4; k++) pfR[k] = to_t(pi[k]);
  } else if (type == FVS_BC_SLIP_WALL) {
    const T un = pfL[1] * nx + pfL[2] * ny;
    pfR[0] = pfL[0];
    pfR[1] = pfL[1] - T(2) * un * nx;
    pfR[2] = pfL[2] - T(2) * un * ny;
    pfR[3] = pfL[3];
  } else if (d.vortex) {
    // compute_isentropic_vortex, src/mms.f90:219-265
    const T g = T(d.gamma), q = T(d.vkappa) / (T(2) * T(3.141592653589793238462643383279502884));
    const T T_inf = T(d.vinf[3]) / T(d.vinf[0]);
    const T dx = x - (T(d.vx) + T(d.vinf[1]) * T(time));
    const T dy = y - (T(d.vy) + T(d.vinf[2]) * T(time));
    const T r = dsqrt_(dx * dx + dy * dy);
    pfR[1] = T(d.vinf[1]) - q * dy * texp_(T(0.5) * (T(1) - r * r));
    pfR[2] = T(d.vinf[2]) + q * dx * texp_(T(0.5) * (T(1) - r * r));
    const T temp = T_inf - (q * q) * (g - T(1)) / (T(2) * g) * texp_(T(1) - r * r);
    pfR[0] = tpow_(temp, T(1) / (g - T(1)));
    pfR[3] = tpow_(pfR[0], g);
  } else {
    // manufactured solution, src/mms.f90:187-213 (values only)
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const double* m = d.mc + 4 * k;
      pfR[k] = T(m[0]) + T(m[1]) * tsin_(T(m[2]) * x + T(m[3]) * y);
    }
  }
}

// ---------------------------------------------------------------------------
// edge fluxes : one thread per edge slot
// ---------------------------------------------------------------------------
// SPEC: non-strict builds only, kappa = 0 and no limiter (phi = 1), where the
// reconstruction reduces to p + (dx, dy).grad exactly
// REC: the reconstruction.  REC_GENERAL: UMUSCL with the limiter;
// REC_SPEC (non-strict builds only): kappa = 0 and no limiter (phi = 1), where
// the reconstruction reduces to p + (dx, dy).grad exactly; REC_FIRST: first
// order, face states = cell states (the reference's p + 0 * (...) for finite
// values) and no gradient is read.
enum : int { REC_GENERAL = 0, REC_SPEC = 1, REC_FIRST = 2 };

#if FVS_DF
// The Roe flux of roe_flux_area_fp64 in double-float arithmetic (the
// double-float build): the same folded constants and order; every FP64 fused
// multiply-add there is dfma here and the sums of like-signed terms are
// sloppy sums (df64.cuh), while the differences of face values, wave speeds
// and dissipation terms keep the accurate sum.  Reciprocals and square roots
// are the accurate double-float division and root.  About 40 % fewer FP32
// instructions per edge than roe_flux_fast_t<df64>; its error stays near
// 2^-47 of the flux's operands.
__device__ __forceinline__ void roe_flux_area_df(df64 gm1, df64 ggm1, const df64* pl, const df64* pr, df64 nx,
                                                 df64 ny, df64 af, df64* flux, df64& wsa) {
  const df64 one(1.f, 0.f);
  const df64 rhoL = pl[0], uL = pl[1], vL = pl[2], pL = pl[3];
  const df64 rhoR = pr[0], uR = pr[1], vR = pr[2], pR = pr[3];
  const df64 riL = one / rhoL, riR = one / rhoR;
  const df64 unL = dfma(uL, nx, vL * ny), unR = dfma(uR, nx, vR * ny);
  const df64 utL = dfma(vL, nx, -(uL * ny)), utR = dfma(vR, nx, -(uR * ny));
  const df64 HL = dfma(ggm1 * pL, riL, half(dfma(uL, uL, vL * vL)));
  const df64 HR = dfma(ggm1 * pR, riR, half(dfma(uR, uR, vR * vR)));
  const df64 RT = dsqrt_(rhoR * riL);
  const df64 rho = RT * rhoL;
  const df64 i1 = one / dadd_s(one, RT);
  const df64 u = dfma(RT, uR, uL) * i1;
  const df64 v = dfma(RT, vR, vL) * i1;
  const df64 H = dfma(RT, HR, HL) * i1;
  const df64 q2 = half(dfma(u, u, v * v));
  const df64 a2 = gm1 * (H - q2);
  const df64 a = dsqrt_(a2);
  const df64 ia2 = one / a2;
  const df64 un = dfma(u, nx, v * ny);
  const df64 ut = dfma(v, nx, -(u * ny));
  const df64 drho = rhoR - rhoL, dp = pR - pL, dun = unR - unL, dut = utR - utL;
  const df64 rad = rho * a * dun;
  const df64 hia2 = half(ia2);
  const df64 L0 = (dp - rad) * hia2;
  const df64 L1 = rho * dut;
  const df64 L2 = dfma(-dp, ia2, drho);
  const df64 L3 = (dp + rad) * hia2;
  df64 ws0 = dabs_(un - a), ws3 = dabs_(un + a);
  const df64 ws1 = dabs_(un);
  // Harten's fix, 0.5 (l^2 / 0.2 + 0.2) = 2.5 l^2 + 0.1
  const df64 lim(0.2), c01(0.1);
  if (ws0 < lim) ws0 = dfma(mul_fp(ws0, 2.5f), ws0, c01);
  if (ws3 < lim) ws3 = dfma(mul_fp(ws3, 2.5f), ws3, c01);
  const df64 w0 = ws0 * L0, w1 = ws1 * L1, w2 = ws1 * L2, w3 = ws3 * L3;
  const df64 s03 = w0 + w3, sd = s03 + w2, dw = (w3 - w0) * a;
  // eigenvector sum with tx = -ny, ty = nx
  const df64 diss1 = dfma(u, sd, dfma(dw, nx, -(w1 * ny)));
  const df64 diss2 = dfma(v, sd, dfma(dw, ny, w1 * nx));
  const df64 diss3 = dfma(H, s03, dfma(un, dw, dfma(w1, ut, w2 * q2)));
  const df64 mL = rhoL * unL, mR = rhoR * unR;
  const df64 pLR = dadd_s(pL, pR);
  const df64 haf = half(af);
  flux[0] = ((mL + mR) - sd) * haf;
  flux[1] = (dfma(mL, uL, mR * uR) + dfma(pLR, nx, -diss1)) * haf;
  flux[2] = (dfma(mL, vL, mR * vR) + dfma(pLR, ny, -diss2)) * haf;
  flux[3] = (dfma(mL, HL, mR * HR) - diss3) * haf;
  wsa = dadd_s(ws1, a) * haf;
}
#endif

// Roe flux of one edge slot from its face states, times the face length
// (flux) and the wave speed times the length (wsa)
__device__ __forceinline__ void flux_eval(const DevView& d, const T* pfL, const T* pfR, T2 n, T af, T* flux, T& wsa) {
#if FVS_FP64_FAST
  roe_flux_area_fp64(d.gm1, d.ggm1, pfL, pfR, n.x, n.y, af, flux, wsa);
#elif FVS_DF
  roe_flux_area_df(TP(gm1), TP(ggm1), pfL, pfR, n.x, n.y, af, flux, wsa);
#else
  T wsm;
#if FVS_STRICT
  roe_flux(T(d.gamma), pfL, pfR, n.x, n.y, flux, wsm);
#else
  roe_flux_fast(TP(gamma), TP(gm1), TP(igm1), pfL, pfR, n.x, n.y, flux, wsm);
#endif
#pragma unroll
  for (int v = 0; v < 4; v++) flux[v] = flux[v] * af;
  wsa = wsm * af;
#endif
}

// ... into the slot's record
__device__ __forceinline__ void flux_finish(const DevView& d, int e, const T* pfL, const T* pfR, T2 n, T af) {
  T flux[4], wsa;
  flux_eval(d, pfL, pfR, n, af, flux, wsa);
  st4(static_cast<T*>(d.eflux), e, flux);
  static_cast<T*>(d.ews)[e] = wsa;
}

// Face states of edge slot e (src/residual.f90:83-92 interior, :128-137
// boundary) from the data of its L cell (pl, gxl, gyl, phiL) and, on an
// interior slot, its R cell; a boundary slot's right state is the ghost
// state.  REC_FIRST reads no gradient; REC_SPEC no limiter value.  Shared by
// the edge-flux kernel and the fused tile stage: the same arithmetic.
template <int REC>
__device__ __forceinline__ void face_states(const DevView& d, int e, bool interior, double time, T2 n, T2 dl, T2 dr,
                                            const T* pl, const T* gxl, const T* gyl, T phiL, const T* pr,
                                            const T* gxr, const T* gyr, T phiR, T* pfL, T* pfR) {
  constexpr bool SPEC = REC == REC_SPEC;
  if (REC == REC_FIRST) {
#pragma unroll
    for (int v = 0; v < 4; v++) pfL[v] = pl[v];
    if (interior) {
#pragma unroll
      for (int v = 0; v < 4; v++) pfR[v] = pr[v];
    } else {
      const T2 xy = ld2(d.exy, e);
      ghost_state(d, d.ebtype[e], time, xy.x, xy.y, n.x, n.y, pfL, pfR);
    }
    return;
  }
  if (interior) {
    // src/residual.f90:83-92
    if (SPEC) {
#pragma unroll
      for (int v = 0; v < 4; v++) {
#if FVS_FP64_FAST
        // two fused multiply-adds per face value
        pfL[v] = fma(dl.x, gxl[v], fma(dl.y, gyl[v], pl[v]));
        pfR[v] = fma(dr.x, gxr[v], fma(dr.y, gyr[v], pr[v]));
#elif FVS_DF
        pfL[v] = dfma(dl.x, gxl[v], dfma(dl.y, gyl[v], pl[v]));
        pfR[v] = dfma(dr.x, gxr[v], dfma(dr.y, gyr[v], pr[v]));
#else
        pfL[v] = pl[v] + (dl.x * gxl[v] + dl.y * gyl[v]);
        pfR[v] = pr[v] + (dr.x * gxr[v] + dr.y * gyr[v]);
#endif
      }
    } else {
      const T kh = TP(khalf), nkh = TP(nkhalf), omk = TP(omk);
#pragma unroll
      for (int v = 0; v < 4; v++) {
        const T gradC = pr[v] - pl[v];
        const T gradL = dl.x * gxl[v] + dl.y * gyl[v];
        const T gradR = dr.x * gxr[v] + dr.y * gyr[v];
        pfL[v] = pl[v] + phiL * (kh * gradC + omk * gradL);
        pfR[v] = pr[v] + phiR * (nkh * gradC + omk * gradR);
      }
    }
  } else {
    // src/residual.f90:128-137
#pragma unroll
    for (int v = 0; v < 4; v++) pfL[v] = pl[v] + phiL * (dl.x * gxl[v] + dl.y * gyl[v]);
    // boundary record of the slot: type | case << 4, face centre
    const T2 xy = ld2(d.exy, e);
    ghost_state(d, d.ebtype[e], time, xy.x, xy.y, n.x, n.y, pfL, pfR);
  }
}

// flux * area and ws * area of edge slot e from the cell data in global
// memory (the edge-flux kernel's loads and arithmetic)
template <int REC, bool COH>
__device__ __forceinline__ void flux_compute(const DevView& d, int e, double time, T* flux, T& wsa) {
  constexpr bool SPEC = REC == REC_SPEC;
  const T* P = static_cast<const T*>(d.Pv);
  const T* GX = static_cast<const T*>(d.Gx);
  const T* GY = static_cast<const T*>(d.Gy);
  const T* PH = static_cast<const T*>(d.phi);
  int2 lr = d.ecell[e];
  lr.x = chk_idx(d.bounds_err, lr.x, 0, d.nc, SITE_EDGE_L);
  lr.y = chk_idx(d.bounds_err, lr.y, -1, d.nc, SITE_EDGE_R);
  const T2 n = ld2(d.enrm, e);
  const T af = static_cast<const T*>(d.earea)[e];
  const bool interior = lr.y >= 0;
  T pl[4], gxl[4], gyl[4], pr[4], gxr[4], gyr[4], pfL[4], pfR[4];
  T phiL = T(1), phiR = T(1);
  ldc4<COH>(P, lr.x, pl);
  if (REC != REC_FIRST) {
    ldc4<COH>(GX, lr.x, gxl);
    ldc4<COH>(GY, lr.x, gyl);
    if (!SPEC) phiL = ldc1<COH>(PH, lr.x);
  }
  if (interior) {
    ldc4<COH>(P, lr.y, pr);
    if (REC != REC_FIRST) {
      ldc4<COH>(GX, lr.y, gxr);
      ldc4<COH>(GY, lr.y, gyr);
      if (!SPEC) phiR = ldc1<COH>(PH, lr.y);
    }
  }
  T2 dl = {T(0), T(0)}, dr = {T(0), T(0)};
  if (REC != REC_FIRST) {
    dl = ld2(d.edL, e);
    if (interior) dr = ld2(d.edR, e);
  }
  face_states<REC>(d, e, interior, time, n, dl, dr, pl, gxl, gyl, phiL, pr, gxr, gyr, phiR, pfL, pfR);
  flux_eval(d, pfL, pfR, n, af, flux, wsa);
}

// ws_out: also store ws * area (read only by a steady scheme's first stage,
// for the local time step, and by residual evaluations)
template <int REC, bool COH>
__device__ __forceinline__ void flux_item(const DevView& d, int e, double time, bool ws_out = true) {
  T flux[4], wsa;
  flux_compute<REC, COH>(d, e, time, flux, wsa);
  st4(static_cast<T*>(d.eflux), e, flux);
  if (ws_out) static_cast<T*>(d.ews)[e] = wsa;
}

// First-order flux of two edge slots per call (e1 < 0: e0 alone).  The
// operands of both are loaded before either flux is evaluated, so each thread
// keeps two chains of dependent loads in flight; the arithmetic is that of
// flux_item<REC_FIRST>.
template <bool COH>
__device__ __forceinline__ void flux_first_pair(const DevView& d, int e0, int e1, double time) {
  const T* P = static_cast<const T*>(d.Pv);
  const int e[2] = {e0, e1 >= 0 ? e1 : e0};
  int2 lr[2];
  T2 n[2];
  T af[2], pl[2][4], pr[2][4];
#pragma unroll
  for (int j = 0; j < 2; j++) {
    lr[j] = d.ecell[e[j]];
    n[j] = ld2(d.enrm, e[j]);
    af[j] = static_cast<const T*>(d.earea)[e[j]];
  }
#pragma unroll
  for (int j = 0; j < 2; j++) {
    ldc4<COH>(P, lr[j].x, pl[j]);
    if (lr[j].y >= 0) ldc4<COH>(P, lr[j].y, pr[j]);
  }
#pragma unroll
  for (int j = 0; j < 2; j++) {
    if (j == 1 && e1 < 0) break;
    if (lr[j].y < 0) {
      const T2 xy = ld2(d.exy, e[j]);
      ghost_state(d, d.ebtype[e[j]], time, xy.x, xy.y, n[j].x, n[j].y, pl[j], pr[j]);
    }
    flux_finish(d, e[j], pl[j], pr[j], n[j], af[j]);
  }
}

// the edge slots [b, end) of a tile with stride `stride` (the block's
// threads), first order two at a time
template <int REC, bool COH>
__device__ __forceinline__ void flux_range(const DevView& d, int b, int end, int stride, double time) {
  if (REC == REC_FIRST) {
    for (int e = b; e < end; e += 2 * stride) flux_first_pair<COH>(d, e, e + stride < end ? e + stride : -1, time);
  } else {
    for (int e = b; e < end; e += stride) flux_item<REC, COH>(d, e, time);
  }
}

template <int REC>
__global__ void __launch_bounds__(256) k_flux(const DevView d, double dts, int ws_out) {
  pdl_wait();
  pdl_trigger();
  const int e = blockIdx.x * blockDim.x + threadIdx.x;
  if (e < d.nedge) flux_item<REC, false>(d, e, d.tctl[1] + dts, ws_out != 0);
}

// ---------------------------------------------------------------------------
// per-cell gather of the edge slots in the reference's summation order
// ---------------------------------------------------------------------------
#if FVS_MIXED
// FP32 flux slots summed with an error-free transformation (TwoSum): hi + lo
// equals the exact sum of the slots to ~2^-48 relative, then one FP64 add per
// component; the result matches an FP64 accumulation of the FP32 fluxes.
__device__ __forceinline__ void two_sum(float& hi, float& lo, float x) {
  const float s = hi + x;
  const float bp = s - hi;
  lo += (hi - (s - bp)) + (x - bp);
  hi = s;
}

template <bool WS, bool COH>
__device__ __forceinline__ void cell_residual(const DevView& d, int ic, double* res, double& ws) {
  float hi[4] = {0.f, 0.f, 0.f, 0.f}, lo[4] = {0.f, 0.f, 0.f, 0.f}, wh = 0.f, wl = 0.f;
  const int4 cf = d.cflist[ic];
  const int sl[4] = {cf.x, cf.y, cf.z, cf.w};
#pragma unroll
  for (int j = 0; j < 4; j++) {
    const int s = sl[j];
    if (s == 0) continue;
    const int idx = (s > 0 ? s : -s) - 1;
    float f[4];
    ldc4<COH>(static_cast<const float*>(d.eflux), idx, f);
#pragma unroll
    for (int v = 0; v < 4; v++) two_sum(hi[v], lo[v], s > 0 ? f[v] : -f[v]);
    if (WS) two_sum(wh, wl, ldc1<COH>(static_cast<const float*>(d.ews), idx));
  }
  const double rv = -d.rvol[ic];
#pragma unroll
  for (int v = 0; v < 4; v++) res[v] = (f2d_bits(hi[v]) + f2d_bits(lo[v])) * rv;
  ws = WS ? f2d_bits(wh) + f2d_bits(wl) : 0.0;
}
#elif FVS_DF
// df64 value as FP64: two exact conversions on the integer pipe, one exact add
__device__ __forceinline__ double to_double(df64 x) { return f2d_bits(x.hi) + f2d_bits(x.lo); }

// df64 flux records of a cell's faces summed in df64 in its gather order
// (the reference's order; see residual_from_faces_f), times -1/vol in df64
template <bool WS, class Get>
__device__ __forceinline__ void residual_from_faces_df(const int* sl, df64 rv, Get get, df64* res, double& ws) {
  df64 r[4] = {df64(0.f, 0.f), df64(0.f, 0.f), df64(0.f, 0.f), df64(0.f, 0.f)}, w(0.f, 0.f);
#pragma unroll
  for (int j = 0; j < 4; j++) {
    const int s = sl[j];
    if (s == 0) continue;
    const int idx = (s > 0 ? s : -s) - 1;
    df64 f[4], wf(0.f, 0.f);
    get(idx, f, wf);
#pragma unroll
    for (int v = 0; v < 4; v++) r[v] = s > 0 ? r[v] + f[v] : r[v] - f[v];
    if (WS) w = w + wf;
  }
#pragma unroll
  for (int v = 0; v < 4; v++) res[v] = r[v] * rv;
  ws = WS ? to_double(w) : 0.0;
}

template <bool WS, bool COH>
__device__ __forceinline__ void cell_residual_df(const DevView& d, int ic, df64* res, double& ws) {
  const int4 cf = d.cflist[ic];
  const int sl[4] = {cf.x, cf.y, cf.z, cf.w};
  const df64 rv = -static_cast<const df64*>(d.volT)[ic];
  residual_from_faces_df<WS>(sl, rv, [&](int idx, df64* f, df64& w) {
    ldc4<COH>(static_cast<const df64*>(d.eflux), idx, f);
    if (WS) w = ldc1<COH>(static_cast<const df64*>(d.ews), idx);
  }, res, ws);
}

// ... as FP64 (one exact FP64 addition per component)
template <bool WS, bool COH>
__device__ __forceinline__ void cell_residual(const DevView& d, int ic, double* res, double& ws) {
  df64 r[4];
  cell_residual_df<WS, COH>(d, ic, r, ws);
#pragma unroll
  for (int v = 0; v < 4; v++) res[v] = to_double(r[v]);
}
#else
template <bool WS, bool COH>
__device__ __forceinline__ void gather_slot(const DevView& d, int s, double* r, double& ws) {
  if (s == 0) return;
  const int idx = chk_idx(d.bounds_err, (s > 0 ? s : -s) - 1, 0, d.nedge, SITE_GATHER);
  double f[4];
  ldc4<COH>(static_cast<const double*>(d.eflux), idx, f);
  if (s > 0) {
#pragma unroll
    for (int v = 0; v < 4; v++) r[v] = r[v] + f[v];
  } else {
#pragma unroll
    for (int v = 0; v < 4; v++) r[v] = r[v] - f[v];
  }
  if (WS) ws = ws + ldc1<COH>(static_cast<const double*>(d.ews), idx);
}

// the flux slots of cell ic summed in its gather order (the reference's
// order); the FP64 build starts the sums from the first slot instead of from
// zero (the same values, four additions fewer)
template <bool WS, bool COH>
__device__ __forceinline__ void cell_flux_sum(const DevView& d, int ic, double* r, double& ws) {
  ws = 0.0;
  const int4 cf = d.cflist[ic];
#if FVS_STRICT
#pragma unroll
  for (int v = 0; v < 4; v++) r[v] = 0.0;
  gather_slot<WS, COH>(d, cf.x, r, ws);
#else
  if (cf.x != 0) {
    const int idx = chk_idx(d.bounds_err, (cf.x > 0 ? cf.x : -cf.x) - 1, 0, d.nedge, SITE_GATHER);
    ldc4<COH>(static_cast<const double*>(d.eflux), idx, r);
    if (cf.x < 0) {
#pragma unroll
      for (int v = 0; v < 4; v++) r[v] = -r[v];
    }
    if (WS) ws = ldc1<COH>(static_cast<const double*>(d.ews), idx);
  } else {
#pragma unroll
    for (int v = 0; v < 4; v++) r[v] = 0.0;
  }
#endif
  gather_slot<WS, COH>(d, cf.y, r, ws);
  gather_slot<WS, COH>(d, cf.z, r, ws);
  gather_slot<WS, COH>(d, cf.w, r, ws);
}

template <bool WS, bool COH>
__device__ __forceinline__ void cell_residual(const DevView& d, int ic, double* res, double& ws) {
  double r[4];
  cell_flux_sum<WS, COH>(d, ic, r, ws);
#if FVS_STRICT
  const double vol = d.vol[ic];
#pragma unroll
  for (int v = 0; v < 4; v++) res[v] = -r[v] / vol;  // src/residual.f90:164-166
#else
  const double rv = -d.rvol[ic];
#pragma unroll
  for (int v = 0; v < 4; v++) res[v] = r[v] * rv;
#endif
}
#endif

#if FVS_DF
// primitives from a double-float conservative state
__device__ __forceinline__ void cons2prim_df(df64 g, const df64* u, df64* p) {
  const df64 r = u[0], ri = df64(1) / r;
  p[0] = r;
  p[1] = u[1] * ri;
  p[2] = u[2] * ri;
  p[3] = g * (u[3] - df64(0.5) * r * (p[1] * p[1] + p[2] * p[2]));
}
#endif

// g = gamma - 1 in the compute type
__device__ __forceinline__ void cons2prim(T g, const double* u, T* p) {
#if FVS_MIXED
  const float r = d2f_bits(u[0]), ri = 1.0f / r;
  p[0] = r;
  p[1] = d2f_bits(u[1]) * ri;
  p[2] = d2f_bits(u[2]) * ri;
  p[3] = g * (d2f_bits(u[3]) - 0.5f * r * (p[1] * p[1] + p[2] * p[2]));
#elif FVS_DF
  const df64 ud[4] = {df_from_double(u[0]), df_from_double(u[1]), df_from_double(u[2]), df_from_double(u[3])};
  cons2prim_df(g, ud, p);
#elif !FVS_STRICT
  const double ri = rcp_nr(u[0]);
  p[0] = u[0];
  p[1] = u[1] * ri;
  p[2] = u[2] * ri;
  p[3] = g * (u[3] - 0.5 * p[0] * (p[1] * p[1] + p[2] * p[2]));
#else
  // cvar2pvar, src/data_solution.f90:78-84
  p[0] = u[0];
  p[1] = u[1] / u[0];
  p[2] = u[2] / u[0];
  p[3] = g * (u[3] - 0.5 * p[0] * (p[1] * p[1] + p[2] * p[2]));
#endif
}

// deterministic block sum of 4 doubles (shared-memory tree: one add per
// element instead of five shuffle-adds per lane); thread 0 gets the sums
// sh: 4 x 256 doubles of shared memory
__device__ __forceinline__ void block_sum4_in(const double* v, double* out, double* sh) {
  const int t = threadIdx.x;
#pragma unroll
  for (int k = 0; k < 4; k++) sh[256 * k + t] = v[k];
  __syncthreads();
  for (int w = blockDim.x >> 1; w > 0; w >>= 1) {
    if (t < w) {
#pragma unroll
      for (int k = 0; k < 4; k++) sh[256 * k + t] += sh[256 * k + t + w];
    }
    __syncthreads();
  }
  if (t == 0)
#pragma unroll
    for (int k = 0; k < 4; k++) out[k] = sh[256 * k];
}
__device__ __forceinline__ void block_sum4(const double* v, double* out) {
  __shared__ double sh[4 * 256];
  block_sum4_in(v, out, sh);
}

// Per-thread sums of the squared increments |U - U0|^2 (the RMS(dU)
// partials).  Mixed precision and double-float: summed as unevaluated pairs
// hi + lo of FP32 numbers (about 48 significant bits, all terms
// non-negative) on the FP32 pipe; mixed adds FP32 squares by TwoSum,
// double-float adds the double-float squares of its increments.  GB300's FP64
// pipe does 2 lane operations per clock and SM: FP64 sums of 4 squares per
// cell and a shared-memory FP64 tree per block made the last stage's mixed
// update kernel 2.8x as long as the others (65 against 23 us at 1,048,576
// cells).  The FP64 builds keep FP64 sums.
#if FVS_MIXED || FVS_DF
// (h, l) += (h2, l2) for non-negative pairs: TwoSum of the high parts, the
// low parts added to its error, renormalised (Fast2Sum)
__device__ __forceinline__ void pair_add(float& h, float& l, float h2, float l2) {
  const float s = h + h2, bp = s - h;
  const float e = ((h - (s - bp)) + (h2 - bp)) + (l + l2);
  h = s + e;
  l = e - (h - s);
}
struct NormAcc {
  float h[4] = {0.f, 0.f, 0.f, 0.f}, l[4] = {0.f, 0.f, 0.f, 0.f};
#if FVS_MIXED
  __device__ __forceinline__ void add(int v, float x) { two_sum(h[v], l[v], x); }
#else
  __device__ __forceinline__ void add(int v, df64 x) { pair_add(h[v], l[v], x.hi, x.lo); }
#endif
  __device__ __forceinline__ void to_double(double* o) const {
#pragma unroll
    for (int v = 0; v < 4; v++) o[v] = f2d_bits(h[v]) + f2d_bits(l[v]);
  }
};
// the block's sums per component into thread 0's a, in a fixed order (lanes
// by shuffle-down, then the warps in index order); sh: 32 x 4 float2
__device__ __forceinline__ void block_pairs4(NormAcc& a, float2* sh) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = (blockDim.x + 31) >> 5;
#pragma unroll
  for (int v = 0; v < 4; v++)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const float h2 = __shfl_down_sync(0xffffffffu, a.h[v], o), l2 = __shfl_down_sync(0xffffffffu, a.l[v], o);
      pair_add(a.h[v], a.l[v], h2, l2);
    }
  if (lane == 0)
#pragma unroll
    for (int v = 0; v < 4; v++) sh[4 * w + v] = make_float2(a.h[v], a.l[v]);
  __syncthreads();
  if (w == 0) {
#pragma unroll
    for (int v = 0; v < 4; v++) {
      const float2 p = lane < nw ? sh[4 * lane + v] : make_float2(0.f, 0.f);
      a.h[v] = p.x;
      a.l[v] = p.y;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) {
        const float h2 = __shfl_down_sync(0xffffffffu, a.h[v], o), l2 = __shfl_down_sync(0xffffffffu, a.l[v], o);
        pair_add(a.h[v], a.l[v], h2, l2);
      }
    }
  }
  __syncthreads();
}
#define FVS_NORM_SH_BYTES (32 * 4 * 8)
#else
struct NormAcc {
  double s[4] = {0.0, 0.0, 0.0, 0.0};
  __device__ __forceinline__ void add(int v, double x) { s[v] += x; }
  __device__ __forceinline__ void to_double(double* o) const {
#pragma unroll
    for (int v = 0; v < 4; v++) o[v] = s[v];
  }
};
#define FVS_NORM_SH_BYTES (4 * 256 * 8)
#endif

#if FVS_MIXED
// Mixed precision: the slot sums are exact (TwoSum) and the state stays FP64,
// but the RK increment h (c R + F) is formed in FP32 (relative error 2^-24
// of the increment, below the FP32 flux rounding already in R) and added to
// the FP64 state: 4-8 FP64 additions per cell and stage instead of ~30 FP64
// operations.  The accumulator F is stored as FP32 (float4 per cell).
// The flux records of a cell's faces summed in its gather order: sl holds
// four signed references (+-(record + 1), 0: none), get(idx, f, w) loads
// record idx (w only when want_ws).  Shared by the update kernel (records in
// global memory) and the fused tile stage (records in shared memory).
template <class Get>
__device__ __forceinline__ void residual_from_faces_f(const int* sl, float rv, bool want_ws, Get get, float* res,
                                                      float& ws) {
  float hi[4] = {0.f, 0.f, 0.f, 0.f}, lo[4] = {0.f, 0.f, 0.f, 0.f}, wh = 0.f, wl = 0.f;
#pragma unroll
  for (int j = 0; j < 4; j++) {
    const int s = sl[j];
    if (s == 0) continue;
    const int idx = (s > 0 ? s : -s) - 1;
    float f[4], w = 0.f;
    get(idx, f, w);
#pragma unroll
    for (int v = 0; v < 4; v++) two_sum(hi[v], lo[v], s > 0 ? f[v] : -f[v]);
    if (want_ws) two_sum(wh, wl, w);
  }
#pragma unroll
  for (int v = 0; v < 4; v++) res[v] = (hi[v] + lo[v]) * rv;
  ws = wh + wl;
}

__device__ __forceinline__ void cell_residual_f(const DevView& d, int ic, bool want_ws, float* res, float& ws) {
  const int4 cf = d.cflist[ic];
  const int sl[4] = {cf.x, cf.y, cf.z, cf.w};
  const float rv = -static_cast<const float*>(d.volT)[ic];
  residual_from_faces_f(sl, rv, want_ws, [&](int idx, float* f, float& w) {
    ldc4<true>(static_cast<const float*>(d.eflux), idx, f);
    if (want_ws) w = ldc1<true>(static_cast<const float*>(d.ews), idx);
  }, res, ws);
}

// the RK stage of one cell from its residual res (and, at a steady first
// stage, its wave-speed sum ws); the new primitives go to Pout.
// The FP64 state U stays the state at the start of the step until the last
// stage writes the new one: each stage's state is U plus an FP32 increment
// (the form above), so an intermediate stage needs only U and, carried in
// the FP32 accumulator F, the accumulated residuals (SSP-RK(4,2), RK) or the
// previous increment (SSP-RK3).  Per cell and SSP-RK3 step that is 192 bytes
// of state traffic instead of 288 for writing U (and U0) at every stage.
template <int MODE, bool COH, class Store>
__device__ __forceinline__ void apply_stage_fs(const DevView& d, const StageParams& sp, int ic, const float* res,
                                               float ws, Store store, NormAcc& na) {
  float h = float(sp.h);
  if (sp.steady) {
    float dtl;
    if (sp.stage == 1) {  // compute_local_time, src/runge_kutta.f90:424-437
      dtl = float(d.cfl) / (static_cast<const float*>(d.volT)[ic] * (0.5f * ws));
      d.dtl[ic] = f2d_bits(dtl);
    } else {
      dtl = d2f_bits(ldc1<COH>(d.dtl, ic));
    }
    h = dtl * float(sp.cst);
  }
  float* F = reinterpret_cast<float*>(d.F);
  double u0[4], u[4];
  float f[4], inc[4];
  ldc4<COH>(d.U, ic, u0);  // the state at the start of the step
  if (sp.stage == 1) {
#pragma unroll
    for (int v = 0; v < 4; v++) f[v] = 0.f;
  } else {
    ldc4<COH>(F, ic, f);
  }
  const float coef = float(sp.coef);
  if (MODE == MODE_SSP42) {
    // src/runge_kutta.f90:225-226 / :383-387
#pragma unroll
    for (int v = 0; v < 4; v++) {
      inc[v] = h * (coef * res[v] + f[v]);
      f[v] = f[v] + res[v];
      u[v] = u0[v] + f2d_bits(inc[v]);
    }
    if (!sp.last) st4(F, ic, f);
  } else if (MODE == MODE_RK) {
    // src/runge_kutta.f90:156-162 / :302-313
#pragma unroll
    for (int v = 0; v < 4; v++) {
      f[v] = f[v] + coef * res[v];
      inc[v] = sp.last ? h * f[v] : h * res[v];
      u[v] = u0[v] + f2d_bits(inc[v]);
    }
    if (!sp.last) st4(F, ic, f);
  } else {
    // SSP-RK3 (Shu-Osher): u = a u0 + b (cur + h R) = u0 + b ((cur - u0) + h R)
    if (sp.stage == 1) {
#pragma unroll
      for (int v = 0; v < 4; v++) {
        inc[v] = h * res[v];
        u[v] = u0[v] + f2d_bits(inc[v]);
      }
    } else {
      // f: the previous stage's increment, its state minus u0
      const float b = float(sp.b);
#pragma unroll
      for (int v = 0; v < 4; v++) {
        inc[v] = b * (f[v] + h * res[v]);
        u[v] = u0[v] + f2d_bits(inc[v]);
      }
    }
    if (!sp.last) st4(F, ic, inc);
  }
  if (sp.last) st4(d.U, ic, u);
  float p[4];
  cons2prim(TP(gm1), u, p);
  store(p);
  if (sp.last) {
#pragma unroll
    for (int v = 0; v < 4; v++) na.add(v, inc[v] * inc[v]);
  }
}

// ... with the new primitives stored at Pout[ic]
template <int MODE, bool COH>
__device__ __forceinline__ void apply_stage_f(const DevView& d, const StageParams& sp, int ic, const float* res,
                                              float ws, float* Pout, NormAcc& na) {
  apply_stage_fs<MODE, COH>(d, sp, ic, res, ws, [&](const float* p) { st4(Pout, ic, p); }, na);
}

template <int MODE, bool COH>
__device__ __forceinline__ void update_item(const DevView& d, const StageParams& sp, int ic, NormAcc& na) {
  float res[4], ws;
  cell_residual_f(d, ic, sp.steady && sp.stage == 1, res, ws);
  apply_stage_f<MODE, COH>(d, sp, ic, res, ws, static_cast<float*>(d.Pv), na);
}

#else
// the RK stage of one cell from its residual res (and, at a steady first
// stage, its wave-speed sum ws); the new primitives go to Pout; at the last
// stage adds |U-U0|^2 to na
// RAW (FP64 build): res holds the flux sums and rv = -1/vol; SSP-RK3 folds
// rv into the step (h rv, one product per cell instead of four), the other
// schemes scale res first.
template <int MODE, bool COH, bool RAW = false>
__device__ __forceinline__ void apply_stage_d(const DevView& d, const StageParams& sp, int ic, const double* res_in,
                                              double ws, T* Pout, NormAcc& na, double rv = 1.0) {
  double res[4];
#pragma unroll
  for (int v = 0; v < 4; v++) res[v] = (RAW && MODE != MODE_SSP3) ? res_in[v] * rv : res_in[v];
  {
    double h = sp.h;
    if (sp.steady) {
      double dtl;
      if (sp.stage == 1) {  // compute_local_time, src/runge_kutta.f90:424-437
        dtl = d.cfl * d.vol[ic] / (0.5 * ws);
        d.dtl[ic] = dtl;
      } else {
        dtl = ldc1<COH>(d.dtl, ic);
      }
      h = dtl * sp.cst;
    }
    double u0[4], u[4], f[4];
    if (sp.stage == 1) {
      ldc4<COH>(d.U, ic, u0);
      st4(d.U0, ic, u0);
#pragma unroll
      for (int v = 0; v < 4; v++) f[v] = 0.0;
    } else {
      ldc4<COH>(d.U0, ic, u0);
      if (MODE != MODE_SSP3) ldc4<COH>(d.F, ic, f);
    }
    if (MODE == MODE_SSP42) {
      // src/runge_kutta.f90:225-226 / :383-387
#pragma unroll
      for (int v = 0; v < 4; v++) {
        u[v] = u0[v] + h * (sp.coef * res[v] + f[v]);
        f[v] = f[v] + res[v];
      }
      if (!sp.last) st4(d.F, ic, f);
    } else if (MODE == MODE_RK) {
      // src/runge_kutta.f90:156-162 / :302-313
#pragma unroll
      for (int v = 0; v < 4; v++) {
        f[v] = f[v] + sp.coef * res[v];
        u[v] = sp.last ? u0[v] + h * f[v] : u0[v] + h * res[v];
      }
      if (!sp.last) st4(d.F, ic, f);
    } else {
      // SSP-RK3 (Shu-Osher), extension
      double cur[4];
      if (sp.stage == 1) {
#pragma unroll
        for (int v = 0; v < 4; v++) cur[v] = u0[v];
      } else {
        ldc4<COH>(d.U, ic, cur);
      }
      const double hs = RAW ? h * rv : h;
#pragma unroll
      for (int v = 0; v < 4; v++) {
        const double s = cur[v] + hs * res[v];
        u[v] = sp.stage == 1 ? s : sp.a * u0[v] + sp.b * s;
      }
    }
    st4(d.U, ic, u);
    T p[4];
    cons2prim(TP(gm1), u, p);
    st4(Pout, ic, p);
    if (sp.last) {
#pragma unroll
      for (int v = 0; v < 4; v++) {
        const double dd = fabs(u[v] - u0[v]);
        na.add(v, dd * dd);
      }
    }
  }
}

#if FVS_DF
// The RK stage of one cell in double-float arithmetic (the double-float
// build): the residual arrives as df64, the state is read as FP64 and split
// exactly on the integer pipe (df_from_double), the stage is formed in df64
// on the FP32 pipe (relative error ~2^-48 per operation, against 2^-53 in
// FP64), and the new state is written as FP64 (one exact addition per
// component).  The accumulator F holds df64 pairs in the same 8 bytes per
// component; U0 stays FP64.  The same formulas and order as apply_stage_d:
// src/runge_kutta.f90:225-226 / :383-387 (SSP-RK(4,2)), :156-162 / :302-313
// (RK), and the SSP-RK3 extension.  Per cell and stage the FP64 pipe is left
// with the four additions of the state store.
template <int MODE, bool COH>
__device__ __forceinline__ void apply_stage_df(const DevView& d, const StageParams& sp, int ic, const df64* res,
                                               double ws, T* Pout, NormAcc& na) {
  df64 h(sp.hp[0], sp.hp[1]);
  if (sp.steady) {
    double dtl;
    if (sp.stage == 1) {  // compute_local_time, src/runge_kutta.f90:424-437
      dtl = d.cfl * d.vol[ic] / (0.5 * ws);
      d.dtl[ic] = dtl;
    } else {
      dtl = ldc1<COH>(d.dtl, ic);
    }
    h = df_from_double(dtl) * df64(sp.cstp[0], sp.cstp[1]);
  }
  double ud[4];
  df64 u0[4], u[4], f[4];
  df64* F = reinterpret_cast<df64*>(d.F);
  if (sp.stage == 1) {
    ldc4<COH>(d.U, ic, ud);
    st4(d.U0, ic, ud);
#pragma unroll
    for (int v = 0; v < 4; v++) f[v] = df64(0.f, 0.f);
  } else {
    ldc4<COH>(d.U0, ic, ud);
    if (MODE != MODE_SSP3) ldc4<COH>(F, ic, f);
  }
#pragma unroll
  for (int v = 0; v < 4; v++) u0[v] = df_from_double(ud[v]);
  const df64 c(sp.coefp[0], sp.coefp[1]);
  if (MODE == MODE_SSP42) {
#pragma unroll
    for (int v = 0; v < 4; v++) {
      u[v] = dfma(h, dfma(c, res[v], f[v]), u0[v]);
      f[v] = f[v] + res[v];
    }
    if (!sp.last) st4(F, ic, f);
  } else if (MODE == MODE_RK) {
#pragma unroll
    for (int v = 0; v < 4; v++) {
      f[v] = dfma(c, res[v], f[v]);
      u[v] = dfma(h, sp.last ? f[v] : res[v], u0[v]);
    }
    if (!sp.last) st4(F, ic, f);
  } else {
    df64 cur[4];
    if (sp.stage == 1) {
#pragma unroll
      for (int v = 0; v < 4; v++) cur[v] = u0[v];
    } else {
      double cd[4];
      ldc4<COH>(d.U, ic, cd);
#pragma unroll
      for (int v = 0; v < 4; v++) cur[v] = df_from_double(cd[v]);
    }
    const df64 a(sp.ap[0], sp.ap[1]), b(sp.bp[0], sp.bp[1]);
#pragma unroll
    for (int v = 0; v < 4; v++) {
      const df64 st = dfma(h, res[v], cur[v]);
      u[v] = sp.stage == 1 ? st : dfma(b, st, a * u0[v]);
    }
  }
  // the stored state is exactly the df64 value (48 significant bits)
  double uo[4];
#pragma unroll
  for (int v = 0; v < 4; v++) uo[v] = to_double(u[v]);
  st4(d.U, ic, uo);
  T p[4];
  cons2prim_df(TP(gm1), u, p);
  st4(Pout, ic, p);
  if (sp.last) {
#pragma unroll
    for (int v = 0; v < 4; v++) {
      const df64 dd = u[v] - u0[v];
      na.add(v, dd * dd);
    }
  }
}

// one cell of an RK stage; at the last stage adds |U-U0|^2 to na
template <int MODE, bool COH>
__device__ __forceinline__ void update_item(const DevView& d, const StageParams& sp, int ic, NormAcc& na) {
  df64 res[4];
  double ws;
  if (sp.steady && sp.stage == 1) cell_residual_df<true, COH>(d, ic, res, ws);
  else cell_residual_df<false, COH>(d, ic, res, ws);
  apply_stage_df<MODE, COH>(d, sp, ic, res, ws, static_cast<T*>(d.Pv), na);
}
#else
// one cell of an RK stage; at the last stage adds |U-U0|^2 to na
template <int MODE, bool COH>
__device__ __forceinline__ void update_item(const DevView& d, const StageParams& sp, int ic, NormAcc& na) {
  double res[4], ws;
#if FVS_STRICT
  if (sp.steady && sp.stage == 1) cell_residual<true, COH>(d, ic, res, ws);
  else cell_residual<false, COH>(d, ic, res, ws);
  apply_stage_d<MODE, COH>(d, sp, ic, res, ws, static_cast<T*>(d.Pv), na);
#else
  if (sp.steady && sp.stage == 1) cell_flux_sum<true, COH>(d, ic, res, ws);
  else cell_flux_sum<false, COH>(d, ic, res, ws);
  apply_stage_d<MODE, COH, true>(d, sp, ic, res, ws, static_cast<T*>(d.Pv), na, -d.rvol[ic]);
#endif
}
#endif

#endif  // FVS_MIXED

// RMS of |U - U0| per component from the block partials, by one block in a
// fixed order (deterministic); advances the step counter.  sh: the shared
// memory of the block sums (FVS_NORM_SH_BYTES)
__device__ __forceinline__ void norm_final_block(const DevView& d, void* sh) {
  double out[4];
#if FVS_MIXED || FVS_DF
  NormAcc a;
  const float2* P = reinterpret_cast<const float2*>(d.partials);
#pragma unroll 4
  for (int i = threadIdx.x; i < d.nblk_red; i += blockDim.x)
#pragma unroll
    for (int k = 0; k < 4; k++) {
      const float2 q = __ldcg(P + 4 * (size_t)i + k);
      pair_add(a.h[k], a.l[k], q.x, q.y);
    }
  block_pairs4(a, static_cast<float2*>(sh));
  a.to_double(out);
#else
  double s[4] = {0.0, 0.0, 0.0, 0.0};
  for (int i = threadIdx.x; i < d.nblk_red; i += blockDim.x)
#pragma unroll
    for (int k = 0; k < 4; k++) s[k] += __ldcg(d.partials + 4 * i + k);
  block_sum4_in(s, out, static_cast<double*>(sh));
#endif
  if (threadIdx.x == 0) {
    const int istep = d.stepctl[0] + 1;
    double* o = d.norms + 4 * (size_t)((istep - 1) % d.norm_cap);
#pragma unroll
    for (int k = 0; k < 4; k++) o[k] = sqrt(out[k] / double(d.nc));
    d.stepctl[0] = istep;
  }
}

// the block's sum of na into partials[blockIdx.x] (mixed precision and
// double-float: four FP32 pairs in the same 32 bytes); the block that finishes last
// (d.nblk_red == gridDim.x) reduces all partials into the step's norms;
// sh: FVS_NORM_SH_BYTES of shared memory
__device__ __forceinline__ void stage_norms(const DevView& d, NormAcc& na, void* sh) {
  __shared__ int s_last;
#if FVS_MIXED || FVS_DF
  block_pairs4(na, static_cast<float2*>(sh));
  if (threadIdx.x == 0) {
    float2* P = reinterpret_cast<float2*>(d.partials) + 4 * (size_t)blockIdx.x;
#pragma unroll
    for (int k = 0; k < 4; k++) P[k] = make_float2(na.h[k], na.l[k]);
#else
  double out[4];
  block_sum4_in(na.s, out, static_cast<double*>(sh));
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < 4; k++) d.partials[4 * blockIdx.x + k] = out[k];
#endif
    __threadfence();
    s_last = atomicAdd(&d.stepctl[1], 1) == (int)gridDim.x - 1;
  }
  __syncthreads();
  if (s_last) {
    __threadfence();
    norm_final_block(d, sh);
    if (threadIdx.x == 0) d.stepctl[1] = 0;
  }
}

// One RK stage over all cells.  At the last stage every block writes its
// partial norms; the block that finishes last (a counter in stepctl[1])
// reduces them, so no separate norm launch is needed.
// STRIDE: one wave of resident blocks strides over the cells (the last
// stage's launch); otherwise one cell per thread.
template <int MODE, bool STRIDE>
__global__ void __launch_bounds__(256) k_update(const DevView d, const StageParams sp) {
  pdl_wait();
  pdl_trigger();
  NormAcc na;
  if (STRIDE) {
    for (int ic = blockIdx.x * blockDim.x + threadIdx.x; ic < d.nc; ic += gridDim.x * blockDim.x)
      update_item<MODE, false>(d, sp, ic, na);
  } else {
    const int ic = blockIdx.x * blockDim.x + threadIdx.x;
    if (ic < d.nc) update_item<MODE, false>(d, sp, ic, na);
  }
  __shared__ __align__(16) unsigned char sh[FVS_NORM_SH_BYTES];
  if (sp.last) stage_norms(d, na, sh);
}

#if FVS_MIXED || FVS_DF
// ---------------------------------------------------------------------------
// fused RK stage: one block per tile (fvs_tiles.hpp)
// ---------------------------------------------------------------------------
// Shared memory of a tile block: primitives of the tile, halo1 and halo2
// (lmax x 4), gradients and limiter values of the tile and halo1 (gmax x 9),
// and the flux * area and ws * area of the tile's faces (fmax x 5).
static size_t tile_smem_bytes(int lmax, int gmax, int fmax) {
  const size_t b = sizeof(T) * (4 * (size_t)lmax + 9 * (size_t)gmax + 5 * (size_t)fmax);
  return b > 4 * 256 * sizeof(double) ? b : 4 * 256 * sizeof(double);
}

// One RK stage of one tile in four phases separated by block barriers:
//  1. primitives of the tile and its halos from global memory (buffer kin)
//  2. gradient (and limiter) of every tile and halo1 cell from shared memory
//     (gradient_core, the separate gradient kernel's arithmetic)
//  3. face states and Roe flux of every face of the tile (face_states,
//     flux_eval: the edge-flux kernel's arithmetic)
//  4. per tile cell the face fluxes summed in the cell's gather order
//     (the update kernel's order and arithmetic), the RK update of the
//     conservative state, the new primitives into buffer kout and, at the
//     last stage, the norm partials
// Gradients and face fluxes never leave the chip.  A cut face (cells in two
// tiles) is evaluated by both tiles with the same operands and the same
// instructions, so both cells receive the same flux.  Results are
// bit-identical to the separate gradient, flux and update kernels.
template <int MODE, int REC, int LIM>
__global__ void __launch_bounds__(256, FVS_MIXED ? 5 : 2) k_tile_stage(const DevView d, const TileView tv, const StageParams sp, int kin,
                                                   int kout) {
  pdl_wait();
  pdl_trigger();
  extern __shared__ __align__(16) unsigned char tile_shm[];
  const int t = blockIdx.x, tid = threadIdx.x, nthr = blockDim.x;
  const int b = tv.c0[t], n = tv.c0[t + 1] - b;
  const int hb = tv.h0[t], nl = n + (tv.h0[t + 1] - hb), ng = n + tv.nh1[t];
  T* sP = reinterpret_cast<T*>(tile_shm);
  T* sGx = sP + 4 * (size_t)tv.lmax;
  T* sGy = sGx + 4 * (size_t)tv.gmax;
  T* sPh = sGy + 4 * (size_t)tv.gmax;
  T* sF = sPh + tv.gmax;
  const T* Pin = static_cast<const T*>(tv.Pbuf[kin]);
  T* Pout = static_cast<T*>(tv.Pbuf[kout]);
  // 1. primitives, two cells per pass (both loads in flight together)
  for (int i0 = tid; i0 < nl; i0 += 2 * nthr) {
    const int i1 = i0 + nthr;
    const int g0 = i0 < n ? b + i0 : tv.halo[hb + i0 - n];
    const int g1 = i1 < n ? b + i1 : (i1 < nl ? tv.halo[hb + i1 - n] : g0);
    T v0[4], v1[4];
    ld4(Pin, g0, v0);
    ld4(Pin, g1, v1);
#pragma unroll
    for (int v = 0; v < 4; v++) sP[4 * i0 + v] = v0[v];
    if (i1 < nl)
#pragma unroll
      for (int v = 0; v < 4; v++) sP[4 * i1 + v] = v1[v];
  }
  __syncthreads();
  // 2. gradients of the tile and halo1 cells; each cell's record holds its
  //    device index and the start of its global stencil entries
  if (REC != REC_FIRST) {
    const uint16_t* lst = tv.lst + tv.s0[t];
    const int* lsp = tv.lsp + tv.g0[t];
    const int2* gcr = tv.gcell + tv.g0[t];
    for (int i = tid; i < ng; i += nthr) {
      const int2 gc = gcr[i];
      const int gid = gc.x, kb = gc.y;
      const uint16_t* L = lst + lsp[i];
      auto load = [&](int k, T* pj) {
        const T* q = sP + 4 * (int)L[k - kb];
#pragma unroll
        for (int v = 0; v < 4; v++) pj[v] = q[v];
      };
      T gx[4], gy[4], ph = T(1);
      if (d.grad_method == FVS_GRAD_LSQ) gradient_core<FVS_GRAD_LSQ, LIM>(d, gid, sP + 4 * i, load, gx, gy, ph);
      else if (d.grad_method == FVS_GRAD_GGCB) gradient_core<FVS_GRAD_GGCB, 0>(d, gid, sP + 4 * i, load, gx, gy, ph);
      else gradient_core<FVS_GRAD_GGNB, 0>(d, gid, sP + 4 * i, load, gx, gy, ph);
#pragma unroll
      for (int v = 0; v < 4; v++) {
        sGx[4 * i + v] = gx[v];
        sGy[4 * i + v] = gy[v];
      }
      if (REC == REC_GENERAL) sPh[i] = LIM ? ph : static_cast<const T*>(d.phi)[gid];
    }
    __syncthreads();
  }
  // 3. face fluxes
  const double time = d.tctl[1] + sp.dts;
  const int fb = tv.f0[t], nf = tv.f0[t + 1] - fb;
  const T* fg = static_cast<const T*>(tv.fgeo) + 8 * (size_t)fb;
  for (int f = tid; f < nf; f += nthr) {
    // the face's record: normal, length, the two centre-to-face offsets
    // (coalesced: the tile's faces are stored one after the other)
    const uint32_t lr = tv.flr[fb + f];
    T g[8];
    ld4(fg, 2 * f, g);
    ld4(fg, 2 * f + 1, g + 4);
    const int l = (int)(lr & 0xFFFFu), rr = (int)(lr >> 16);
    const bool interior = rr != 0xFFFF;
    const int r = interior ? rr : l;  // a boundary slot reads no right cell
    const int e = interior ? -1 : tv.face[fb + f];  // the slot's boundary record
    const T2 nn = {g[0], g[1]};
    const T af = g[2];
    const T2 dl = {g[3], g[4]}, dr = {g[5], g[6]};
    T pfL[4], pfR[4], flux[4], wsa;
    const T phiL = REC == REC_GENERAL ? sPh[l] : T(1), phiR = REC == REC_GENERAL ? sPh[r] : T(1);
    face_states<REC>(d, e, interior, time, nn, dl, dr, sP + 4 * l, sGx + 4 * l, sGy + 4 * l, phiL, sP + 4 * r,
                     sGx + 4 * r, sGy + 4 * r, phiR, pfL, pfR);
    flux_eval(d, pfL, pfR, nn, af, flux, wsa);
#pragma unroll
    for (int v = 0; v < 4; v++) sF[5 * f + v] = flux[v];
    sF[5 * f + 4] = wsa;
  }
  __syncthreads();
  // 4. gather and RK update of the tile's cells
  NormAcc na;
  const bool want_ws = sp.steady && sp.stage == 1;
  for (int i = tid; i < n; i += nthr) {
    const int gid = b + i;
    const int2 q = tv.lcf[gid];
    const int sl[4] = {(int)(int16_t)(q.x & 0xFFFF), (int)(int16_t)((unsigned)q.x >> 16),
                       (int)(int16_t)(q.y & 0xFFFF), (int)(int16_t)((unsigned)q.y >> 16)};
    auto get = [&](int idx, T* f, T& w) {
#pragma unroll
      for (int v = 0; v < 4; v++) f[v] = sF[5 * idx + v];
      w = sF[5 * idx + 4];
    };
#if FVS_MIXED
    float res[4], ws;
    residual_from_faces_f(sl, -static_cast<const float*>(d.volT)[gid], want_ws, get, res, ws);
    apply_stage_f<MODE, false>(d, sp, gid, res, ws, Pout, na);
#else
    df64 res[4];
    double ws;
    const df64 rv = -static_cast<const df64*>(d.volT)[gid];
    if (want_ws) residual_from_faces_df<true>(sl, rv, get, res, ws);
    else residual_from_faces_df<false>(sl, rv, get, res, ws);
    apply_stage_df<MODE, false>(d, sp, gid, res, ws, Pout, na);
#endif
  }
  // the norm reduction reuses the primitives' shared memory, unused in
  // phase 4 (at least 4 x 256 doubles: tile_smem_bytes)
  if (sp.last) stage_norms(d, na, tile_shm);
}

template <int MODE, int REC, int LIM>
static cudaError_t launch_tile_t(const DevView& d, const TileView& tv, const StageParams& sp, int k, cudaStream_t s) {
  launch_k(k_tile_stage<MODE, REC, LIM>, (unsigned)tv.ntiles, 256, tv.smem_bytes, s, d, tv, sp, k % tv.nbuf,
           (k + 1) % tv.nbuf);
  return cudaGetLastError();
}

template <int MODE>
static cudaError_t launch_tile_mode(const DevView& d, const TileView& tv, const StageParams& sp, int k,
                                    cudaStream_t s) {
  const bool spec = d.khalf == 0.0 && d.omk == 1.0 && d.limiter == FVS_LIM_NONE;
  if (d.first_order) return launch_tile_t<MODE, REC_FIRST, 0>(d, tv, sp, k, s);
  if (spec) return launch_tile_t<MODE, REC_SPEC, 0>(d, tv, sp, k, s);
  if (d.limiter != FVS_LIM_NONE) return launch_tile_t<MODE, REC_GENERAL, 1>(d, tv, sp, k, s);
  return launch_tile_t<MODE, REC_GENERAL, 0>(d, tv, sp, k, s);
}

static cudaError_t launch_tile_stage(const DevView& d, const TileView& tv, const StageParams& sp, int k,
                                     cudaStream_t s) {
  if (sp.mode == MODE_SSP42) return launch_tile_mode<MODE_SSP42>(d, tv, sp, k, s);
  if (sp.mode == MODE_SSP3) return launch_tile_mode<MODE_SSP3>(d, tv, sp, k, s);
  return launch_tile_mode<MODE_RK>(d, tv, sp, k, s);
}

// ---------------------------------------------------------------------------
// face flux + update per tile (gradients from the separate gradient kernel)
// ---------------------------------------------------------------------------
// One block per tile: the fluxes of every face of the tile (the edge-flux
// kernel's loads from global memory and its arithmetic) into shared memory,
// then the tile's cells summed in their gather order and updated (the update
// kernel's arithmetic).  The flux records never go through global memory, a
// stage has two launches instead of three, and shared memory holds only the
// fluxes, so occupancy stays that of the separate kernels.  The primitives
// alternate between buffers (a block's new values must not reach a
// neighbouring tile that still reads the old ones for a cut face).
// Bit-identical to the separate flux and update kernels.
static size_t tile_fu_smem_bytes(int fmax) {
  const size_t b = 5 * sizeof(T) * (size_t)fmax;
  return b > 4 * 256 * sizeof(double) ? b : 4 * 256 * sizeof(double);
}

template <int MODE, int REC>
__global__ void __launch_bounds__(256) k_tile_flux_update(const DevView d, const TileView tv, const StageParams sp,
                                                         int kout) {
  pdl_wait();
  pdl_trigger();
  extern __shared__ __align__(16) unsigned char tile_shm[];
  T* sF = reinterpret_cast<T*>(tile_shm);
  const int t = blockIdx.x, tid = threadIdx.x, nthr = blockDim.x;
  const int b = tv.c0[t], n = tv.c0[t + 1] - b;
  T* Pout = static_cast<T*>(tv.Pbuf[kout]);
  const double time = d.tctl[1] + sp.dts;
  const int fb = tv.f0[t], nf = tv.f0[t + 1] - fb;
  for (int f = tid; f < nf; f += nthr) {
    T flux[4], wsa;
    flux_compute<REC, false>(d, tv.face[fb + f], time, flux, wsa);
#pragma unroll
    for (int v = 0; v < 4; v++) sF[5 * f + v] = flux[v];
    sF[5 * f + 4] = wsa;
  }
  __syncthreads();
  NormAcc na;
  const bool want_ws = sp.steady && sp.stage == 1;
  for (int i = tid; i < n; i += nthr) {
    const int gid = b + i;
    const int2 q = tv.lcf[gid];
    const int sl[4] = {(int)(int16_t)(q.x & 0xFFFF), (int)(int16_t)((unsigned)q.x >> 16),
                       (int)(int16_t)(q.y & 0xFFFF), (int)(int16_t)((unsigned)q.y >> 16)};
    auto get = [&](int idx, T* f, T& w) {
#pragma unroll
      for (int v = 0; v < 4; v++) f[v] = sF[5 * idx + v];
      w = sF[5 * idx + 4];
    };
#if FVS_MIXED
    float res[4], ws;
    residual_from_faces_f(sl, -static_cast<const float*>(d.volT)[gid], want_ws, get, res, ws);
    apply_stage_f<MODE, false>(d, sp, gid, res, ws, Pout, na);
#else
    df64 res[4];
    double ws;
    const df64 rv = -static_cast<const df64*>(d.volT)[gid];
    if (want_ws) residual_from_faces_df<true>(sl, rv, get, res, ws);
    else residual_from_faces_df<false>(sl, rv, get, res, ws);
    apply_stage_df<MODE, false>(d, sp, gid, res, ws, Pout, na);
#endif
  }
  if (sp.last) {
    __syncthreads();  // the norm buffer reuses the flux records
    stage_norms(d, na, tile_shm);
  }
}

template <int MODE>
static cudaError_t launch_tile_fu_mode(const DevView& d, const TileView& tv, const StageParams& sp, int k,
                                       cudaStream_t s) {
  const bool spec = d.khalf == 0.0 && d.omk == 1.0 && d.limiter == FVS_LIM_NONE;
  const unsigned g = (unsigned)tv.ntiles;
  const size_t sm = tile_fu_smem_bytes(tv.fmax);
  const int ko = (k + 1) % tv.nbuf;
  if (d.first_order) launch_k(k_tile_flux_update<MODE, REC_FIRST>, g, 256, sm, s, d, tv, sp, ko);
  else if (spec) launch_k(k_tile_flux_update<MODE, REC_SPEC>, g, 256, sm, s, d, tv, sp, ko);
  else launch_k(k_tile_flux_update<MODE, REC_GENERAL>, g, 256, sm, s, d, tv, sp, ko);
  return cudaGetLastError();
}

// the tile flux+update of stage k; d.Pv must be the stage's input buffer
// Pbuf[k % nbuf] (the gradient kernel, launched before it, reads the same)
static cudaError_t launch_tile_fu_stage(const DevView& d, const TileView& tv, const StageParams& sp, int k,
                                        cudaStream_t s) {
  if (sp.mode == MODE_SSP42) return launch_tile_fu_mode<MODE_SSP42>(d, tv, sp, k, s);
  if (sp.mode == MODE_SSP3) return launch_tile_fu_mode<MODE_SSP3>(d, tv, sp, k, s);
  return launch_tile_fu_mode<MODE_RK>(d, tv, sp, k, s);
}

#if FVS_MIXED
// ---------------------------------------------------------------------------
// bulk-copy fused stage (FVS2D_TILE_STAGE=3; mixed, LSQ gradients)
// ---------------------------------------------------------------------------
__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// one bulk copy global -> shared, completing on the mbarrier (16-byte
// aligned addresses, a multiple of 16 bytes; checked on the host)
__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, uint32_t bytes, uint32_t mbar) {
  if (bytes == 0) return;
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(
                   smem_addr(dst)),
               "l"(src), "r"(bytes), "r"(mbar)
               : "memory");
}

// bounded wait for phase 0 of the mbarrier; false when the budget ran out
__device__ __forceinline__ bool mbar_wait0(uint32_t mbar, long long budget) {
  const long long t0 = clock64();
  while (true) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\n selp.u32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(mbar)
        : "memory");
    if (done) return true;
    if (clock64() - t0 > budget) return false;
  }
}

// One RK stage of one tile with every input brought in by bulk copies:
//  0. thread 0 arms the block's mbarrier with the byte count and issues one
//     cp.async.bulk per segment (the tile's gather records of buffer kin,
//     face records, coefficients, stencil lists and offsets, face cells,
//     gather lists); every thread waits for them (bounded: after ~0.5 s the
//     block sets dv.err, waits once more for its copies and returns)
//  2.-4. the phases of k_tile_stage, all operands in shared memory, with the
//     same arithmetic (gradient_core_r, face_states, flux_eval, the ordered
//     residual sum, apply_stage_fs); the new primitives of a cell go to every
//     gather record of buffer kout that holds it (home and halos) and, at
//     the last stage, to DevView::Pv
template <int MODE, int REC, int LIM>
__global__ void __launch_bounds__(256) k_tile_dma(const DevView d, const TileView tv, const TileDmaView dv,
                                                 const StageParams sp, int kin, int kout) {
  pdl_wait();
  pdl_trigger();
  extern __shared__ __align__(128) unsigned char dsm[];
  const int t = blockIdx.x, tid = threadIdx.x, nthr = blockDim.x;
  const int b = tv.c0[t], n = tv.c0[t + 1] - b;
  const int hb = tv.h0[t], nl = n + (tv.h0[t + 1] - hb), ng = n + tv.nh1[t];
  const int fb = tv.f0[t], nf = tv.f0[t + 1] - fb;
  float* sP = reinterpret_cast<float*>(dsm + dv.o_P);
  const float* sFg = reinterpret_cast<const float*>(dsm + dv.o_Fg);
  const T2* sC = reinterpret_cast<const T2*>(dsm + dv.o_C);
  const uint16_t* sL = reinterpret_cast<const uint16_t*>(dsm + dv.o_L);
  const uint16_t* sS = reinterpret_cast<const uint16_t*>(dsm + dv.o_S);
  const uint32_t* sR = reinterpret_cast<const uint32_t*>(dsm + dv.o_R);
  const int2* sQ = reinterpret_cast<const int2*>(dsm + dv.o_Q);
  float* sGx = reinterpret_cast<float*>(dsm + dv.o_Gx);
  float* sGy = reinterpret_cast<float*>(dsm + dv.o_Gy);
  float* sPh = reinterpret_cast<float*>(dsm + dv.o_Ph);
  float* sF = reinterpret_cast<float*>(dsm + dv.o_F);
  const uint32_t mbar = smem_addr(dsm);
  const int s0 = dv.sb0[t], ns = dv.sb0[t + 1] - s0;
  const int p0 = dv.pb0[t], np = dv.pb0[t + 1] - p0;
  const int r0 = dv.rb0[t], nr = dv.rb0[t + 1] - r0;
  const int q0 = dv.cb0[t], nq = dv.cb0[t + 1] - q0;
  const int g0 = dv.gb0[t];
  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(mbar) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  __syncthreads();
  if (tid == 0) {
    const uint32_t bytes = (uint32_t)(16 * nl + 32 * nf + 8 * ns + 2 * ns + 2 * np + 4 * nr + 8 * nq);
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(mbar), "r"(bytes) : "memory");
    bulk_g2s(sP, static_cast<const float*>(dv.GB[kin]) + 4 * (size_t)g0, 16u * nl, mbar);
    bulk_g2s((void*)sFg, static_cast<const float*>(tv.fgeo) + 8 * (size_t)fb, 32u * nf, mbar);
    bulk_g2s((void*)sC, static_cast<const T2*>(dv.coef) + s0, 8u * ns, mbar);
    bulk_g2s((void*)sL, dv.lst + s0, 2u * ns, mbar);
    bulk_g2s((void*)sS, dv.lsp + p0, 2u * np, mbar);
    bulk_g2s((void*)sR, dv.flr + r0, 4u * nr, mbar);
    bulk_g2s((void*)sQ, dv.lcf + q0, 8u * nq, mbar);
  }
  if (!mbar_wait0(mbar, 1000000000ll)) {
    // the copies are in flight: wait for them once more before leaving, so
    // that no copy lands in shared memory after the block has exited
    if (tid == 0) atomicExch(dv.err, 1);
    mbar_wait0(mbar, 2000000000ll);
    return;
  }
  // 2. gradients of the tile and halo1 cells (LSQ), from shared memory
  if (REC != REC_FIRST) {
    for (int i = tid; i < ng; i += nthr) {
      const int gid = !LIM ? 0 : (i < n ? b + i : tv.halo[hb + i - n]);  // limiter data by device cell
      auto load = [&](int k, float* pj) {
        const float* q = sP + 4 * (int)sL[k];
#pragma unroll
        for (int v = 0; v < 4; v++) pj[v] = q[v];
      };
      auto coef = [&](int k) { return sC[k]; };
      float gx[4], gy[4], ph = 1.f;
      gradient_core_r<FVS_GRAD_LSQ, LIM>(d, gid, sP + 4 * i, (int)sS[i], (int)sS[i + 1], load, coef, gx, gy, ph);
#pragma unroll
      for (int v = 0; v < 4; v++) {
        sGx[4 * i + v] = gx[v];
        sGy[4 * i + v] = gy[v];
      }
      if (REC == REC_GENERAL) sPh[i] = LIM ? ph : static_cast<const float*>(d.phi)[i < n ? b + i : tv.halo[hb + i - n]];
    }
  }
  __syncthreads();
  // 3. face fluxes
  const double time = d.tctl[1] + sp.dts;
  for (int f = tid; f < nf; f += nthr) {
    const uint32_t lr = sR[f];
    const float* g = sFg + 8 * f;
    const int l = (int)(lr & 0xFFFFu), rr = (int)(lr >> 16);
    const bool interior = rr != 0xFFFF;
    const int r = interior ? rr : l;
    const int e = interior ? -1 : tv.face[fb + f];
    const T2 nn = {g[0], g[1]};
    const float af = g[2];
    const T2 dl = {g[3], g[4]}, dr = {g[5], g[6]};
    float pfL[4], pfR[4], flux[4], wsa;
    const float phiL = REC == REC_GENERAL ? sPh[l] : 1.f, phiR = REC == REC_GENERAL ? sPh[r] : 1.f;
    face_states<REC>(d, e, interior, time, nn, dl, dr, sP + 4 * l, sGx + 4 * l, sGy + 4 * l, phiL, sP + 4 * r,
                     sGx + 4 * r, sGy + 4 * r, phiR, pfL, pfR);
    flux_eval(d, pfL, pfR, nn, af, flux, wsa);
#pragma unroll
    for (int v = 0; v < 4; v++) sF[5 * f + v] = flux[v];
    sF[5 * f + 4] = wsa;
  }
  __syncthreads();
  // 4. gather, RK update, new primitives to every record of the cell
  float* GBo = static_cast<float*>(dv.GB[kout]);
  float* Pv = static_cast<float*>(d.Pv);
  NormAcc na;
  const bool want_ws = sp.steady && sp.stage == 1;
  for (int i = tid; i < n; i += nthr) {
    const int gid = b + i;
    const int2 q = sQ[i];
    const int sl[4] = {(int)(int16_t)(q.x & 0xFFFF), (int)(int16_t)((unsigned)q.x >> 16),
                       (int)(int16_t)(q.y & 0xFFFF), (int)(int16_t)((unsigned)q.y >> 16)};
    auto get = [&](int idx, float* f, float& w) {
#pragma unroll
      for (int v = 0; v < 4; v++) f[v] = sF[5 * idx + v];
      w = sF[5 * idx + 4];
    };
    float res[4], ws;
    residual_from_faces_f(sl, -static_cast<const float*>(d.volT)[gid], want_ws, get, res, ws);
    const int j0 = dv.dptr[gid], j1 = dv.dptr[gid + 1];
    apply_stage_fs<MODE, false>(d, sp, gid, res, ws, [&](const float* p) {
      for (int j = j0; j < j1; j++) st4(GBo, dv.dpos[j], p);
      if (sp.last) st4(Pv, gid, p);
    }, na);
  }
  if (sp.last) {
    __syncthreads();  // the norm buffer reuses the gradient regions
    stage_norms(d, na, dsm + dv.o_Gx);
  }
}

// copies the primitives of every cell into its records of gather buffer buf
__global__ void __launch_bounds__(256) k_dma_fill(const DevView d, const TileDmaView dv, int buf) {
  pdl_wait();
  pdl_trigger();
  const int c = blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= d.nc) return;
  float p[4];
  ld4(static_cast<const float*>(d.Pv), c, p);
  float* G = static_cast<float*>(dv.GB[buf]);
  for (int j = dv.dptr[c]; j < dv.dptr[c + 1]; j++) st4(G, dv.dpos[j], p);
}

template <int MODE>
static cudaError_t launch_tile_dma_mode(const DevView& d, const TileView& tv, const TileDmaView& dv,
                                        const StageParams& sp, int k, cudaStream_t s) {
  const bool spec = d.khalf == 0.0 && d.omk == 1.0 && d.limiter == FVS_LIM_NONE;
  const unsigned g = (unsigned)tv.ntiles;
  const int ki = k % tv.nbuf, ko = (k + 1) % tv.nbuf;
  if (d.first_order) launch_k(k_tile_dma<MODE, REC_FIRST, 0>, g, 256, dv.smem_bytes, s, d, tv, dv, sp, ki, ko);
  else if (spec) launch_k(k_tile_dma<MODE, REC_SPEC, 0>, g, 256, dv.smem_bytes, s, d, tv, dv, sp, ki, ko);
  else if (d.limiter != FVS_LIM_NONE)
    launch_k(k_tile_dma<MODE, REC_GENERAL, 1>, g, 256, dv.smem_bytes, s, d, tv, dv, sp, ki, ko);
  else launch_k(k_tile_dma<MODE, REC_GENERAL, 0>, g, 256, dv.smem_bytes, s, d, tv, dv, sp, ki, ko);
  return cudaGetLastError();
}

static cudaError_t launch_tile_dma_stage(const DevView& d, const TileView& tv, const TileDmaView& dv,
                                         const StageParams& sp, int k, cudaStream_t s) {
  if (sp.mode == MODE_SSP42) return launch_tile_dma_mode<MODE_SSP42>(d, tv, dv, sp, k, s);
  if (sp.mode == MODE_SSP3) return launch_tile_dma_mode<MODE_SSP3>(d, tv, dv, sp, k, s);
  return launch_tile_dma_mode<MODE_RK>(d, tv, dv, sp, k, s);
}

static cudaError_t launch_tile_dma_fill(const DevView& d, const TileDmaView& dv, int buf, cudaStream_t s) {
  launch_k(k_dma_fill, (unsigned)((d.nc + 255) / 256), 256, 0, s, d, dv, buf);
  return cudaGetLastError();
}

// opts the instantiations in to dv.smem_bytes; returns it (0 if a block may
// not have that much)
static size_t tile_dma_smem(const TileView& tv, const TileDmaView& dv) {
  (void)tv;
  int dev = 0, cap = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&cap, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess)
    return 0;
  if (dv.smem_bytes + 64 > (size_t)cap) return 0;
  const int b = (int)dv.smem_bytes;
  bool ok = true;
#define FVS_DMA_ATTR(M, R, L) \
  ok = ok && cudaFuncSetAttribute(k_tile_dma<M, R, L>, cudaFuncAttributeMaxDynamicSharedMemorySize, b) == cudaSuccess
  FVS_DMA_ATTR(MODE_SSP42, REC_FIRST, 0); FVS_DMA_ATTR(MODE_SSP42, REC_SPEC, 0);
  FVS_DMA_ATTR(MODE_SSP42, REC_GENERAL, 0); FVS_DMA_ATTR(MODE_SSP42, REC_GENERAL, 1);
  FVS_DMA_ATTR(MODE_SSP3, REC_FIRST, 0); FVS_DMA_ATTR(MODE_SSP3, REC_SPEC, 0);
  FVS_DMA_ATTR(MODE_SSP3, REC_GENERAL, 0); FVS_DMA_ATTR(MODE_SSP3, REC_GENERAL, 1);
  FVS_DMA_ATTR(MODE_RK, REC_FIRST, 0); FVS_DMA_ATTR(MODE_RK, REC_SPEC, 0);
  FVS_DMA_ATTR(MODE_RK, REC_GENERAL, 0); FVS_DMA_ATTR(MODE_RK, REC_GENERAL, 1);
#undef FVS_DMA_ATTR
  return ok ? dv.smem_bytes : 0;
}
#endif  // FVS_MIXED

// opts every instantiation in to the shared memory of the plan's largest
// tile; returns the bytes of one block (0: more than a block may have)
static size_t tile_smem(int lmax, int gmax, int fmax) {
  const size_t bytes = tile_smem_bytes(lmax, gmax, fmax);
  int dev = 0, cap = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&cap, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess)
    return 0;
  if (bytes + 64 > (size_t)cap) return 0;
  const int b = (int)bytes;
  bool ok = true;
#define FVS_TILE_ATTR(M)                                                                                           \
  ok = ok && cudaFuncSetAttribute(k_tile_stage<M, REC_FIRST, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, b) == \
                 cudaSuccess;                                                                                      \
  ok = ok && cudaFuncSetAttribute(k_tile_stage<M, REC_SPEC, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize, b) ==  \
                 cudaSuccess;                                                                                      \
  ok = ok && cudaFuncSetAttribute(k_tile_stage<M, REC_GENERAL, 0>, cudaFuncAttributeMaxDynamicSharedMemorySize,     \
                                  b) == cudaSuccess;                                                               \
  ok = ok && cudaFuncSetAttribute(k_tile_stage<M, REC_GENERAL, 1>, cudaFuncAttributeMaxDynamicSharedMemorySize,     \
                                  b) == cudaSuccess
  FVS_TILE_ATTR(MODE_SSP42);
  FVS_TILE_ATTR(MODE_SSP3);
  FVS_TILE_ATTR(MODE_RK);
#undef FVS_TILE_ATTR
  const int bf = (int)tile_fu_smem_bytes(fmax);
#define FVS_TILE_FU_ATTR(M)                                                                                         \
  ok = ok && cudaFuncSetAttribute(k_tile_flux_update<M, REC_FIRST>, cudaFuncAttributeMaxDynamicSharedMemorySize,   \
                                  bf) == cudaSuccess;                                                              \
  ok = ok && cudaFuncSetAttribute(k_tile_flux_update<M, REC_SPEC>, cudaFuncAttributeMaxDynamicSharedMemorySize,    \
                                  bf) == cudaSuccess;                                                              \
  ok = ok && cudaFuncSetAttribute(k_tile_flux_update<M, REC_GENERAL>, cudaFuncAttributeMaxDynamicSharedMemorySize, \
                                  bf) == cudaSuccess
  FVS_TILE_FU_ATTR(MODE_SSP42);
  FVS_TILE_FU_ATTR(MODE_SSP3);
  FVS_TILE_FU_ATTR(MODE_RK);
#undef FVS_TILE_FU_ATTR
  return ok ? bytes : 0;
}
#endif  // FVS_MIXED || FVS_DF

// standalone compute_residual output: resid and ws_nrml
__global__ void __launch_bounds__(256) k_residual_out(const DevView d) {
  pdl_wait();
  pdl_trigger();
  const int ic = blockIdx.x * blockDim.x + threadIdx.x;
  if (ic >= d.nc) return;
  double res[4], ws;
  cell_residual<true, false>(d, ic, res, ws);
  st4(d.resid, ic, res);
  d.ws[ic] = ws;
}

__global__ void __launch_bounds__(256) k_cvar2pvar(const DevView d) {
  pdl_wait();
  pdl_trigger();
  const int ic = blockIdx.x * blockDim.x + threadIdx.x;
  if (ic >= d.nc) return;
  double u[4];
  T p[4];
  ld4(d.U, ic, u);
  cons2prim(TP(gm1), u, p);
  st4(static_cast<T*>(d.Pv), ic, p);
}

// told = t1 + (istep-1)*dt, src/runge_kutta.f90:207-208
__global__ void k_begin_step(const DevView d) {
  pdl_wait();
  pdl_trigger();
  const int istep = d.stepctl[0] + 1;
  d.tctl[1] = d.tctl[0] + double(istep - 1) * d.dt;
}


// ---------------------------------------------------------------------------
// persistent kernel: whole RK steps in one cooperative launch
// ---------------------------------------------------------------------------
// Bounded software grid barrier (all blocks are co-resident: cooperative
// launch).  Returns false once any wait has run out of budget.
__device__ __forceinline__ bool grid_sync(GridBarrier* gb, long long budget) {
  __shared__ int s_ok;
  __syncthreads();
  if (threadIdx.x == 0) {
    volatile unsigned int* vgen = &gb->gen;
    volatile int* verr = &gb->err;
    const unsigned int g = *vgen;
    __threadfence();
    const unsigned int arrived = atomicAdd(&gb->count, 1u) + 1u;
    if (arrived == gridDim.x) {
      atomicExch(&gb->count, 0u);
      __threadfence();
      atomicAdd(&gb->gen, 1u);
    } else {
      const long long t0 = clock64();
      while (*vgen == g) {
        if (*verr) break;
        if (clock64() - t0 > budget) {
          atomicExch(&gb->err, 1);
          break;
        }
        __nanosleep(64);
      }
    }
    __threadfence();
    s_ok = (*verr == 0);
  }
  __syncthreads();
  return s_ok != 0;
}

// the block's norm sums of a tile into tile_partials[t] (FP64 tree: the
// persistent kernels' register budget has no room for the FP32-pair tree)
__device__ __forceinline__ void tile_norm_partial(const PersistPlan& p, const NormAcc& na, int t) {
  double d2[4], out[4];
  na.to_double(d2);
  block_sum4(d2, out);
  if (threadIdx.x == 0)
#pragma unroll
    for (int k = 0; k < 4; k++) p.tile_partials[4 * (size_t)t + k] = out[k];
}

template <int MODE>
__device__ __forceinline__ void update_tile(const DevView& d, const PersistPlan& p, const StageParams& sp, int t) {
  const int4 tl = p.cell_tiles[t];
  NormAcc na;
  for (int ic = tl.x + threadIdx.x; ic < tl.y; ic += blockDim.x) update_item<MODE, true>(d, sp, ic, na);
  if (sp.last) tile_norm_partial(p, na, t);
}

// a case's sums of its tile partials [ct.y, ct.z) by all threads of the
// block, in a fixed order for a given block size: thread i adds tiles i,
// i + blockDim, ..., then the block's FP64 tree; thread 0 holds the sums.
// (Summed by one thread, tile after tile, this took ~0.2 us per tile: 55 us of
// a 135 us step on a 261,120-cell case in tiles of 1024 cells.)
__device__ __forceinline__ void case_tile_sum(const PersistPlan& p, int4 ct, double* a) {
  double s[4] = {0.0, 0.0, 0.0, 0.0};
  for (int t = ct.y + threadIdx.x; t < ct.z; t += blockDim.x)
#pragma unroll
    for (int k = 0; k < 4; k++) s[k] += __ldcg(p.tile_partials + 4 * (size_t)t + k);  // written by other blocks
  block_sum4(s, a);
  __syncthreads();  // the next sum reuses the tree's shared memory
}

// per-case RMS(dU) of a step from the tile partials (fixed order), one block
// per case; the partials are rewritten only at the next step's last stage
__device__ __forceinline__ void case_norms_of_step(const PersistPlan& p, int step) {
  const int slot = step % p.norm_cap;
  for (int c = blockIdx.x; c < p.ncase_active; c += gridDim.x) {
    const int4 ct = p.case_tiles[c];
    double a[4];
    case_tile_sum(p, ct, a);
    if (threadIdx.x == 0) {
      double* o = p.case_norms + 4 * ((size_t)ct.x * p.norm_cap + slot);
#pragma unroll
      for (int k = 0; k < 4; k++) o[k] = sqrt(a[k] / double(ct.w));
    }
  }
}

// Graph form, last stage: the block that finishes the last tile of a case
// (a counter per case) sums that case's norm from its tile partials; the
// last case of the step advances the device step counter.  This replaces a
// separate norm launch per step (~8 us of a 64 us step on a single
// 261,120-cell case).  Call after the tile's partial is written; every
// thread of the block calls it.
__device__ __forceinline__ void tiled_case_norm(const PersistPlan& p, int t) {
  __shared__ int s_last;
  const int slot = p.cell_tiles[t].w;
  const int4 ct = p.case_tiles[slot];
  if (threadIdx.x == 0) {
    __threadfence();
    s_last = atomicAdd(&p.case_count[slot], 1) == ct.z - ct.y - 1;
  }
  __syncthreads();
  if (!s_last) return;
  __threadfence();
  double a[4];
  case_tile_sum(p, ct, a);
  if (threadIdx.x == 0) {
    const int step = __ldcg(p.step0_dev);
    double* o = p.case_norms + 4 * ((size_t)ct.x * p.norm_cap + step % p.norm_cap);
#pragma unroll
    for (int k = 0; k < 4; k++) o[k] = sqrt(a[k] / double(ct.w));
    p.case_count[slot] = 0;
    __threadfence();
    if (atomicAdd(&p.bar->count, 1u) == (unsigned)p.ncase_active - 1) {
      p.bar->count = 0u;
      *const_cast<int*>(p.step0_dev) = step + 1;
    }
  }
}

template <int LIM, int REC>
__global__ void __launch_bounds__(256) k_persistent(const DevView d, const PersistPlan p) {
  const int nb = gridDim.x;
  const int step0 = *p.step0_dev;
  for (int s = 0; s < p.nsteps; s++) {
    const double told = p.t1 + double(step0 + s) * d.dt;
    for (int k = 0; k < p.nstages; k++) {
      const StageParams& sp = p.sp[k];
      if (REC != REC_FIRST) {
        for (int t = blockIdx.x; t < p.ncell_tiles; t += nb) {
          const int4 tl = p.cell_tiles[t];
          for (int ic = tl.x + threadIdx.x; ic < tl.y; ic += blockDim.x) gradient_item<FVS_GRAD_LSQ, LIM, true>(d, ic);
        }
        if (!grid_sync(p.bar, p.budget)) return;
      }
      for (int t = blockIdx.x; t < p.nedge_tiles; t += nb) {
        const int2 tl = p.edge_tiles[t];
        flux_range<REC, true>(d, tl.x + threadIdx.x, tl.y, blockDim.x, told + sp.dts);
      }
      if (!grid_sync(p.bar, p.budget)) return;
      for (int t = blockIdx.x; t < p.ncell_tiles; t += nb) {
        if (sp.mode == MODE_SSP42) update_tile<MODE_SSP42>(d, p, sp, t);
        else if (sp.mode == MODE_SSP3) update_tile<MODE_SSP3>(d, p, sp, t);
        else update_tile<MODE_RK>(d, p, sp, t);
      }
      if (!grid_sync(p.bar, p.budget)) return;
    }
    case_norms_of_step(p, step0 + s);
  }
}

#if FVS_MIXED
// One face of a cell for the fused first-order stage: the cell's signed
// slot s (0: none; > 0: the cell is the edge's L), the other cell nb (-1 on
// a boundary edge), its primitives, and the edge's normal and area.
struct FaceRec {
  float p[4];
  T2 n;
  float af;
  int s, nb;
};

__device__ __forceinline__ void load_face(const DevView& d, const float* P, int s, FaceRec& r) {
  r.s = s;
  r.nb = -1;
  if (s == 0) return;
  const int e = (s > 0 ? s : -s) - 1;
  const int2 lr = d.ecell[e];
  r.nb = s > 0 ? lr.y : lr.x;
  r.n = ld2(d.enrm, e);
  r.af = static_cast<const float*>(d.earea)[e];
  if (r.nb >= 0) ldc4<true>(P, r.nb, r.p);
}

// Roe flux x area and wave speed x area of a face in the edge's own
// orientation (L, R, n), pc the cell's primitives: the REC_FIRST branch of
// flux_item with the same operands
__device__ __forceinline__ void face_flux_first(const DevView& d, const float* pc, const FaceRec& r, double time,
                                                float* flux, float& wsa) {
  float pfL[4], pfR[4];
  if (r.s > 0) {
#pragma unroll
    for (int v = 0; v < 4; v++) pfL[v] = pc[v];
    if (r.nb >= 0) {
#pragma unroll
      for (int v = 0; v < 4; v++) pfR[v] = r.p[v];
    } else {
      const int e = r.s - 1;
      const T2 xy = ld2(d.exy, e);
      ghost_state(d, d.ebtype[e], time, xy.x, xy.y, r.n.x, r.n.y, pfL, pfR);
    }
  } else {
#pragma unroll
    for (int v = 0; v < 4; v++) {
      pfL[v] = r.p[v];
      pfR[v] = pc[v];
    }
  }
  float wsm;
  roe_flux_fast(TP(gamma), TP(gm1), TP(igm1), pfL, pfR, r.n.x, r.n.y, flux, wsm);
#pragma unroll
  for (int v = 0; v < 4; v++) flux[v] = flux[v] * r.af;
  wsa = wsm * r.af;
}

// Fused first-order stage of one cell: the fluxes of its own faces, summed
// in its slot order as cell_residual_f sums the edge records, then the RK
// stage.  An interior face is evaluated by both of its cells with the same
// operands and the edge's own orientation (L, R, n).  All face records are
// loaded first (independent loads); the flux loop is kept rolled, shifting
// the records down one place per pass, so that every face runs the same
// instructions and the two cells receive bit-identical fluxes of opposite
// sign.
template <int MODE>
__device__ __forceinline__ void cell_stage_item(const DevView& d, const StageParams& sp, const float* Pin,
                                                float* Pout, int ic, double time, NormAcc& na) {
  const int4 cf = d.cflist[ic];
  FaceRec f0, f1, f2, f3;
  load_face(d, Pin, cf.x, f0);
  load_face(d, Pin, cf.y, f1);
  load_face(d, Pin, cf.z, f2);
  load_face(d, Pin, cf.w, f3);
  float pc[4];
  ldc4<true>(Pin, ic, pc);
  float hi[4] = {0.f, 0.f, 0.f, 0.f}, lo[4] = {0.f, 0.f, 0.f, 0.f}, wh = 0.f, wl = 0.f;
  const bool want_ws = sp.steady && sp.stage == 1;
#pragma unroll 1
  for (int j = 0; j < 4; j++) {
    if (f0.s != 0) {
      float f[4], wsa;
      face_flux_first(d, pc, f0, time, f, wsa);
#pragma unroll
      for (int v = 0; v < 4; v++) two_sum(hi[v], lo[v], f0.s > 0 ? f[v] : -f[v]);
      if (want_ws) two_sum(wh, wl, wsa);
    }
    f0 = f1;
    f1 = f2;
    f2 = f3;
    f3.s = 0;
  }
  const float rv = -static_cast<const float*>(d.volT)[ic];
  float res[4];
#pragma unroll
  for (int v = 0; v < 4; v++) res[v] = (hi[v] + lo[v]) * rv;
  apply_stage_f<MODE, true>(d, sp, ic, res, wh + wl, Pout, na);
}

template <int MODE>
__device__ __forceinline__ void cell_stage_tile(const DevView& d, const PersistPlan& p, const StageParams& sp,
                                                const float* Pin, float* Pout, int t, double time) {
  const int4 tl = p.cell_tiles[t];
  NormAcc na;
  for (int ic = tl.x + threadIdx.x; ic < tl.y; ic += blockDim.x) cell_stage_item<MODE>(d, sp, Pin, Pout, ic, time, na);
  if (sp.last) tile_norm_partial(p, na, t);
}

// primitives read by stage k (0-based) and written by it: Pv and Pv2 in
// turn, so that with an even stage count every step ends in Pv
__device__ __forceinline__ const float* stage_pin(const DevView& d, int k) {
  return static_cast<const float*>((k & 1) ? d.Pv2 : d.Pv);
}
__device__ __forceinline__ float* stage_pout(const DevView& d, int k) {
  return static_cast<float*>((k & 1) ? d.Pv : d.Pv2);
}

template <int MODE>
__device__ __forceinline__ void cell_stage_phase(const DevView& d, const PersistPlan& p, int k, double time) {
  for (int t = blockIdx.x; t < p.ncell_tiles; t += gridDim.x)
    cell_stage_tile<MODE>(d, p, p.sp[k], stage_pin(d, k), stage_pout(d, k), t, time);
}

// First-order mixed stages with the flux evaluated per cell: one phase and
// one grid barrier per stage instead of a flux phase and an update phase,
// and no edge flux records in memory.
// (every stage of a scheme has the same MODE)
template <int MODE>
__global__ void __launch_bounds__(256, 2) k_persistent_cell(const DevView d, const PersistPlan p) {
  const int step0 = *p.step0_dev;
  for (int s = 0; s < p.nsteps; s++) {
    const double told = p.t1 + double(step0 + s) * d.dt;
    for (int k = 0; k < p.nstages; k++) {
      cell_stage_phase<MODE>(d, p, k, told + p.sp[k].dts);
      if (!grid_sync(p.bar, p.budget)) return;
    }
    case_norms_of_step(p, step0 + s);
  }
}

template <int MODE>
__global__ void __launch_bounds__(256, 2) k_tiles_cell(const DevView d, const PersistPlan p, int k) {
  const double time = p.t1 + double(*p.step0_dev) * d.dt + p.sp[k].dts;
  cell_stage_tile<MODE>(d, p, p.sp[k], stage_pin(d, k), stage_pout(d, k), blockIdx.x, time);
  if (p.sp[k].last) tiled_case_norm(p, blockIdx.x);
}
#endif

// the fused first-order stage is in use (the host sets Pv2 only for
// first-order mixed batches with an even number of stages)
static inline bool cell_fused(const DevView& d) { return FVS_MIXED && d.Pv2 != nullptr && d.first_order; }

template <int LIM, int REC>
static cudaError_t launch_persistent_t(const DevView& d, const PersistPlan& p, int grid, int block, cudaStream_t s) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3((unsigned)block);
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  return cudaLaunchKernelEx(&cfg, k_persistent<LIM, REC>, d, p);
}

static bool persistent_spec(const DevView& d) {
  return !FVS_STRICT && d.khalf == 0.0 && d.omk == 1.0 && d.limiter == FVS_LIM_NONE && !d.first_order;
}

static int persistent_occupancy(const DevView& d, int block) {
  if (d.grad_method != FVS_GRAD_LSQ) return 0;
  int n = 0;
  cudaError_t e;
#if FVS_MIXED
  if (cell_fused(d)) {
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_persistent_cell<MODE_SSP42>, block, 0);
    return e == cudaSuccess ? n : 0;
  }
#endif
  if (d.first_order) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_persistent<0, REC_FIRST>, block, 0);
  else if (d.limiter != FVS_LIM_NONE)
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_persistent<1, REC_GENERAL>, block, 0);
  else if (persistent_spec(d)) e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_persistent<0, REC_SPEC>, block, 0);
  else e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_persistent<0, REC_GENERAL>, block, 0);
  return e == cudaSuccess ? n : 0;
}

static cudaError_t launch_persistent(const DevView& d, const PersistPlan& p, int grid, int block, cudaStream_t s) {
#if FVS_MIXED
  if (cell_fused(d)) {
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3((unsigned)grid);
    cfg.blockDim = dim3((unsigned)block);
    cfg.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    cfg.attrs = attr;
    cfg.numAttrs = 1;
    if (p.sp[0].mode == MODE_SSP42) return cudaLaunchKernelEx(&cfg, k_persistent_cell<MODE_SSP42>, d, p);
    if (p.sp[0].mode == MODE_SSP3) return cudaLaunchKernelEx(&cfg, k_persistent_cell<MODE_SSP3>, d, p);
    return cudaLaunchKernelEx(&cfg, k_persistent_cell<MODE_RK>, d, p);
  }
#endif
  if (d.first_order) return launch_persistent_t<0, REC_FIRST>(d, p, grid, block, s);
  if (d.limiter != FVS_LIM_NONE) return launch_persistent_t<1, REC_GENERAL>(d, p, grid, block, s);
  if (persistent_spec(d)) return launch_persistent_t<0, REC_SPEC>(d, p, grid, block, s);
  return launch_persistent_t<0, REC_GENERAL>(d, p, grid, block, s);
}

// ---------------------------------------------------------------------------
// tiled step: the same tile work as the persistent kernel, one launch per
// phase (one block per tile), for capture in a CUDA graph; the device step
// counter (*step0_dev) advances at the end of each step
// ---------------------------------------------------------------------------
template <int LIM>
__global__ void __launch_bounds__(256) k_tiles_gradient(const DevView d, const PersistPlan p) {
  const int4 tl = p.cell_tiles[blockIdx.x];
  for (int ic = tl.x + threadIdx.x; ic < tl.y; ic += blockDim.x) gradient_item<FVS_GRAD_LSQ, LIM, false>(d, ic);
}

// ONE: tiles as long as the block, one edge slot or cell per thread (the
// single-mesh kernels' shape and register budget: no paired slots, no loop)
template <int REC, bool ONE>
__global__ void __launch_bounds__(256) k_tiles_flux(const DevView d, const PersistPlan p, int stage) {
  const double told = p.t1 + double(*p.step0_dev) * d.dt;
  const int2 tl = p.edge_tiles[blockIdx.x];
  if (ONE) {
    const int e = tl.x + threadIdx.x;
    if (e < tl.y) flux_item<REC, false>(d, e, told + p.sp[stage].dts);
  } else {
    flux_range<REC, false>(d, tl.x + threadIdx.x, tl.y, blockDim.x, told + p.sp[stage].dts);
  }
}

template <int MODE, bool ONE>
__global__ void __launch_bounds__(256) k_tiles_update(const DevView d, const PersistPlan p, int stage) {
  const StageParams& sp = p.sp[stage];
  if (ONE) {
    const int4 tl = p.cell_tiles[blockIdx.x];
    const int ic = tl.x + threadIdx.x;
    NormAcc na;
    if (ic < tl.y) update_item<MODE, false>(d, sp, ic, na);
    if (sp.last) tile_norm_partial(p, na, blockIdx.x);
  } else {
    update_tile<MODE>(d, p, sp, blockIdx.x);
  }
  if (sp.last) tiled_case_norm(p, blockIdx.x);
}

static cudaError_t launch_tiled_step(const DevView& d, const PersistPlan& p, int block, cudaStream_t s) {
  const bool one = p.tile == block;
#if FVS_MIXED
  if (cell_fused(d)) {
    for (int k = 0; k < p.nstages; k++) {
      switch (p.sp[k].mode) {
        case MODE_SSP42: k_tiles_cell<MODE_SSP42><<<p.ncell_tiles, block, 0, s>>>(d, p, k); break;
        case MODE_SSP3: k_tiles_cell<MODE_SSP3><<<p.ncell_tiles, block, 0, s>>>(d, p, k); break;
        default: k_tiles_cell<MODE_RK><<<p.ncell_tiles, block, 0, s>>>(d, p, k); break;
      }
    }
    return cudaGetLastError();
  }
#endif
  for (int k = 0; k < p.nstages; k++) {
    if (!d.first_order) {
      if (d.limiter != FVS_LIM_NONE) k_tiles_gradient<1><<<p.ncell_tiles, block, 0, s>>>(d, p);
      else k_tiles_gradient<0><<<p.ncell_tiles, block, 0, s>>>(d, p);
    }
    if (one) {
      if (d.first_order) k_tiles_flux<REC_FIRST, true><<<p.nedge_tiles, block, 0, s>>>(d, p, k);
      else if (persistent_spec(d)) k_tiles_flux<REC_SPEC, true><<<p.nedge_tiles, block, 0, s>>>(d, p, k);
      else k_tiles_flux<REC_GENERAL, true><<<p.nedge_tiles, block, 0, s>>>(d, p, k);
      switch (p.sp[k].mode) {
        case MODE_SSP42: k_tiles_update<MODE_SSP42, true><<<p.ncell_tiles, block, 0, s>>>(d, p, k); break;
        case MODE_SSP3: k_tiles_update<MODE_SSP3, true><<<p.ncell_tiles, block, 0, s>>>(d, p, k); break;
        default: k_tiles_update<MODE_RK, true><<<p.ncell_tiles, block, 0, s>>>(d, p, k); break;
      }
      continue;
    }
    if (d.first_order) k_tiles_flux<REC_FIRST, false><<<p.nedge_tiles, block, 0, s>>>(d, p, k);
    else if (persistent_spec(d)) k_tiles_flux<REC_SPEC, false><<<p.nedge_tiles, block, 0, s>>>(d, p, k);
    else k_tiles_flux<REC_GENERAL, false><<<p.nedge_tiles, block, 0, s>>>(d, p, k);
    switch (p.sp[k].mode) {
      case MODE_SSP42: k_tiles_update<MODE_SSP42, false><<<p.ncell_tiles, block, 0, s>>>(d, p, k); break;
      case MODE_SSP3: k_tiles_update<MODE_SSP3, false><<<p.ncell_tiles, block, 0, s>>>(d, p, k); break;
      default: k_tiles_update<MODE_RK, false><<<p.ncell_tiles, block, 0, s>>>(d, p, k); break;
    }
  }
  return cudaGetLastError();
}


// ---------------------------------------------------------------------------
// launchers
// ---------------------------------------------------------------------------
static inline unsigned grid_of(int n) { return (unsigned)((n + 255) / 256); }


static void launch_begin_step(const DevView& d, cudaStream_t s) { launch_k(k_begin_step, 1, 1, 0, s, d); }
static void launch_cvar2pvar(const DevView& d, cudaStream_t s) { launch_k(k_cvar2pvar, grid_of(d.nc), 256, 0, s, d); }

static void launch_gradient(const DevView& d, cudaStream_t s) {
  if (d.first_order) return;
  const unsigned g = grid_of(d.nc);
  const bool lim = d.limiter != FVS_LIM_NONE;
  switch (d.grad_method) {
    case FVS_GRAD_LSQ:
      if (lim) launch_k(k_gradient<FVS_GRAD_LSQ, 1>, g, 256, 0, s, d);
      else launch_k(k_gradient<FVS_GRAD_LSQ, 0>, g, 256, 0, s, d);
      break;
    case FVS_GRAD_GGCB: launch_k(k_gradient<FVS_GRAD_GGCB, 0>, g, 256, 0, s, d); break;
    default: launch_k(k_gradient<FVS_GRAD_GGNB, 0>, g, 256, 0, s, d); break;
  }
}

static void launch_flux(const DevView& d, double dts, bool ws_out, cudaStream_t s) {
  const bool spec = !FVS_STRICT && d.khalf == 0.0 && d.omk == 1.0 && d.limiter == FVS_LIM_NONE && !d.first_order;
  const int w = ws_out ? 1 : 0;
  if (d.first_order) launch_k(k_flux<REC_FIRST>, grid_of(d.nedge), 256, 0, s, d, dts, w);
  else if (spec) launch_k(k_flux<REC_SPEC>, grid_of(d.nedge), 256, 0, s, d, dts, w);
  else launch_k(k_flux<REC_GENERAL>, grid_of(d.nedge), 256, 0, s, d, dts, w);
}

// blocks of 256 threads of kernel k resident on the whole device at once
template <class K>
static unsigned resident_blocks(K k) {
  int dev = 0, nsm = 0, per_sm = 0;
  if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess ||
      cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k, 256, 0) != cudaSuccess || nsm <= 0 || per_sm <= 0)
    return 0;
  return (unsigned)(nsm * per_sm);
}

static int update_wave(int mode) {
  const unsigned w = mode == MODE_SSP42 ? resident_blocks(k_update<MODE_SSP42, true>)
                     : mode == MODE_SSP3 ? resident_blocks(k_update<MODE_SSP3, true>)
                                         : resident_blocks(k_update<MODE_RK, true>);
  return (int)w;
}

template <int MODE>
static void launch_update_mode(const DevView& d, const StageParams& sp, cudaStream_t s) {
  const unsigned g = grid_of(d.nc);
  if (!sp.last || d.upd_grid <= 0 || (unsigned)d.upd_grid >= g) {
    launch_k(k_update<MODE, false>, g, 256, 0, s, d, sp);
    return;
  }
  // The last stage reduces the norms: one wave of resident blocks walks the
  // cells (grid stride), so that the block-end reduction, fence and counter
  // run once per resident block instead of once per 256 cells, and the last
  // block sums that many partials.
  DevView dl = d;
  dl.nblk_red = d.upd_grid;
  launch_k(k_update<MODE, true>, (unsigned)d.upd_grid, 256, 0, s, dl, sp);
}

static void launch_update(const DevView& d, const StageParams& sp, cudaStream_t s) {
  switch (sp.mode) {
    case MODE_SSP42: launch_update_mode<MODE_SSP42>(d, sp, s); break;
    case MODE_SSP3: launch_update_mode<MODE_SSP3>(d, sp, s); break;
    default: launch_update_mode<MODE_RK>(d, sp, s); break;
  }
}

static void launch_residual_out(const DevView& d, cudaStream_t s) { launch_k(k_residual_out, grid_of(d.nc), 256, 0, s, d); }

#if FVS_MIXED
// ---------------------------------------------------------------------------
// defect correction (first-order steady batches)
// ---------------------------------------------------------------------------
// FP32 dual number (value, tangent): forward-mode derivative of the Roe flux,
// i.e. the Jacobian-vector product J(U) dU of the linearised residual.
struct Dual {
  float v, d;
  __device__ __forceinline__ Dual() {}
  __device__ __forceinline__ Dual(float x) : v(x), d(0.f) {}
  __device__ __forceinline__ Dual(float x, float dx) : v(x), d(dx) {}
};
__device__ __forceinline__ Dual operator+(Dual a, Dual b) { return Dual(a.v + b.v, a.d + b.d); }
__device__ __forceinline__ Dual operator-(Dual a, Dual b) { return Dual(a.v - b.v, a.d - b.d); }
__device__ __forceinline__ Dual operator-(Dual a) { return Dual(-a.v, -a.d); }
__device__ __forceinline__ Dual operator*(Dual a, Dual b) { return Dual(a.v * b.v, a.d * b.v + a.v * b.d); }
__device__ __forceinline__ Dual operator/(Dual a, Dual b) {
  const float r = 1.0f / b.v, q = a.v * r;
  return Dual(q, (a.d - q * b.d) * r);
}
__device__ __forceinline__ bool operator<(Dual a, Dual b) { return a.v < b.v; }
__device__ __forceinline__ Dual dsqrt_(Dual a) {
  const float s = sqrtf(a.v);
  return Dual(s, 0.5f * a.d / s);
}
__device__ __forceinline__ Dual dabs_(Dual a) { return a.v < 0.f ? -a : a; }
__device__ __forceinline__ Dual half(Dual a) { return Dual(0.5f * a.v, 0.5f * a.d); }

// ghost state of boundary slot e and its tangent: the slip-wall mirror is
// linear in the interior state; free-stream and Dirichlet ghost states do not
// depend on it
__device__ __forceinline__ void dc_ghost(const DevView& d, int e, T2 n, const float* pl, const float* ql, float* pr,
                                         float* qr) {
  const int rec = d.ebtype[e];
  const T2 xy = ld2(d.exy, e);
  ghost_state(d, rec, 0.0, xy.x, xy.y, n.x, n.y, pl, pr);
  if ((rec & 15) == FVS_BC_SLIP_WALL) {
    const float un = ql[1] * n.x + ql[2] * n.y;
    qr[0] = ql[0];
    qr[1] = ql[1] - 2.0f * un * n.x;
    qr[2] = ql[2] - 2.0f * un * n.y;
    qr[3] = ql[3];
  } else {
#pragma unroll
    for (int v = 0; v < 4; v++) qr[v] = 0.0f;
  }
}

// dual-number helpers of the linearised flux: a*b + c, a*x and x*a for a
// constant x, and the reciprocal and reciprocal square root from the fast
// hardware approximations (the tangent only steers the correction; its fixed
// point is the FP64 residual's whatever the tangent's last bits)
__device__ __forceinline__ Dual dfma_(Dual a, Dual b, Dual c) {
  return Dual(fmaf(a.v, b.v, c.v), fmaf(a.d, b.v, fmaf(a.v, b.d, c.d)));
}
__device__ __forceinline__ Dual dmulf_(Dual a, float x) { return Dual(a.v * x, a.d * x); }
__device__ __forceinline__ Dual dfmaf_(Dual a, float x, Dual c) { return Dual(fmaf(a.v, x, c.v), fmaf(a.d, x, c.d)); }
__device__ __forceinline__ Dual drcp_(Dual a) {
  const float r = __fdividef(1.0f, a.v);
  return Dual(r, -a.d * r * r);
}
__device__ __forceinline__ Dual drsqrt_(Dual a) {
  const float r = rsqrtf(a.v);
  return Dual(r, -0.5f * a.d * r * r * r);
}

// The Roe flux of roe_flux_area_fp64 (the same folded constants and order)
// on dual numbers: value and tangent of flux * area in the direction of the
// primitive tangents.  The value part is the FP32 flux the tangent needs.
__device__ __forceinline__ void roe_flux_area_dual(float gm1, float ggm1, const Dual* pl, const Dual* pr, float nx,
                                                   float ny, float af, Dual* flux) {
  const Dual rhoL = pl[0], uL = pl[1], vL = pl[2], pL = pl[3];
  const Dual rhoR = pr[0], uR = pr[1], vR = pr[2], pR = pr[3];
  const Dual riL = drcp_(rhoL), riR = drcp_(rhoR);
  const Dual unL = dfmaf_(uL, nx, dmulf_(vL, ny)), unR = dfmaf_(uR, nx, dmulf_(vR, ny));
  const Dual utL = dfmaf_(vL, nx, -dmulf_(uL, ny)), utR = dfmaf_(vR, nx, -dmulf_(uR, ny));
  const Dual HL = dfma_(dmulf_(pL, ggm1), riL, half(dfma_(uL, uL, vL * vL)));
  const Dual HR = dfma_(dmulf_(pR, ggm1), riR, half(dfma_(uR, uR, vR * vR)));
  const Dual sRL = rhoR * riL;
  const Dual RT = sRL * drsqrt_(sRL);
  const Dual rho = RT * rhoL;
  const Dual i1 = drcp_(Dual(1.0f + RT.v, RT.d));
  const Dual u = dfma_(RT, uR, uL) * i1;
  const Dual v = dfma_(RT, vR, vL) * i1;
  const Dual H = dfma_(RT, HR, HL) * i1;
  const Dual q2 = half(dfma_(u, u, v * v));
  const Dual a2 = dmulf_(H - q2, gm1);
  const Dual ra = drsqrt_(a2);
  const Dual a = a2 * ra, ia2 = ra * ra;
  const Dual un = dfmaf_(u, nx, dmulf_(v, ny));
  const Dual ut = dfmaf_(v, nx, -dmulf_(u, ny));
  const Dual drho = rhoR - rhoL, dp = pR - pL, dun = unR - unL, dut = utR - utL;
  const Dual rad = rho * a * dun;
  const Dual hia2 = half(ia2);
  const Dual L0 = (dp - rad) * hia2;
  const Dual L1 = rho * dut;
  const Dual L2 = dfma_(-dp, ia2, drho);
  const Dual L3 = (dp + rad) * hia2;
  Dual ws0 = dabs_(un - a), ws3 = dabs_(un + a);
  const Dual ws1 = dabs_(un);
  // Harten's fix, 0.5 (l^2 / 0.2 + 0.2) = 2.5 l^2 + 0.1
  if (ws0.v < 0.2f) ws0 = dfma_(dmulf_(ws0, 2.5f), ws0, Dual(0.1f));
  if (ws3.v < 0.2f) ws3 = dfma_(dmulf_(ws3, 2.5f), ws3, Dual(0.1f));
  const Dual w0 = ws0 * L0, w1 = ws1 * L1, w2 = ws1 * L2, w3 = ws3 * L3;
  const Dual s03 = w0 + w3, sd = s03 + w2, dw = (w3 - w0) * a;
  // eigenvector sum with tx = -ny, ty = nx
  const Dual diss1 = dfma_(u, sd, dfmaf_(dw, nx, -dmulf_(w1, ny)));
  const Dual diss2 = dfma_(v, sd, dfmaf_(dw, ny, dmulf_(w1, nx)));
  const Dual diss3 = dfma_(H, s03, dfma_(un, dw, dfma_(w1, ut, w2 * q2)));
  const Dual mL = rhoL * unL, mR = rhoR * unR;
  const Dual pLR = pL + pR;
  const float haf = 0.5f * af;
  flux[0] = dmulf_((mL + mR) - sd, haf);
  flux[1] = dmulf_(dfma_(mL, uL, mR * uR) + dfmaf_(pLR, nx, -diss1), haf);
  flux[2] = dmulf_(dfma_(mL, vL, mR * vR) + dfmaf_(pLR, ny, -diss2), haf);
  flux[3] = dmulf_(dfma_(mL, HL, mR * HR) - diss3, haf);
}

// tangent of the Roe flux at (pl, pr) in the direction (ql, qr), times the
// face area
__device__ __forceinline__ void dc_jvp_core(const DevView& d, const float* pl, const float* ql, const float* pr,
                                            const float* qr, T2 n, float af, float* f) {
  Dual L[4], R[4], F[4];
#pragma unroll
  for (int v = 0; v < 4; v++) {
    L[v] = Dual(pl[v], ql[v]);
    R[v] = Dual(pr[v], qr[v]);
  }
  roe_flux_area_dual(d.fgm1, d.fggm1, L, R, n.x, n.y, af, F);
#pragma unroll
  for (int v = 0; v < 4; v++) f[v] = F[v].d;
}

// J dU of one edge slot (first order: face states are the cell states),
// times the face area; primitive tangents read from dP
__device__ __forceinline__ void dc_edge_jvp(const DevView& d, const float* dP, int e, float* f) {
  const float* P = static_cast<const float*>(d.Pv);
  const int2 lr = d.ecell[e];
  const T2 n = ld2(d.enrm, e);
  const float af = static_cast<const float*>(d.earea)[e];
  float pl[4], ql[4], pr[4], qr[4];
  ld4(P, lr.x, pl);
  ldc4<true>(dP, lr.x, ql);
  if (lr.y >= 0) {
    ld4(P, lr.y, pr);
    ldc4<true>(dP, lr.y, qr);
  } else {
    dc_ghost(d, e, n, pl, ql, pr, qr);
  }
  dc_jvp_core(d, pl, ql, pr, qr, n, af, f);
}

// J dU of one edge slot into the slot's flux record
__device__ __forceinline__ void dc_flux_item(const DevView& d, const DcView& c, int e) {
  float f[4];
  dc_edge_jvp(d, c.dP, e, f);
  st4(static_cast<float*>(d.eflux), e, f);
}

// the edge slots [b, end) of a tile with stride `stride`, one at a time (two
// per pass, as flux_range does, spilled at this kernel's register budget and
// ran slower)
__device__ __forceinline__ void dc_flux_range(const DevView& d, const DcView& c, int b, int end, int stride) {
  for (int e = b; e < end; e += stride) dc_flux_item(d, c, e);
}

// One cell of an RK stage of the correction with the residual R0 + J dU (the
// same stage formulas as update_item, local dt frozen at the base state);
// writes the primitive tangent of the new dU and, at the last stage, adds
// |dU - dU0|^2 to d2.
template <int MODE>
__device__ __forceinline__ void dc_apply_stage(const DevView& d, const DcView& c, const StageParams& sp, int ic,
                                               const float* acc, float* dPout, float* d2) {
  const float rv = -static_cast<const float*>(d.volT)[ic];
  float r0[4], res[4];
  ld4(c.R0, ic, r0);
#pragma unroll
  for (int v = 0; v < 4; v++) res[v] = r0[v] + acc[v] * rv;
  const float h = c.dtl[ic] * float(sp.cst);
  float u0[4], u[4], f[4];
  if (sp.stage == 1) {
    ldc4<true>(c.D, ic, u0);
    st4(c.D0, ic, u0);
#pragma unroll
    for (int v = 0; v < 4; v++) f[v] = 0.f;
  } else {
    ldc4<true>(c.D0, ic, u0);
    ldc4<true>(c.DF, ic, f);
  }
  const float coef = float(sp.coef);
  if (MODE == MODE_SSP42) {
#pragma unroll
    for (int v = 0; v < 4; v++) {
      u[v] = u0[v] + h * (coef * res[v] + f[v]);
      f[v] = f[v] + res[v];
    }
  } else {
#pragma unroll
    for (int v = 0; v < 4; v++) {
      f[v] = f[v] + coef * res[v];
      u[v] = sp.last ? u0[v] + h * f[v] : u0[v] + h * res[v];
    }
  }
  if (!sp.last) st4(c.DF, ic, f);
  st4(c.D, ic, u);
  // tangent of cvar2pvar at the base primitives p
  float p[4];
  ld4(static_cast<const float*>(d.Pv), ic, p);
  const float ri = 1.0f / p[0];
  const float du = (u[1] - p[1] * u[0]) * ri, dv = (u[2] - p[2] * u[0]) * ri;
  const float q[4] = {u[0], du, dv,
                      d.fgm1 * (u[3] - 0.5f * u[0] * (p[1] * p[1] + p[2] * p[2]) - p[0] * (p[1] * du + p[2] * dv))};
  st4(dPout, ic, q);
  if (sp.last) {
#pragma unroll
    for (int v = 0; v < 4; v++) {
      const float dd = u[v] - u0[v];
      d2[v] += dd * dd;
    }
  }
}

template <int MODE>
__device__ __forceinline__ void dc_update_item(const DevView& d, const DcView& c, const StageParams& sp, int ic,
                                               float* d2) {
  float acc[4] = {0.f, 0.f, 0.f, 0.f};
  const int4 cf = d.cflist[ic];
  const int sl[4] = {cf.x, cf.y, cf.z, cf.w};
#pragma unroll
  for (int j = 0; j < 4; j++) {
    const int s = sl[j];
    if (s == 0) continue;
    float f[4];
    ldc4<true>(static_cast<const float*>(d.eflux), (s > 0 ? s : -s) - 1, f);
#pragma unroll
    for (int v = 0; v < 4; v++) acc[v] += s > 0 ? f[v] : -f[v];
  }
  dc_apply_stage<MODE>(d, c, sp, ic, acc, c.dP, d2);
}

// the correction tangents read and written by stage k (0-based) of the fused
// stage: dP and dP2 in turn, so that with an even stage count every step
// ends in dP
__device__ __forceinline__ const float* dc_pin(const DcView& c, int k) { return (k & 1) ? c.dP2 : c.dP; }
__device__ __forceinline__ float* dc_pout(const DcView& c, int k) { return (k & 1) ? c.dP : c.dP2; }

// one face of a cell for the fused correction stage (as FaceRec, with the
// other cell's base primitives p and tangent q)
struct DcFace {
  float p[4], q[4];
  T2 n;
  float af;
  int s, nb;
};

__device__ __forceinline__ void load_dc_face(const DevView& d, const float* dP, int s, DcFace& r) {
  r.s = s;
  r.nb = -1;
  if (s == 0) return;
  const int e = (s > 0 ? s : -s) - 1;
  const int2 lr = d.ecell[e];
  r.nb = s > 0 ? lr.y : lr.x;
  r.n = ld2(d.enrm, e);
  r.af = static_cast<const float*>(d.earea)[e];
  if (r.nb >= 0) {
    ld4(static_cast<const float*>(d.Pv), r.nb, r.p);
    ldc4<true>(dP, r.nb, r.q);
  }
}

// J dU of a face in the edge's own orientation; (pc, qc) the cell's base
// primitives and tangent
__device__ __forceinline__ void dc_face_jvp(const DevView& d, const float* pc, const float* qc, const DcFace& r,
                                            float* f) {
  float pl[4], ql[4], pr[4], qr[4];
  if (r.s > 0) {
#pragma unroll
    for (int v = 0; v < 4; v++) {
      pl[v] = pc[v];
      ql[v] = qc[v];
    }
    if (r.nb >= 0) {
#pragma unroll
      for (int v = 0; v < 4; v++) {
        pr[v] = r.p[v];
        qr[v] = r.q[v];
      }
    } else {
      dc_ghost(d, r.s - 1, r.n, pl, ql, pr, qr);
    }
  } else {
#pragma unroll
    for (int v = 0; v < 4; v++) {
      pl[v] = r.p[v];
      ql[v] = r.q[v];
      pr[v] = pc[v];
      qr[v] = qc[v];
    }
  }
  dc_jvp_core(d, pl, ql, pr, qr, r.n, r.af, f);
}

// Fused correction stage of one cell: J dU of its own faces (each interior
// face evaluated by both cells in the edge's orientation; records loaded
// first and the loop kept rolled, as in cell_stage_item), summed in slot
// order, then the stage.
template <int MODE>
__device__ __forceinline__ void dc_cell_item(const DevView& d, const DcView& c, const StageParams& sp,
                                             const float* dPin, float* dPout, int ic, float* d2) {
  const int4 cf = d.cflist[ic];
  DcFace f0, f1, f2, f3;
  load_dc_face(d, dPin, cf.x, f0);
  load_dc_face(d, dPin, cf.y, f1);
  load_dc_face(d, dPin, cf.z, f2);
  load_dc_face(d, dPin, cf.w, f3);
  float pc[4], qc[4];
  ld4(static_cast<const float*>(d.Pv), ic, pc);
  ldc4<true>(dPin, ic, qc);
  float acc[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll 1
  for (int j = 0; j < 4; j++) {
    if (f0.s != 0) {
      float f[4];
      dc_face_jvp(d, pc, qc, f0, f);
#pragma unroll
      for (int v = 0; v < 4; v++) acc[v] += f0.s > 0 ? f[v] : -f[v];
    }
    f0 = f1;
    f1 = f2;
    f2 = f3;
    f3.s = 0;
  }
  dc_apply_stage<MODE>(d, c, sp, ic, acc, dPout, d2);
}

// One cell tile of a correction stage (FUSED: with the cell's own face
// J dU; otherwise from the edge records of a separate J dU phase) and, at
// the last stage, the tile's partial sums of |dU - dU0|^2
template <int MODE, bool FUSED>
__device__ __forceinline__ void dc_stage_tile(const DevView& d, const DcView& c, const PersistPlan& p, int k, int t) {
  const StageParams& sp = p.sp[k];
  const int4 tl = p.cell_tiles[t];
  float d2f[4] = {0.f, 0.f, 0.f, 0.f};
  for (int ic = tl.x + threadIdx.x; ic < tl.y; ic += blockDim.x) {
    if (FUSED) dc_cell_item<MODE>(d, c, sp, dc_pin(c, k), dc_pout(c, k), ic, d2f);
    else dc_update_item<MODE>(d, c, sp, ic, d2f);
  }
  if (sp.last) {
    const double d2[4] = {f2d_bits(d2f[0]), f2d_bits(d2f[1]), f2d_bits(d2f[2]), f2d_bits(d2f[3])};
    double out[4];
    block_sum4(d2, out);
    if (threadIdx.x == 0)
#pragma unroll
      for (int q = 0; q < 4; q++) p.tile_partials[4 * (size_t)t + q] = out[q];
  }
}

template <int MODE>
__global__ void __launch_bounds__(256, 4) k_persistent_dc(const DevView d, const PersistPlan p, const DcView c) {
  const int nb = gridDim.x;
  const int step0 = *p.step0_dev;
  for (int s = 0; s < p.nsteps; s++) {
    for (int k = 0; k < p.nstages; k++) {
      for (int t = blockIdx.x; t < p.nedge_tiles; t += nb) {
        const int2 tl = p.edge_tiles[t];
        dc_flux_range(d, c, tl.x + threadIdx.x, tl.y, blockDim.x);
      }
      if (!grid_sync(p.bar, p.budget)) return;
      for (int t = blockIdx.x; t < p.ncell_tiles; t += nb) dc_stage_tile<MODE, false>(d, c, p, k, t);
      if (!grid_sync(p.bar, p.budget)) return;
    }
    // per-case RMS of the correction increments of this step (fixed order)
    case_norms_of_step(p, step0 + s);
  }
}

// fused correction stages: one phase and one grid barrier per stage
template <int MODE>
__global__ void __launch_bounds__(256, 2) k_persistent_dc_cell(const DevView d, const PersistPlan p, const DcView c) {
  const int step0 = *p.step0_dev;
  for (int s = 0; s < p.nsteps; s++) {
    for (int k = 0; k < p.nstages; k++) {
      for (int t = blockIdx.x; t < p.ncell_tiles; t += gridDim.x) dc_stage_tile<MODE, true>(d, c, p, k, t);
      if (!grid_sync(p.bar, p.budget)) return;
    }
    case_norms_of_step(p, step0 + s);
  }
}

__global__ void __launch_bounds__(256) k_dc_fold(const DevView d, const DcView c, double* U64) {
  const int ic = blockIdx.x * blockDim.x + threadIdx.x;
  if (ic >= d.nc) return;
  float du[4];
  ld4(c.D, ic, du);
  double u[4];
  ld4(U64, ic, u);
#pragma unroll
  for (int v = 0; v < 4; v++) u[v] += double(du[v]);
  st4(U64, ic, u);
  const float z[4] = {0.f, 0.f, 0.f, 0.f};
  st4(c.D, ic, z);
  st4(c.dP, ic, z);
}

__global__ void __launch_bounds__(256) k_dc_base(const DevView d, const DcView c, const double* U64,
                                                 const double* resid64, const double* ws64) {
  const int ic = blockIdx.x * blockDim.x + threadIdx.x;
  if (ic >= d.nc) return;
  double u[4], r[4];
  ld4(U64, ic, u);
  float p[4];
  cons2prim(d.fgm1, u, p);
  st4(static_cast<float*>(d.Pv), ic, p);
  ld4(resid64, ic, r);
  const float rf[4] = {float(r[0]), float(r[1]), float(r[2]), float(r[3])};
  st4(c.R0, ic, rf);
  // compute_local_time, src/runge_kutta.f90:424-437, at the base state
  d.dtl[ic] = d.cfl * d.vol[ic] / (0.5 * ws64[ic]);
  c.dtl[ic] = d2f_bits(d.dtl[ic]);
}

static void dc_fold(const DevView& d, const DcView& c, double* U64, cudaStream_t s) {
  k_dc_fold<<<grid_of(d.nc), 256, 0, s>>>(d, c, U64);
}
static void dc_base(const DevView& d, const DcView& c, const double* U64, const double* resid64, const double* ws64,
                    cudaStream_t s) {
  k_dc_base<<<grid_of(d.nc), 256, 0, s>>>(d, c, U64, resid64, ws64);
}
static int dc_occupancy(const DcView& c, int block) {
  int n = 0;
  const cudaError_t e =
      c.dP2 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_persistent_dc_cell<MODE_SSP42>, block, 0)
            : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_persistent_dc<MODE_SSP42>, block, 0);
  return e == cudaSuccess ? n : 0;
}
static cudaError_t dc_persistent(const DevView& d, const PersistPlan& p, const DcView& c, int grid, int block,
                                 cudaStream_t s) {
  cudaLaunchConfig_t cfg = {};
  cfg.gridDim = dim3((unsigned)grid);
  cfg.blockDim = dim3((unsigned)block);
  cfg.stream = s;
  cudaLaunchAttribute attr[1];
  attr[0].id = cudaLaunchAttributeCooperative;
  attr[0].val.cooperative = 1;
  cfg.attrs = attr;
  cfg.numAttrs = 1;
  if (c.dP2) {
    if (p.sp[0].mode == MODE_SSP42) return cudaLaunchKernelEx(&cfg, k_persistent_dc_cell<MODE_SSP42>, d, p, c);
    return cudaLaunchKernelEx(&cfg, k_persistent_dc_cell<MODE_RK>, d, p, c);
  }
  if (p.sp[0].mode == MODE_SSP42) return cudaLaunchKernelEx(&cfg, k_persistent_dc<MODE_SSP42>, d, p, c);
  return cudaLaunchKernelEx(&cfg, k_persistent_dc<MODE_RK>, d, p, c);
}
// one defect-correction step as tile launches (for graph capture)
// four blocks of 256 per SM: the dual-number flux fits 64 registers without
// spilling
__global__ void __launch_bounds__(256, 4) k_tiles_dc_flux(const DevView d, const DcView c, const PersistPlan p) {
  const int2 tl = p.edge_tiles[blockIdx.x];
  dc_flux_range(d, c, tl.x + threadIdx.x, tl.y, blockDim.x);
}

template <int MODE, bool FUSED>
__global__ void __launch_bounds__(256) k_tiles_dc_update(const DevView d, const DcView c, const PersistPlan p,
                                                         int stage) {
  dc_stage_tile<MODE, FUSED>(d, c, p, stage, blockIdx.x);
  if (p.sp[stage].last) tiled_case_norm(p, blockIdx.x);
}

static cudaError_t dc_tiled_step(const DevView& d, const PersistPlan& p, const DcView& c, int block, cudaStream_t s) {
  for (int k = 0; k < p.nstages; k++) {
    if (c.dP2) {
      if (p.sp[k].mode == MODE_SSP42) k_tiles_dc_update<MODE_SSP42, true><<<p.ncell_tiles, block, 0, s>>>(d, c, p, k);
      else k_tiles_dc_update<MODE_RK, true><<<p.ncell_tiles, block, 0, s>>>(d, c, p, k);
      continue;
    }
    k_tiles_dc_flux<<<p.nedge_tiles, block, 0, s>>>(d, c, p);
    if (p.sp[k].mode == MODE_SSP42) k_tiles_dc_update<MODE_SSP42, false><<<p.ncell_tiles, block, 0, s>>>(d, c, p, k);
    else k_tiles_dc_update<MODE_RK, false><<<p.ncell_tiles, block, 0, s>>>(d, c, p, k);
  }
  return cudaGetLastError();
}
#endif  // FVS_MIXED

}  // namespace FVS_NS
}  // namespace fvs
