// hc_slp_ops.cuh — scalar operations of the straight-line programs that hc_slp.cu turns into
// CUDA C (ModelKit's op semantics, src/model_kit/operations.jl:183-248), for the three
// arithmetics of the tracker: complex FP64 (c64), complex FP32 (c32) and complex double-double
// (cdd, the extended-precision residual). Division and inversion are the reference's fast
// forms, a·conj(b)/|b|² (op_div = div_fast, op_inv = inv_fast).
#pragma once
#include "hc_types.cuh"

namespace hcslp {
using hcd::c32;
using hcd::c64;
using hcd::cdd;
using hcd::ddv;

// ---- constants
template <class T>
__device__ __forceinline__ T kc(double re, double im);
template <>
__device__ __forceinline__ c64 kc<c64>(double re, double im) {
  return c64{re, im};
}
template <>
__device__ __forceinline__ c32 kc<c32>(double re, double im) {
  return c32{(float)re, (float)im};
}
template <>
__device__ __forceinline__ cdd kc<cdd>(double re, double im) {
  return hcd::cdd_of(c64{re, im});
}
// a variable x_j (FP64 in the tracker) in arithmetic T
template <class T>
__device__ __forceinline__ T var(hcd::c64 x);
template <>
__device__ __forceinline__ c64 var<c64>(c64 x) {
  return x;
}
template <>
__device__ __forceinline__ c32 var<c32>(c64 x) {
  return hcd::to32(x);
}
template <>
__device__ __forceinline__ cdd var<cdd>(c64 x) {
  return hcd::cdd_of(x);
}
// parameter k of a parameter homotopy at t: t p + (1 - t) q (tp!,
// src/homotopies/parameter_homotopy.jl:64-87; real t in real arithmetic, as there)
__device__ __forceinline__ c64 param_at(c64 p, c64 q, c64 t) {
  if (t.im == 0.0) {
    const double s = t.re, r = 1.0 - t.re;
    return c64{s * p.re + r * q.re, s * p.im + r * q.im};
  }
  return t * p + (c64{1.0, 0.0} - t) * q;
}
// 1 when sel, else 0 (the seed of a tangent)
template <class T>
__device__ __forceinline__ T unit(bool sel) {
  return kc<T>(sel ? 1.0 : 0.0, 0.0);
}

// ---- double-double helpers (division restated from the standard long-division scheme:
// quotient digits q1 = a/b, q2 = (a - q1 b)/b, q3 likewise, renormalised)
__device__ __forceinline__ ddv dd_neg(ddv a) { return ddv{-a.hi, -a.lo}; }
__device__ __forceinline__ ddv dd_mul_d(ddv a, double b) { return a * hcd::dd_of(b); }
__device__ __forceinline__ ddv dd_div(ddv a, ddv b) {
  double q1 = a.hi / b.hi;
  ddv r = a - dd_mul_d(b, q1);
  double q2 = r.hi / b.hi;
  r = r - dd_mul_d(b, q2);
  double q3 = r.hi / b.hi;
  double s, e;
  hcd::quick_two_sum(q1, q2, s, e);
  return ddv{s, e} + hcd::dd_of(q3);
}

// ---- arithmetic on c64 / c32 (operators from hc_types.cuh) and cdd
__device__ __forceinline__ cdd operator-(cdd a) { return cdd{dd_neg(a.re), dd_neg(a.im)}; }

__device__ __forceinline__ c64 sdiv(c64 a, c64 b) { return hcd::div_fast(a, b); }
__device__ __forceinline__ c32 sdiv(c32 a, c32 b) { return hcd::div_fast(a, b); }
__device__ __forceinline__ cdd sdiv(cdd a, cdd b) {
  ddv d = b.re * b.re + b.im * b.im;
  return cdd{dd_div(a.re * b.re + a.im * b.im, d), dd_div(a.im * b.re - a.re * b.im, d)};
}
template <class T>
__device__ __forceinline__ T sinv(T a) {
  return sdiv(kc<T>(1.0, 0.0), a);
}

// complex square root, principal branch: with r = |z|, t = sqrt((r + |re z|)/2)
__device__ __forceinline__ c64 csqrt64(c64 z) {
  if (z.re == 0.0 && z.im == 0.0) return c64{0.0, z.im};
  double r = hypot(z.re, z.im);
  double t = sqrt(0.5 * (r + fabs(z.re)));
  if (z.re >= 0.0) return c64{t, z.im / (2.0 * t)};
  return c64{fabs(z.im) / (2.0 * t), copysign(t, z.im)};
}
__device__ __forceinline__ c64 ssqrt(c64 a) { return csqrt64(a); }
__device__ __forceinline__ c32 ssqrt(c32 a) { return hcd::to32(csqrt64(hcd::to64(a))); }
// double-double: the FP64 root s refined by one Newton step s + (a - s²)/(2s), the correction
// taken in FP64 (it is of the order of s's rounding error)
__device__ __forceinline__ cdd ssqrt(cdd a) {
  c64 s = csqrt64(hcd::round_c(a));
  if (s.re == 0.0 && s.im == 0.0) return hcd::cdd_of(s);
  cdd sd = hcd::cdd_of(s);
  c64 r = hcd::round_c(a - sd * sd);
  return sd + hcd::cdd_of(hcd::div_fast(r, c64{2.0 * s.re, 2.0 * s.im}));
}

__device__ __forceinline__ bool is_zero(c64 a) { return a.re == 0.0 && a.im == 0.0; }
__device__ __forceinline__ bool is_zero(c32 a) { return a.re == 0.f && a.im == 0.f; }
__device__ __forceinline__ bool is_zero(cdd a) { return a.re.hi == 0.0 && a.im.hi == 0.0; }

// a · k for a small integer k (derivative factors)
__device__ __forceinline__ c64 smul(c64 a, int k) { return c64{a.re * k, a.im * k}; }
__device__ __forceinline__ c32 smul(c32 a, int k) { return c32{a.re * (float)k, a.im * (float)k}; }
__device__ __forceinline__ cdd smul(cdd a, int k) {
  ddv d = hcd::dd_of((double)k);
  return cdd{a.re * d, a.im * d};
}

// x^p by repeated squaring (op_pow_int: power_by_squaring, inverted for p < 0)
template <class T>
__device__ __forceinline__ T spow(T a, int p) {
  bool neg = p < 0;
  unsigned q = neg ? (unsigned)(-p) : (unsigned)p;
  T r = kc<T>(1.0, 0.0), b = a;
  bool first = true;
  while (q) {
    if (q & 1u) {
      r = first ? b : r * b;
      first = false;
    }
    q >>= 1;
    if (q) b = b * b;
  }
  return neg ? sinv(r) : r;
}

}  // namespace hcslp
