// hc_types.cuh — complex FP64/FP32 and double-double arithmetic plus warp primitives for
// the path-tracking kernel. Complex products use the plain formula (ac-bd, ad+bc) and the
// @fastmath division of the reference's LU (src/linear_algebra.jl:171, :288); regular
// divisions use Smith's algorithm. Double-double routines restate src/DoubleDouble.jl:14-66,
// 166-266 with explicitly rounded operations (__dadd_rn/__dmul_rn) so that nvcc cannot fuse
// the error-free transforms into FMAs.
#pragma once
#include "hc_rtc.h"
#ifndef __CUDACC_RTC__
#include <cuda_runtime.h>
#endif

namespace hcd {

constexpr unsigned FULL = 0xffffffffu;
__device__ __forceinline__ double dINF() { return __longlong_as_double(0x7ff0000000000000LL); }
__device__ __forceinline__ double dNaN() { return __longlong_as_double(0x7ff8000000000000LL); }
constexpr double EPS = 2.220446049250313e-16;

// ---------------------------------------------------------------- complex types
struct c64 {
  double re, im;
};
struct c32 {
  float re, im;
};
__device__ __forceinline__ c64 C64(double r, double i = 0.0) { return c64{r, i}; }
__device__ __forceinline__ c32 C32(float r, float i = 0.f) { return c32{r, i}; }

#define HC_COMPLEX_OPS(T, R)                                                                       \
  __device__ __forceinline__ T operator+(T a, T b) { return T{a.re + b.re, a.im + b.im}; }        \
  __device__ __forceinline__ T operator-(T a, T b) { return T{a.re - b.re, a.im - b.im}; }        \
  __device__ __forceinline__ T operator-(T a) { return T{-a.re, -a.im}; }                         \
  __device__ __forceinline__ T operator*(T a, T b) {                                              \
    return T{a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};                               \
  }                                                                                               \
  __device__ __forceinline__ T operator*(R s, T a) { return T{s * a.re, s * a.im}; }              \
  __device__ __forceinline__ T operator*(T a, R s) { return T{a.re * s, a.im * s}; }              \
  __device__ __forceinline__ T operator/(T a, R s) { return T{a.re / s, a.im / s}; }              \
  __device__ __forceinline__ R abs2(T a) { return a.re * a.re + a.im * a.im; }                    \
  __device__ __forceinline__ T conj(T a) { return T{a.re, -a.im}; }                               \
  __device__ __forceinline__ T div_fast(T a, T b) {                                               \
    R d = b.re * b.re + b.im * b.im;                                                              \
    return T{(a.re * b.re + a.im * b.im) / d, (a.im * b.re - a.re * b.im) / d};                   \
  }
HC_COMPLEX_OPS(c64, double)
HC_COMPLEX_OPS(c32, float)

// acc + a·b and acc − a·b with two fused multiply-adds per component (4 per complex op;
// the operator form compiles to a multiply, a multiply-add and an add per component)
__device__ __forceinline__ c64 cfma(c64 a, c64 b, c64 acc) {
  return c64{fma(a.re, b.re, fma(-a.im, b.im, acc.re)), fma(a.re, b.im, fma(a.im, b.re, acc.im))};
}
__device__ __forceinline__ c32 cfma(c32 a, c32 b, c32 acc) {
  return c32{fmaf(a.re, b.re, fmaf(-a.im, b.im, acc.re)), fmaf(a.re, b.im, fmaf(a.im, b.re, acc.im))};
}
__device__ __forceinline__ c64 cfms(c64 a, c64 b, c64 acc) {
  return c64{fma(-a.re, b.re, fma(a.im, b.im, acc.re)), fma(-a.re, b.im, fma(-a.im, b.re, acc.im))};
}
__device__ __forceinline__ c32 cfms(c32 a, c32 b, c32 acc) {
  return c32{fmaf(-a.re, b.re, fmaf(a.im, b.im, acc.re)), fmaf(-a.re, b.im, fmaf(-a.im, b.re, acc.im))};
}

// Out of line (here and below): the scalar control code calls these at many sites, and one
// copy per kernel instead of one per site keeps the code a step runs small enough for the
// instruction cache. The results are those of the inlined forms.
static __device__ __noinline__ double fast_abs(c64 a) { return sqrt(abs2(a)); }
__device__ __forceinline__ double cabs(c64 a) { return hypot(a.re, a.im); }
__device__ __forceinline__ bool isnanc(c64 a) { return isnan(a.re) || isnan(a.im); }
__device__ __forceinline__ c64 to64(c32 a) { return c64{(double)a.re, (double)a.im}; }
__device__ __forceinline__ c64 to64(c64 a) { return a; }
__device__ __forceinline__ c32 to32(c64 a) { return c32{(float)a.re, (float)a.im}; }
template <class T>
__device__ __forceinline__ T conv(c64 a);
template <>
__device__ __forceinline__ c64 conv<c64>(c64 a) {
  return a;
}
template <>
__device__ __forceinline__ c32 conv<c32>(c64 a) {
  return to32(a);
}

// Smith's algorithm for a regular complex division
static __device__ __noinline__ c64 cdiv(c64 a, c64 b) {
  if (fabs(b.re) >= fabs(b.im)) {
    if (b.re == 0.0 && b.im == 0.0) return c64{a.re / 0.0, a.im / 0.0};
    double r = b.im / b.re, den = b.re + b.im * r;
    return c64{(a.re + a.im * r) / den, (a.im - a.re * r) / den};
  } else {
    double r = b.re / b.im, den = b.re * r + b.im;
    return c64{(a.re * r + a.im) / den, (a.im * r - a.re) / den};
  }
}
static __device__ __noinline__ c64 cis(double th) {
  double s, c;
  sincos(th, &s, &c);
  return c64{c, s};
}

// Julia semantics of max/min (NaN propagating), @fastmath max and clamp
__device__ __forceinline__ double jmax(double a, double b) {
  if (isnan(a) || isnan(b)) return dNaN();
  return a > b ? a : b;
}
__device__ __forceinline__ double jmin(double a, double b) {
  if (isnan(a) || isnan(b)) return dNaN();
  return a < b ? a : b;
}
__device__ __forceinline__ double max_fast(double a, double b) { return a > b ? a : b; }
__device__ __forceinline__ double jclamp(double x, double lo, double hi) {
  return x > hi ? hi : (x < lo ? lo : x);
}
__device__ __forceinline__ double nanmin(double a, double b) {
  return isnan(a) ? b : (isnan(b) ? a : fmin(a, b));
}
__device__ __forceinline__ double nanmax(double a, double b) {
  return isnan(a) ? b : (isnan(b) ? a : fmax(a, b));
}
static __device__ __noinline__ double hc_log(double x) { return log(x); }
static __device__ __noinline__ double hc_exp(double x) { return exp(x); }
static __device__ __noinline__ double hc_pow(double x, double y) { return pow(x, y); }
static __device__ __noinline__ double hc_atan2(double y, double x) { return atan2(y, x); }
static __device__ __noinline__ double nthroot(double x, int N) {  // src/utils.jl:408-422
  if (N == 4) return sqrt(sqrt(x));
  if (N == 2) return sqrt(x);
  if (N == 3) return cbrt(x);
  if (N == 1) return x;
  if (N == 0) return 1.0;
  return pow(x, 1.0 / N);
}

// ---------------------------------------------------------------- double-double
struct ddv {
  double hi, lo;
};
__device__ __forceinline__ void quick_two_sum(double a, double b, double& s, double& e) {
  s = __dadd_rn(a, b);
  e = __dsub_rn(b, __dsub_rn(s, a));
}
__device__ __forceinline__ void two_sum(double a, double b, double& s, double& e) {
  s = __dadd_rn(a, b);
  double v = __dsub_rn(s, a);
  e = __dadd_rn(__dsub_rn(a, __dsub_rn(s, v)), __dsub_rn(b, v));
}
__device__ __forceinline__ void two_diff(double a, double b, double& s, double& e) {
  s = __dsub_rn(a, b);
  double v = __dsub_rn(s, a);
  e = __dsub_rn(__dsub_rn(a, __dsub_rn(s, v)), __dadd_rn(b, v));
}
__device__ __forceinline__ ddv dd_of(double x) { return ddv{x, isinf(x) ? x : 0.0}; }
__device__ __forceinline__ ddv operator+(ddv a, ddv b) {
  double hi, lo;
  two_sum(a.hi, b.hi, hi, lo);
  lo = __dadd_rn(lo, __dadd_rn(a.lo, b.lo));
  quick_two_sum(hi, lo, hi, lo);
  return ddv{hi, lo};
}
__device__ __forceinline__ ddv operator-(ddv a, ddv b) {
  double hi, lo;
  two_diff(a.hi, b.hi, hi, lo);
  lo = __dadd_rn(lo, a.lo);
  lo = __dsub_rn(lo, b.lo);
  quick_two_sum(hi, lo, hi, lo);
  return ddv{hi, lo};
}
__device__ __forceinline__ ddv operator*(ddv a, ddv b) {
  double p1 = __dmul_rn(a.hi, b.hi);
  double p2 = fma(a.hi, b.hi, -p1);
  p2 = __dadd_rn(p2, __dadd_rn(__dmul_rn(a.hi, b.lo), __dmul_rn(a.lo, b.hi)));
  quick_two_sum(p1, p2, p1, p2);
  return ddv{p1, p2};
}
struct cdd {
  ddv re, im;
};
__device__ __forceinline__ cdd cdd_of(c64 a) { return cdd{dd_of(a.re), dd_of(a.im)}; }
__device__ __forceinline__ cdd operator+(cdd a, cdd b) { return cdd{a.re + b.re, a.im + b.im}; }
__device__ __forceinline__ cdd operator-(cdd a, cdd b) { return cdd{a.re - b.re, a.im - b.im}; }
__device__ __forceinline__ cdd operator*(cdd a, cdd b) {
  return cdd{a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
__device__ __forceinline__ c64 round_c(cdd a) { return c64{a.re.hi, a.im.hi}; }

// ---------------------------------------------------------------- warp primitives
__device__ __forceinline__ c64 shfl(c64 v, int src) {
  return c64{__shfl_sync(FULL, v.re, src), __shfl_sync(FULL, v.im, src)};
}
__device__ __forceinline__ c32 shfl(c32 v, int src) {
  return c32{__shfl_sync(FULL, v.re, src), __shfl_sync(FULL, v.im, src)};
}
__device__ __forceinline__ double wsum(double v) {
#pragma unroll
  for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
  return v;
}
__device__ __forceinline__ double wmax_plain(double v) {  // no NaN inputs
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    double u = __shfl_xor_sync(FULL, v, o);
    v = u > v ? u : v;
  }
  return v;
}
__device__ __forceinline__ int wmax_int(int v) {
#pragma unroll
  for (int o = 16; o; o >>= 1) v = max(v, __shfl_xor_sync(FULL, v, o));
  return v;
}
// Julia's sequential `m = d[0]; for i ≥ 1: m = max_fast(m, d[i])` over lanes 0..n-1:
// a NaN resets the running maximum, so the result is NaN if d[n-1] is NaN and otherwise the
// maximum of the entries after the last NaN.
__device__ __forceinline__ double wseq_max_fast(double d, int lane, int n) {
  int kn = wmax_int((lane < n && isnan(d)) ? lane : -1);
  if (kn == n - 1) return dNaN();
  double v = (lane < n && lane > kn) ? d : -dINF();
  return wmax_plain(v);
}
// Julia `maximum` (NaN propagating) over lanes 0..n-1
__device__ __forceinline__ double wjmax(double d, int lane, int n) {
  unsigned anynan = __ballot_sync(FULL, lane < n && isnan(d));
  if (anynan) return dNaN();
  return wmax_plain(lane < n ? d : -dINF());
}
__device__ __forceinline__ float wjmaxf(float d, int lane, int n) {
  unsigned anynan = __ballot_sync(FULL, lane < n && isnan(d));
  if (anynan) return __int_as_float(0x7fc00000);
  float v = lane < n ? d : -__int_as_float(0x7f800000);
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    float u = __shfl_xor_sync(FULL, v, o);
    v = u > v ? u : v;
  }
  return v;
}

}  // namespace hcd
