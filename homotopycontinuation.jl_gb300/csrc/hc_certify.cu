// hc_certify.cu — certification of approximate solutions of F (the target system of the
// handle's homotopy, H at t = 0) by the Krawczyk method (Moore 1977; the reference certifies
// the same way, src/certification.jl:691-745, with the approach of Breiding, Rose and Timme,
// "Certifying zeros of polynomial systems using interval arithmetic", 2020).
//
// One warp per candidate x̃. Arithmetic: complex midpoint-radius balls (c, ρ) meaning
// {z : |z − c| ≤ ρ}; centres are computed with round-to-nearest FP64, radii with upward
// rounding and absorb the centres' rounding errors (Rump, "Verification methods: rigorous
// results using floating-point arithmetic", Acta Numerica 2010, §3):
//   |fl(a ± b) − (a ± b)| ≤ 2^-53 |fl(a ± b)|₁ ≤ 2^-52 |·|₁,
//   |fl(a·b) − a·b| ≤ 2^-51 |a|₁ |b|₁ (complex product, with or without fused multiply-adds),
// with |z|₁ = |Re z| + |Im z| ≥ |z| as the (upward-rounded) modulus bound.
//
// Steps: one Newton refinement x̃ ← x̃ − Y F(x̃) with Y ≈ J(x̃)⁻¹ (Gauss–Jordan); then for box
// radius r (up to four tries, ×4 each) the Krawczyk operator on the polydisc B = B(x̃, r),
//     K = x̃ − Y F(x̃) + (I − Y J(B)) (B − x̃),
// with F(x̃) and J(B) evaluated in ball arithmetic along the compiled monomial program.
// K ⊂ int B proves that B holds exactly one solution s, which lies in K. Real coefficients and
// conj(K) ⊂ B prove s real; |Im K_i| > ρ(K_i) for some i proves s non-real.
//
// Candidates that FP64 balls cannot certify (rounding noise of F(x̃) above what the contraction
// allows, e.g. ill-conditioned roots) are run again with double-word centres — the reference
// falls back to Arb balls of 128 bits and more (src/certification.jl:1120-1200). Double-word
// (pairs of doubles, ~106 bits) operations are the accurate algorithms of Joldes, Muller and
// Popescu, "Tight and rigorous error bounds for basic building blocks of double-word arithmetic",
// ACM TOMS 44(2), 2017: AccurateDWPlusDW (Algorithm 6, relative error ≤ 3u² + 13u³) and
// DWTimesDW3 (Algorithm 12, relative error ≤ 4u²), u = 2⁻⁵³; the radii charge 2⁻¹⁰⁰ of the
// result's modulus per operation (16 times those bounds) plus 2⁻⁹⁶⁰ absolute against underflow.
// The reported box is centred at x̃ rounded to FP64 with its radius reduced by that rounding
// (a subset of the proven box), the enclosure widened by it.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <string>
#include <vector>

#include "hc_dev.h"
#include "hc_types.cuh"

namespace hcd {
namespace {

template <class V>
struct cb_t {
  V c;
  double r;
};

__device__ __forceinline__ double absu(c64 z) { return __dadd_ru(fabs(z.re), fabs(z.im)); }

// ---- double-word centres
struct dw {
  double h, l;
};
struct cw {
  dw re, im;
};
__device__ __forceinline__ void tsum(double a, double b, double& s, double& e) {  // 2Sum
  s = __dadd_rn(a, b);
  double ap = __dsub_rn(s, b), bp = __dsub_rn(s, ap);
  e = __dadd_rn(__dsub_rn(a, ap), __dsub_rn(b, bp));
}
__device__ __forceinline__ void fsum(double a, double b, double& s, double& e) {  // Fast2Sum, |a| ≥ |b|
  s = __dadd_rn(a, b);
  e = __dsub_rn(b, __dsub_rn(s, a));
}
__device__ __forceinline__ dw dw_add(dw x, dw y) {  // AccurateDWPlusDW
  double sh, sl, th, tl, vh, vl, zh, zl;
  tsum(x.h, y.h, sh, sl);
  tsum(x.l, y.l, th, tl);
  double c = __dadd_rn(sl, th);
  fsum(sh, c, vh, vl);
  double w = __dadd_rn(tl, vl);
  fsum(vh, w, zh, zl);
  return dw{zh, zl};
}
__device__ __forceinline__ dw dw_neg(dw x) { return dw{-x.h, -x.l}; }
__device__ __forceinline__ dw dw_mul(dw x, dw y) {  // DWTimesDW3
  double ch = __dmul_rn(x.h, y.h);
  double cl1 = __fma_rn(x.h, y.h, -ch);
  double tl0 = __dmul_rn(x.l, y.l);
  double tl1 = __fma_rn(x.h, y.l, tl0);
  double cl2 = __fma_rn(x.l, y.h, tl1);
  double cl3 = __dadd_rn(cl1, cl2);
  double zh, zl;
  fsum(ch, cl3, zh, zl);
  return dw{zh, zl};
}
__device__ __forceinline__ cw cw_add(cw a, cw b) { return cw{dw_add(a.re, b.re), dw_add(a.im, b.im)}; }
__device__ __forceinline__ cw cw_sub(cw a, cw b) { return cw{dw_add(a.re, dw_neg(b.re)), dw_add(a.im, dw_neg(b.im))}; }
__device__ __forceinline__ cw cw_mul(cw a, cw b) {
  return cw{dw_add(dw_mul(a.re, b.re), dw_neg(dw_mul(a.im, b.im))), dw_add(dw_mul(a.re, b.im), dw_mul(a.im, b.re))};
}
__device__ __forceinline__ cw cw_of(c64 z) { return cw{dw{z.re, 0.0}, dw{z.im, 0.0}}; }
__device__ __forceinline__ c64 cw_round(cw z) { return C64(z.re.h, z.im.h); }
// upper bound of |z|₁ = |Re z| + |Im z|
__device__ __forceinline__ double absu(cw z) {
  return __dadd_ru(__dadd_ru(fabs(z.re.h), fabs(z.re.l)), __dadd_ru(fabs(z.im.h), fabs(z.im.l)));
}

// Ball arithmetic over a centre type: FP64 (B64) or double-word (BDW)
struct B64 {
  using V = c64;
  static constexpr int bits = 53;
  __device__ static V pt(c64 c) { return c; }
  __device__ static V zero() { return C64(0.0); }
  __device__ static c64 round(V c) { return c; }
  __device__ static double mag(V c) { return absu(c); }
  __device__ static cb_t<V> add(cb_t<V> a, cb_t<V> b) {
    V c = a.c + b.c;
    return {c, __dadd_ru(__dadd_ru(a.r, b.r), __dmul_ru(0x1p-52, absu(c)))};
  }
  __device__ static cb_t<V> sub(cb_t<V> a, cb_t<V> b) {
    V c = a.c - b.c;
    return {c, __dadd_ru(__dadd_ru(a.r, b.r), __dmul_ru(0x1p-52, absu(c)))};
  }
  __device__ static cb_t<V> mul(cb_t<V> a, cb_t<V> b) {
    V c = a.c * b.c;
    double A = absu(a.c), B = absu(b.c);
    return {c, __dadd_ru(__dadd_ru(__dmul_ru(A, b.r), __dmul_ru(a.r, B)),
                         __dadd_ru(__dmul_ru(a.r, b.r), __dmul_ru(0x1p-51, __dmul_ru(A, B))))};
  }
  __device__ static V vsub(V a, V b) { return a - b; }
  __device__ static double rnd(double m) { return __dmul_ru(0x1p-52, m); }  // rounding of a difference
};
struct BDW {
  using V = cw;
  static constexpr int bits = 106;
  __device__ static V pt(c64 c) { return cw_of(c); }
  __device__ static V zero() { return cw_of(C64(0.0)); }
  __device__ static c64 round(V c) { return cw_round(c); }
  __device__ static double mag(V c) { return absu(c); }
  __device__ static cb_t<V> add(cb_t<V> a, cb_t<V> b) {
    V c = cw_add(a.c, b.c);
    return {c, __dadd_ru(__dadd_ru(__dadd_ru(a.r, b.r), __dmul_ru(0x1p-100, absu(c))), 0x1p-960)};
  }
  __device__ static cb_t<V> sub(cb_t<V> a, cb_t<V> b) {
    V c = cw_sub(a.c, b.c);
    return {c, __dadd_ru(__dadd_ru(__dadd_ru(a.r, b.r), __dmul_ru(0x1p-100, absu(c))), 0x1p-960)};
  }
  // each component: two products and a sum, ≤ 2·2⁻¹⁰⁰ (|a_re||b_re| + |a_im||b_im|) (+ slack);
  // both components ≤ 2⁻⁹⁸ |a|₁ |b|₁
  __device__ static cb_t<V> mul(cb_t<V> a, cb_t<V> b) {
    V c = cw_mul(a.c, b.c);
    double A = absu(a.c), B = absu(b.c);
    double r = __dadd_ru(__dadd_ru(__dmul_ru(A, b.r), __dmul_ru(a.r, B)),
                         __dadd_ru(__dmul_ru(a.r, b.r), __dmul_ru(0x1p-98, __dmul_ru(A, B))));
    return {c, __dadd_ru(r, 0x1p-958)};
  }
  __device__ static V vsub(V a, V b) { return cw_sub(a, b); }
  __device__ static double rnd(double m) { return __dadd_ru(__dmul_ru(0x1p-99, m), 0x1p-960); }
};

// per-warp shared memory (byte offsets), sized on the host
struct CertLayout {
  int bytes;
  int mono, vslot, jslot, F, J, Y, M, x;
  int n2;
};

struct CertLaunch {
  DevProg P;
  CertLayout L;
  int64_t nsols;
  const double2* in;         // candidates (nsols × n, or indexed by list)
  const int64_t* list;       // null: candidate k is item k; else item k is candidate list[k]
  hc_certificate* out;       // per candidate
  double2* centers;          // per candidate × n: box centres x̃ (rounded to FP64)
  double2* enclosures;       // per candidate × n: centres of K
  int real_coefficients;
};

__device__ __forceinline__ int lane_id() { return threadIdx.x & 31; }

// monomial balls for x_i ∈ B(x_i, rho) (rho = 0: the point)
template <class A>
__device__ void mono_balls(const DevProg& P, const typename A::V* x, double rho, typename A::V* mc, double* mr) {
  const int lane = lane_id();
  if (lane == 0) {
    mc[0] = A::pt(C64(1.0));
    mr[0] = 0.0;
  }
  __syncwarp();
  for (int L = 1; L < P.nlev; ++L) {
    int b = P.lev[L], e = P.lev[L + 1];
    for (int m = b + lane; m < e; m += 32) {
      int2 d = P.mdef[m];
      auto v = A::mul({mc[d.x], mr[d.x]}, {x[d.y], rho});
      mc[m] = v.c;
      mr[m] = v.r;
    }
    __syncwarp();
  }
}

// rows of a DevRows table as balls: value rows (jac = false) use coefficient × monomial, Jacobian
// rows (jac = true) multiplier × coefficient × derivative monomial; out rows [0, nrows_out)
template <class A>
__device__ void rows_balls(const DevProg& P, const DevRows& R, bool jac, const typename A::V* mc, const double* mr,
                           typename A::V* sc, double* sr, int nrows_out, typename A::V* oc, double* orr) {
  const int lane = lane_id();
  for (int s = R.lane_seg[lane]; s < R.lane_seg[lane + 1]; ++s) {
    int4 g = R.seg[s];
    cb_t<typename A::V> acc{A::zero(), 0.0};
    const int mult = (g.w >> 24) & 0xff;
    for (int t = g.y; t < g.z; t += g.x) {
      int m, vt;
      if (jac) {
        uint32_t code = P.jcode[t];
        m = code & 0xffff;
        vt = code >> 16;
      } else {
        m = P.vmono[t];
        vt = t;
      }
      double2 cf = P.vcoef64[vt];
      acc = A::add(acc, A::mul({A::pt(C64(cf.x, cf.y)), 0.0}, {mc[m], mr[m]}));
    }
    if (jac && mult != 1) acc = A::mul(acc, {A::pt(C64((double)mult)), 0.0});
    int slot = g.w & 0xffffff;
    sc[slot] = acc.c;
    sr[slot] = acc.r;
  }
  __syncwarp();
  for (int r = lane; r < nrows_out; r += 32) {
    cb_t<typename A::V> acc{A::zero(), 0.0};
    for (int k = R.row_slot[r]; k < R.row_slot[r + 1]; ++k) acc = A::add(acc, {sc[k], sr[k]});
    oc[r] = acc.c;
    orr[r] = acc.r;
  }
  __syncwarp();
}

// Y = A⁻¹ by Gauss–Jordan with partial pivoting (lane 0; n ≤ 32); A (column-major: A[j*n+i] =
// ∂F_i/∂x_j) is destroyed. Returns false if a pivot vanishes.
__device__ bool invert(c64* A, c64* Y, int n) {
  bool ok = true;
  if (lane_id() == 0) {
    for (int i = 0; i < n; ++i)
      for (int j = 0; j < n; ++j) Y[j * n + i] = C64(i == j ? 1.0 : 0.0);
    for (int k = 0; k < n && ok; ++k) {
      int p = k;
      double best = abs2(A[k * n + k]);
      for (int i = k + 1; i < n; ++i) {
        double v = abs2(A[k * n + i]);
        if (v > best) {
          best = v;
          p = i;
        }
      }
      if (!(best > 0.0) || !isfinite(best)) {
        ok = false;
        break;
      }
      if (p != k)
        for (int j = 0; j < n; ++j) {
          c64 t = A[j * n + k];
          A[j * n + k] = A[j * n + p];
          A[j * n + p] = t;
          t = Y[j * n + k];
          Y[j * n + k] = Y[j * n + p];
          Y[j * n + p] = t;
        }
      c64 inv = div_fast(C64(1.0), A[k * n + k]);
      for (int j = 0; j < n; ++j) {
        A[j * n + k] = A[j * n + k] * inv;
        Y[j * n + k] = Y[j * n + k] * inv;
      }
      for (int i = 0; i < n; ++i) {
        if (i == k) continue;
        c64 f = A[k * n + i];
        if (f.re == 0.0 && f.im == 0.0) continue;
        for (int j = 0; j < n; ++j) {
          A[j * n + i] = A[j * n + i] - f * A[j * n + k];
          Y[j * n + i] = Y[j * n + i] - f * Y[j * n + k];
        }
      }
    }
  }
  return __shfl_sync(FULL, ok ? 1 : 0, 0) != 0;
}

template <class A>
__global__ void __launch_bounds__(32) certify_kernel(const __grid_constant__ CertLaunch cl) {
  using V = typename A::V;
  extern __shared__ __align__(16) char smem[];
  const DevProg& P = cl.P;
  const CertLayout& L = cl.L;
  const int n = P.n, n2 = n * n, lane = lane_id();
  V* mc = (V*)(smem + L.mono);
  double* mr = (double*)(mc + P.M);
  V* vsc = (V*)(smem + L.vslot);
  double* vsr = (double*)(vsc + P.val.nslots);
  V* jsc = (V*)(smem + L.jslot);
  double* jsr = (double*)(jsc + P.jac.nslots);
  V* Fc = (V*)(smem + L.F);
  double* Fr = (double*)(Fc + 2 * n);
  V* Jc = (V*)(smem + L.J);
  double* Jr = (double*)(Jc + 2 * n2);
  c64* Y = (c64*)(smem + L.Y);
  c64* J64 = Y + n2;  // FP64 copy of the Jacobian's centres for the inversion
  V* Mc = (V*)(smem + L.M);
  double* Mr = (double*)(Mc + n2);
  V* x = (V*)(smem + L.x);
  V* kc = x + n;
  for (int64_t item = blockIdx.x; item < cl.nsols; item += gridDim.x) {
    const int64_t k = cl.list ? cl.list[item] : item;
    for (int i = lane; i < n; i += 32) x[i] = A::pt(C64(cl.in[k * n + i].x, cl.in[k * n + i].y));
    __syncwarp();
    bool ok = true;
    // Newton refinement of the centre in the centre arithmetic, then Y at the refined point:
    // one step with FP64 centres; with double-word centres up to 8, until the step is below
    // 2⁻¹⁰⁰ of x̃ (the reference refines to machine precision with extended-precision
    // residuals before certifying, src/certification.jl:1040-1056: up to 8 iterations)
    const int maxit = A::bits > 53 ? 8 : 1;
    for (int it = 0; ok; ++it) {
      mono_balls<A>(P, x, 0.0, mc, mr);
      rows_balls<A>(P, P.val, false, mc, mr, vsc, vsr, n, Fc, Fr);
      rows_balls<A>(P, P.jac, true, mc, mr, jsc, jsr, n2, Jc, Jr);
      for (int e = lane; e < n2; e += 32) J64[e] = A::round(Jc[e]);
      __syncwarp();
      ok = invert(J64, Y, n);
      if (!ok || it == maxit) break;
      double step = 0.0, size = 0.0;
      for (int i = lane; i < n; i += 32) {
        cb_t<V> d{A::zero(), 0.0};
        for (int j = 0; j < n; ++j) d = A::add(d, A::mul({A::pt(Y[j * n + i]), 0.0}, {Fc[j], 0.0}));
        x[i] = A::vsub(x[i], d.c);
        step = fmax(step, A::mag(d.c));
        size = fmax(size, A::mag(x[i]));
      }
      for (int o = 16; o; o >>= 1) {
        step = fmax(step, __shfl_xor_sync(FULL, step, o));
        size = fmax(size, __shfl_xor_sync(FULL, size, o));
      }
      __syncwarp();
      if (A::bits > 53 && !(step > 0x1p-100 * size)) it = maxit - 1;  // converged: Y at this point
    }
    hc_certificate C;
    C.certified = 0;
    C.realness = 0;
    C.precision = A::bits;
    C.reserved = 0;
    C.radius = 0.0;
    C.enclosure = 0.0;
    if (ok) {
      // YF = Y F(x̃) in balls: centre (vector per lane i), radius
      cb_t<V> yf{A::zero(), 0.0};
      double xnorm = 0.0, delta = 0.0;
      for (int i = 0; i < n; ++i) xnorm = fmax(xnorm, A::mag(x[i]));
      if (lane < n) {
        for (int j = 0; j < n; ++j) yf = A::add(yf, A::mul({A::pt(Y[j * n + lane]), 0.0}, {Fc[j], Fr[j]}));
        delta = __dadd_ru(A::mag(yf.c), yf.r);
      }
      for (int o = 16; o; o >>= 1) delta = fmax(delta, __shfl_xor_sync(FULL, delta, o));
      // the smallest box: 8‖YF‖ plus a floor at the centre arithmetic's resolution, and at
      // least 8 times the rounding of x̃ to FP64, so that the reported box (around x̃ rounded,
      // shrunk by that rounding) keeps a positive radius
      double dx0 = 0.0;
      for (int i = lane; i < n; i += 32) dx0 = fmax(dx0, A::mag(A::vsub(x[i], A::pt(A::round(x[i])))));
      for (int o = 16; o; o >>= 1) dx0 = fmax(dx0, __shfl_xor_sync(FULL, dx0, o));
      double r = __dadd_ru(__dmul_ru(8.0, delta), __dmul_ru(A::bits > 53 ? 0x1p-96 : 0x1p-45, fmax(xnorm, 1.0)));
      r = fmax(r, __dmul_ru(8.0, dx0));
      for (int attempt = 0; attempt < 4; ++attempt, r = __dmul_ru(r, 4.0)) {
        mono_balls<A>(P, x, r, mc, mr);
        rows_balls<A>(P, P.jac, true, mc, mr, jsc, jsr, n2, Jc, Jr);
        // M = I − Y J(B)
        for (int e = lane; e < n2; e += 32) {
          int i = e % n, j = e / n;
          cb_t<V> acc{A::pt(C64(i == j ? 1.0 : 0.0)), 0.0};
          for (int q = 0; q < n; ++q)
            acc = A::sub(acc, A::mul({A::pt(Y[q * n + i]), 0.0}, {Jc[j * n + q], Jr[j * n + q]}));
          Mc[e] = acc.c;
          Mr[e] = acc.r;
        }
        __syncwarp();
        int inside = 1, real_in = cl.real_coefficients ? 1 : 0, nonreal = 0;
        double encl = 0.0;
        if (lane < n) {
          double v = 0.0;
          for (int j = 0; j < n; ++j) v = __dadd_ru(v, __dadd_ru(A::mag(Mc[j * n + lane]), Mr[j * n + lane]));
          // K_i = x̃_i − YF_i + M_i·B(0, r)
          V kcen = A::vsub(x[lane], yf.c);
          double krad = __dadd_ru(__dadd_ru(yf.r, __dmul_ru(v, r)), A::rnd(A::mag(kcen)));
          V dk = A::vsub(kcen, x[lane]);
          double dist = __dadd_ru(A::mag(dk), A::rnd(__dadd_ru(A::mag(kcen), A::mag(x[lane]))));
          inside = __dadd_ru(dist, krad) < r ? 1 : 0;
          V ck = kcen;
          if constexpr (A::bits > 53) {
            ck.im = dw_neg(ck.im);
          } else {
            ck = conj(kcen);
          }
          V dc = A::vsub(ck, x[lane]);
          double cdist = __dadd_ru(A::mag(dc), A::rnd(__dadd_ru(A::mag(ck), A::mag(x[lane]))));
          if (!(__dadd_ru(cdist, krad) < r)) real_in = 0;
          const c64 k64 = A::round(kcen);
          nonreal = fabs(k64.im) > __dadd_ru(__dadd_ru(krad, A::rnd(A::mag(kcen))), A::mag(A::vsub(kcen, A::pt(k64))))
                        ? 1
                        : 0;
          kc[lane] = kcen;
          encl = krad;
        }
        inside = __all_sync(FULL, inside);
        real_in = __all_sync(FULL, real_in);
        nonreal = __any_sync(FULL, nonreal);
        for (int o = 16; o; o >>= 1) encl = fmax(encl, __shfl_xor_sync(FULL, encl, o));
        __syncwarp();
        if (inside) {
          C.certified = 1;
          C.realness = real_in ? 1 : (nonreal ? 2 : 0);
          // reported in FP64: the box around x̃ rounded, shrunk by that rounding (a subset of the
          // proven box); K around its centre rounded, widened by it
          double dx = 0.0, dk = 0.0;
          for (int i = lane; i < n; i += 32) {
            dx = fmax(dx, A::mag(A::vsub(x[i], A::pt(A::round(x[i])))));
            dk = fmax(dk, A::mag(A::vsub(kc[i], A::pt(A::round(kc[i])))));
          }
          for (int o = 16; o; o >>= 1) {
            dx = fmax(dx, __shfl_xor_sync(FULL, dx, o));
            dk = fmax(dk, __shfl_xor_sync(FULL, dk, o));
          }
          C.radius = __dsub_rd(r, dx);
          C.enclosure = __dadd_ru(encl, dk);
          break;
        }
      }
    }
    for (int i = lane; i < n; i += 32) {
      const c64 xi = A::round(x[i]), ki = C.certified ? A::round(kc[i]) : xi;
      cl.centers[k * n + i] = make_double2(xi.re, xi.im);
      cl.enclosures[k * n + i] = make_double2(ki.re, ki.im);
    }
    if (lane == 0) cl.out[k] = C;
    __syncwarp();
  }
}

}  // namespace

// host side: layout and launch (called from hc_capi.cu with the handle's program)
static CertLayout make_layout(const DevProg& P, bool dw) {
  CertLayout L{};
  size_t off = 0;
  auto take = [&](size_t b) {
    size_t o = off;
    off += (b + 15) & ~(size_t)15;
    return (int)o;
  };
  const size_t ball = (dw ? sizeof(cw) : sizeof(c64)) + sizeof(double), cen = dw ? sizeof(cw) : sizeof(c64);
  const int n = P.n, n2 = n * n;
  L.mono = take((size_t)P.M * ball);
  L.vslot = take((size_t)P.val.nslots * ball);
  L.jslot = take((size_t)P.jac.nslots * ball);
  L.F = take((size_t)2 * n * ball);
  L.J = take((size_t)2 * n2 * ball);
  L.Y = take((size_t)2 * n2 * sizeof(c64));
  L.M = take((size_t)n2 * ball);
  L.x = take((size_t)2 * n * cen);
  L.bytes = (int)off;
  L.n2 = n2;
  return L;
}

int certify_layout(const DevProg& P, int* bytes_out) {
  CertLayout L = make_layout(P, true);  // the double-word pass needs the most
  *bytes_out = L.bytes;
  return L.bytes <= 227 * 1024 ? 0 : 1;
}

cudaError_t launch_certify(const DevProg& P, int64_t nitems, const int64_t* d_list, bool dw, const double* d_in,
                           hc_certificate* d_out, double* d_centers, double* d_enclosures, int real_coefficients,
                           int num_sms, cudaStream_t stream) {
  CertLaunch cl{};
  cl.P = P;
  cl.L = make_layout(P, dw);
  cl.nsols = nitems;
  cl.list = d_list;
  cl.in = (const double2*)d_in;
  cl.out = d_out;
  cl.centers = (double2*)d_centers;
  cl.enclosures = (double2*)d_enclosures;
  cl.real_coefficients = real_coefficients;
  const int bytes = cl.L.bytes;
  const void* fn = dw ? (const void*)certify_kernel<BDW> : (const void*)certify_kernel<B64>;
  cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, 32, bytes);
  if (e != cudaSuccess) return e;
  int blocks = (int)std::min<int64_t>(nitems, (int64_t)std::max(1, per_sm) * num_sms);
  if (dw)
    certify_kernel<BDW><<<blocks, 32, bytes, stream>>>(cl);
  else
    certify_kernel<B64><<<blocks, 32, bytes, stream>>>(cl);
  return cudaGetLastError();
}

}  // namespace hcd
