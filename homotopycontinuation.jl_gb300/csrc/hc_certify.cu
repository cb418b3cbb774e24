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
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <string>
#include <vector>

#include "hc_dev.h"
#include "hc_types.cuh"

namespace hcd {
namespace {

struct cb {
  c64 c;
  double r;
};

__device__ __forceinline__ double absu(c64 z) { return __dadd_ru(fabs(z.re), fabs(z.im)); }
__device__ __forceinline__ cb cb_point(c64 c) { return cb{c, 0.0}; }
__device__ __forceinline__ cb cb_add(cb a, cb b) {
  c64 c = a.c + b.c;
  return cb{c, __dadd_ru(__dadd_ru(a.r, b.r), __dmul_ru(0x1p-52, absu(c)))};
}
__device__ __forceinline__ cb cb_sub(cb a, cb b) {
  c64 c = a.c - b.c;
  return cb{c, __dadd_ru(__dadd_ru(a.r, b.r), __dmul_ru(0x1p-52, absu(c)))};
}
__device__ __forceinline__ cb cb_mul(cb a, cb b) {
  c64 c = a.c * b.c;
  double A = absu(a.c), B = absu(b.c);
  double r = __dadd_ru(__dadd_ru(__dmul_ru(A, b.r), __dmul_ru(a.r, B)),
                       __dadd_ru(__dmul_ru(a.r, b.r), __dmul_ru(0x1p-51, __dmul_ru(A, B))));
  return cb{c, r};
}

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
  const double2* in;         // nsols × n candidates
  hc_certificate* out;       // nsols
  double2* centers;          // nsols × n: refined box centres x̃
  double2* enclosures;       // nsols × n: centres of K
  int real_coefficients;
};

__device__ __forceinline__ int lane_id() { return threadIdx.x & 31; }

// monomial balls for x_i ∈ B(x_i, rho) (rho = 0: the point)
__device__ void mono_balls(const DevProg& P, const c64* x, double rho, c64* mc, double* mr) {
  const int lane = lane_id();
  if (lane == 0) {
    mc[0] = C64(1.0);
    mr[0] = 0.0;
  }
  __syncwarp();
  for (int L = 1; L < P.nlev; ++L) {
    int b = P.lev[L], e = P.lev[L + 1];
    for (int m = b + lane; m < e; m += 32) {
      int2 d = P.mdef[m];
      cb v = cb_mul(cb{mc[d.x], mr[d.x]}, cb{x[d.y], rho});
      mc[m] = v.c;
      mr[m] = v.r;
    }
    __syncwarp();
  }
}

// rows of a DevRows table as balls: value rows (jac = false) use coefficient × monomial, Jacobian
// rows (jac = true) multiplier × coefficient × derivative monomial; out rows [0, nrows_out)
__device__ void rows_balls(const DevProg& P, const DevRows& R, bool jac, const c64* mc, const double* mr,
                           c64* sc, double* sr, int nrows_out, c64* oc, double* orr) {
  const int lane = lane_id();
  for (int s = R.lane_seg[lane]; s < R.lane_seg[lane + 1]; ++s) {
    int4 g = R.seg[s];
    cb acc = cb_point(C64(0.0));
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
      acc = cb_add(acc, cb_mul(cb_point(C64(cf.x, cf.y)), cb{mc[m], mr[m]}));
    }
    if (jac && mult != 1) acc = cb_mul(acc, cb_point(C64((double)mult)));
    int slot = g.w & 0xffffff;
    sc[slot] = acc.c;
    sr[slot] = acc.r;
  }
  __syncwarp();
  for (int r = lane; r < nrows_out; r += 32) {
    cb acc = cb_point(C64(0.0));
    for (int k = R.row_slot[r]; k < R.row_slot[r + 1]; ++k) acc = cb_add(acc, cb{sc[k], sr[k]});
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

__global__ void __launch_bounds__(32) certify_kernel(const __grid_constant__ CertLaunch cl) {
  extern __shared__ __align__(16) char smem[];
  const DevProg& P = cl.P;
  const CertLayout& L = cl.L;
  const int n = P.n, n2 = n * n, lane = lane_id();
  c64* mc = (c64*)(smem + L.mono);
  double* mr = (double*)(mc + P.M);
  c64* vsc = (c64*)(smem + L.vslot);
  double* vsr = (double*)(vsc + P.val.nslots);
  c64* jsc = (c64*)(smem + L.jslot);
  double* jsr = (double*)(jsc + P.jac.nslots);
  c64* Fc = (c64*)(smem + L.F);
  double* Fr = (double*)(Fc + 2 * n);
  c64* Jc = (c64*)(smem + L.J);
  double* Jr = (double*)(Jc + 2 * n2);
  c64* Y = (c64*)(smem + L.Y);
  c64* Mc = (c64*)(smem + L.M);
  double* Mr = (double*)(Mc + n2);
  c64* x = (c64*)(smem + L.x);
  c64* kc = x + n;
  for (int64_t k = blockIdx.x; k < cl.nsols; k += gridDim.x) {
    for (int i = lane; i < n; i += 32) x[i] = C64(cl.in[k * n + i].x, cl.in[k * n + i].y);
    __syncwarp();
    bool ok = true;
    // Newton refinement of the centre, then Y at the refined point
    for (int it = 0; it < 2 && ok; ++it) {
      mono_balls(P, x, 0.0, mc, mr);
      rows_balls(P, P.val, false, mc, mr, vsc, vsr, n, Fc, Fr);
      rows_balls(P, P.jac, true, mc, mr, jsc, jsr, n2, Jc, Jr);
      ok = invert(Jc, Y, n);
      if (!ok || it == 1) break;
      for (int i = lane; i < n; i += 32) {
        c64 d = C64(0.0);
        for (int j = 0; j < n; ++j) d = d + Y[j * n + i] * Fc[j];
        x[i] = x[i] - d;
      }
      __syncwarp();
    }
    hc_certificate C;
    C.certified = 0;
    C.realness = 0;
    C.radius = 0.0;
    C.enclosure = 0.0;
    if (ok) {
      // YF = Y F(x̃) in balls: centre (vector per lane i), radius
      cb yf = cb_point(C64(0.0));
      double xnorm = 0.0, delta = 0.0;
      for (int i = 0; i < n; ++i) xnorm = fmax(xnorm, absu(x[i]));
      if (lane < n) {
        for (int j = 0; j < n; ++j) yf = cb_add(yf, cb_mul(cb_point(Y[j * n + lane]), cb{Fc[j], Fr[j]}));
        delta = __dadd_ru(absu(yf.c), yf.r);
      }
      for (int o = 16; o; o >>= 1) delta = fmax(delta, __shfl_xor_sync(FULL, delta, o));
      double r = __dadd_ru(__dmul_ru(8.0, delta), __dmul_ru(0x1p-45, fmax(xnorm, 1.0)));
      for (int attempt = 0; attempt < 4; ++attempt, r = __dmul_ru(r, 4.0)) {
        mono_balls(P, x, r, mc, mr);
        rows_balls(P, P.jac, true, mc, mr, jsc, jsr, n2, Jc, Jr);
        // M = I − Y J(B)
        for (int e = lane; e < n2; e += 32) {
          int i = e % n, j = e / n;
          cb acc = cb_point(C64(i == j ? 1.0 : 0.0));
          for (int q = 0; q < n; ++q) acc = cb_sub(acc, cb_mul(cb_point(Y[q * n + i]), cb{Jc[j * n + q], Jr[j * n + q]}));
          Mc[e] = acc.c;
          Mr[e] = acc.r;
        }
        __syncwarp();
        int inside = 1, real_in = cl.real_coefficients ? 1 : 0, nonreal = 0;
        double encl = 0.0;
        if (lane < n) {
          double v = 0.0;
          for (int j = 0; j < n; ++j) v = __dadd_ru(v, __dadd_ru(absu(Mc[j * n + lane]), Mr[j * n + lane]));
          // K_i = x̃_i − YF_i + M_i·B(0, r)
          c64 kcen = x[lane] - yf.c;
          double krad = __dadd_ru(__dadd_ru(yf.r, __dmul_ru(v, r)), __dmul_ru(0x1p-52, absu(kcen)));
          double dist = __dadd_ru(absu(kcen - x[lane]), __dmul_ru(0x1p-52, __dadd_ru(absu(kcen), absu(x[lane]))));
          inside = __dadd_ru(dist, krad) < r ? 1 : 0;
          c64 ck = conj(kcen);
          double cdist = __dadd_ru(absu(ck - x[lane]), __dmul_ru(0x1p-52, __dadd_ru(absu(ck), absu(x[lane]))));
          if (!(__dadd_ru(cdist, krad) < r)) real_in = 0;
          nonreal = fabs(kcen.im) > __dadd_ru(krad, __dmul_ru(0x1p-52, absu(kcen))) ? 1 : 0;
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
          C.radius = r;
          C.enclosure = encl;
          break;
        }
      }
    }
    for (int i = lane; i < n; i += 32) {
      cl.centers[k * n + i] = make_double2(x[i].re, x[i].im);
      cl.enclosures[k * n + i] = C.certified ? make_double2(kc[i].re, kc[i].im) : make_double2(x[i].re, x[i].im);
    }
    if (lane == 0) cl.out[k] = C;
    __syncwarp();
  }
}

}  // namespace

// host side: layout and launch (called from hc_capi.cu with the handle's program)
int certify_layout(const DevProg& P, int* bytes_out) {
  CertLayout L{};
  size_t off = 0;
  auto take = [&](size_t b) {
    size_t o = off;
    off += (b + 15) & ~(size_t)15;
    return (int)o;
  };
  const int n = P.n, n2 = n * n;
  L.mono = take((size_t)P.M * 24);
  L.vslot = take((size_t)P.val.nslots * 24);
  L.jslot = take((size_t)P.jac.nslots * 24);
  L.F = take((size_t)2 * n * 24);
  L.J = take((size_t)2 * n2 * 24);
  L.Y = take((size_t)n2 * 16);
  L.M = take((size_t)n2 * 24);
  L.x = take((size_t)2 * n * 16);
  L.bytes = (int)off;
  *bytes_out = L.bytes;
  return L.bytes <= 227 * 1024 ? 0 : 1;
}

cudaError_t launch_certify(const DevProg& P, int64_t nsols, const double* d_in, hc_certificate* d_out,
                           double* d_centers, double* d_enclosures, int real_coefficients, int num_sms,
                           cudaStream_t stream) {
  CertLaunch cl{};
  cl.P = P;
  CertLayout& L = cl.L;
  size_t off = 0;
  auto take = [&](size_t b) {
    size_t o = off;
    off += (b + 15) & ~(size_t)15;
    return (int)o;
  };
  const int n = P.n, n2 = n * n;
  L.mono = take((size_t)P.M * 24);
  L.vslot = take((size_t)P.val.nslots * 24);
  L.jslot = take((size_t)P.jac.nslots * 24);
  L.F = take((size_t)2 * n * 24);
  L.J = take((size_t)2 * n2 * 24);
  L.Y = take((size_t)n2 * 16);
  L.M = take((size_t)n2 * 24);
  L.x = take((size_t)2 * n * 16);
  L.bytes = (int)off;
  L.n2 = n2;
  cl.nsols = nsols;
  cl.in = (const double2*)d_in;
  cl.out = d_out;
  cl.centers = (double2*)d_centers;
  cl.enclosures = (double2*)d_enclosures;
  cl.real_coefficients = real_coefficients;
  cudaError_t e = cudaFuncSetAttribute(certify_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, L.bytes);
  if (e != cudaSuccess) return e;
  int per_sm = 0;
  e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, certify_kernel, 32, L.bytes);
  if (e != cudaSuccess) return e;
  int blocks = (int)std::min<int64_t>(nsols, (int64_t)std::max(1, per_sm) * num_sms);
  certify_kernel<<<blocks, 32, L.bytes, stream>>>(cl);
  return cudaGetLastError();
}

}  // namespace hcd
