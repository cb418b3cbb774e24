// hc_oracle.cpp — CPU restatement of HomotopyContinuation.jl's total-degree path-tracking
// hot path (Tracker + EndgameTracker over a StraightLineHomotopy of polynomial systems).
//
// TEST INFRASTRUCTURE ONLY. This file is the parity oracle: tests/, __graft_entry__.smoke()
// and bench.py's cpu_baseline / --impl reference legs load it as the checker. The product
// (libhcgpu.so) never links, loads or calls it.
//
// Every routine names the reference file:line it restates (paths relative to the
// HomotopyContinuation.jl v2.20 source tree). Arithmetic is plain IEEE FP64 with Julia's
// formulas (complex mul = (ac-bd, ad+bc), @fastmath division = naive, regular complex
// division = Smith); this file must be compiled with -ffp-contract=off so that neither the
// complex products nor the double-double error-free transforms get fused.
//
// Polynomials are evaluated term by term from (equation, coefficient, exponent) lists. The
// reference evaluates a CSE'd straight-line program instead (src/model_kit/*); the two agree
// to rounding, which is all the parity protocol (relative 1e-10 on endpoints, identical
// return-code counts) relies on.

#include <algorithm>
#include <atomic>
#include <cmath>
#include <complex>
#include <cstdint>
#include <cstring>
#include <limits>
#include <thread>
#include <vector>

namespace hco {

static const double INF = std::numeric_limits<double>::infinity();
static const double NaN = std::numeric_limits<double>::quiet_NaN();
static const double EPS = 2.220446049250313e-16;  // eps(Float64)

// ---------------------------------------------------------------------------------------
// Complex FP64 with Julia's formulas
// ---------------------------------------------------------------------------------------
struct C {
  double re, im;
};
static inline C cx(double r, double i = 0.0) { return C{r, i}; }
static inline C operator+(C a, C b) { return {a.re + b.re, a.im + b.im}; }
static inline C operator-(C a, C b) { return {a.re - b.re, a.im - b.im}; }
static inline C operator-(C a) { return {-a.re, -a.im}; }
static inline C operator*(C a, C b) {
  return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
static inline C operator*(double s, C a) { return {s * a.re, s * a.im}; }
static inline C operator*(C a, double s) { return {a.re * s, a.im * s}; }
static inline C operator/(C a, double s) { return {a.re / s, a.im / s}; }
static inline double abs2(C a) { return a.re * a.re + a.im * a.im; }
// src/utils.jl:207
static inline double fast_abs(C a) { return std::sqrt(abs2(a)); }
static inline double cabs(C a) { return std::hypot(a.re, a.im); }
static inline bool isnanC(C a) { return std::isnan(a.re) || std::isnan(a.im); }
static inline C conj(C a) { return {a.re, -a.im}; }
// @fastmath complex division (lu!, ldiv_upper!): naive formula
static inline C div_fast(C a, C b) {
  double d = b.re * b.re + b.im * b.im;
  return {(a.re * b.re + a.im * b.im) / d, (a.im * b.re - a.re * b.im) / d};
}
// regular complex division (Smith's algorithm)
static inline C cdiv(C a, C b) {
  if (std::fabs(b.re) >= std::fabs(b.im)) {
    if (b.re == 0.0 && b.im == 0.0) return {a.re / 0.0, a.im / 0.0};
    double r = b.im / b.re, den = b.re + b.im * r;
    return {(a.re + a.im * r) / den, (a.im - a.re * r) / den};
  } else {
    double r = b.re / b.im, den = b.re * r + b.im;
    return {(a.re * r + a.im) / den, (a.im * r - a.re) / den};
  }
}
static inline C cis(double th) { return {std::cos(th), std::sin(th)}; }
static inline C cpow_int(C a, int k) {
  C r = cx(1.0);
  for (int i = 0; i < k; ++i) r = r * a;
  return r;
}

// Julia's max/min on Float64 propagate NaN; @fastmath max_fast(x, y) = ifelse(x > y, x, y)
static inline double jmax(double a, double b) {
  if (std::isnan(a) || std::isnan(b)) return NaN;
  return a > b ? a : b;
}
static inline double jmin(double a, double b) {
  if (std::isnan(a) || std::isnan(b)) return NaN;
  return a < b ? a : b;
}
static inline double max_fast(double a, double b) { return a > b ? a : b; }
// clamp(x, lo, hi) = x > hi ? hi : (x < lo ? lo : x)
static inline double jclamp(double x, double lo, double hi) { return x > hi ? hi : (x < lo ? lo : x); }

// src/utils.jl:211-212
static inline double nanmin(double a, double b) {
  return std::isnan(a) ? b : (std::isnan(b) ? a : std::min(a, b));
}
static inline double nanmax(double a, double b) {
  return std::isnan(a) ? b : (std::isnan(b) ? a : std::max(a, b));
}
// src/utils.jl:408-422
static inline double nthroot(double x, int N) {
  if (N == 4) return std::sqrt(std::sqrt(x));
  if (N == 2) return std::sqrt(x);
  if (N == 3) return std::cbrt(x);
  if (N == 1) return x;
  if (N == 0) return 1.0;
  return std::pow(x, 1.0 / N);
}

// ---------------------------------------------------------------------------------------
// Double-double (src/DoubleDouble.jl:14-66, 166-266): sloppy add, two_prod with fma
// ---------------------------------------------------------------------------------------
struct DD {
  double hi, lo;
};
static inline void quick_two_sum(double a, double b, double& s, double& e) {
  s = a + b;
  e = b - (s - a);
}
static inline void two_sum(double a, double b, double& s, double& e) {
  s = a + b;
  double v = s - a;
  e = (a - (s - v)) + (b - v);
}
static inline void two_diff(double a, double b, double& s, double& e) {
  s = a - b;
  double v = s - a;
  e = (a - (s - v)) - (b + v);
}
static inline void two_prod(double a, double b, double& p, double& e) {
  p = a * b;
  e = std::fma(a, b, -p);
}
static inline DD dd(double x) { return DD{x, std::isinf(x) ? INF : 0.0}; }
static inline DD operator+(DD a, DD b) {  // DoubleDouble.jl:185-191
  double hi, lo;
  two_sum(a.hi, b.hi, hi, lo);
  lo += (a.lo + b.lo);
  quick_two_sum(hi, lo, hi, lo);
  return {hi, lo};
}
static inline DD operator-(DD a, DD b) {  // DoubleDouble.jl:226-233
  double hi, lo;
  two_diff(a.hi, b.hi, hi, lo);
  lo += a.lo;
  lo -= b.lo;
  quick_two_sum(hi, lo, hi, lo);
  return {hi, lo};
}
static inline DD operator*(DD a, DD b) {  // DoubleDouble.jl:260-266
  double p1, p2;
  two_prod(a.hi, b.hi, p1, p2);
  p2 += a.hi * b.lo + a.lo * b.hi;
  quick_two_sum(p1, p2, p1, p2);
  return {p1, p2};
}
struct CDD {
  DD re, im;
};
static inline CDD cdd(C a) { return CDD{dd(a.re), dd(a.im)}; }
static inline CDD operator+(CDD a, CDD b) { return {a.re + b.re, a.im + b.im}; }
static inline CDD operator-(CDD a, CDD b) { return {a.re - b.re, a.im - b.im}; }
static inline CDD operator*(CDD a, CDD b) {
  return {a.re * b.re - a.im * b.im, a.re * b.im + a.im * b.re};
}
static inline C round_c(CDD a) { return C{a.re.hi, a.im.hi}; }

// ---------------------------------------------------------------------------------------
// Polynomial systems and the straight-line homotopy
// ---------------------------------------------------------------------------------------
struct Term {
  int eq;
  C coef;
  std::vector<std::pair<int, int>> vars;  // (variable, exponent>0)
};
struct Slp;
struct System {
  int n = 0, m = 0, maxdeg = 0;
  std::vector<Term> terms;
  const Slp* slp = nullptr;  // F given as a straight-line program instead of terms
};

static System make_system(int n, int m, int nterms, const int32_t* eq, const int32_t* exps,
                          const double* coefs) {
  System S;
  S.n = n;
  S.m = m;
  S.terms.resize(nterms);
  for (int k = 0; k < nterms; ++k) {
    Term& T = S.terms[k];
    T.eq = eq[k];
    T.coef = C{coefs[2 * k], coefs[2 * k + 1]};
    for (int j = 0; j < n; ++j) {
      int e = exps[(size_t)k * n + j];
      if (e > 0) {
        T.vars.push_back({j, e});
        S.maxdeg = std::max(S.maxdeg, e);
      }
    }
  }
  return S;
}

// ---------------------------------------------------------------------------------------
// Straight-line programs: ModelKit's InstructionSequence interpreted (op semantics of
// src/model_kit/operations.jl:183-248; Taylor rules of src/model_kit/taylor.jl). Tape slots:
// constants [0, nconst), variables [voff, voff + n), instruction outputs above.
// ---------------------------------------------------------------------------------------
enum SlpOp {
  SOP_STOP = 0, SOP_CB, SOP_ACOS, SOP_ASIN, SOP_COS, SOP_COSH, SOP_EXP, SOP_INV, SOP_INV_NOT_ZERO, SOP_INVSQR,
  SOP_NEG, SOP_SIN, SOP_SINH, SOP_SQR, SOP_SQRT, SOP_TAN, SOP_TANH, SOP_IDENTITY, SOP_ADD, SOP_DIV, SOP_MUL,
  SOP_SUB, SOP_POW_INT, SOP_POW, SOP_ADD3, SOP_MUL3, SOP_MULADD, SOP_MULSUB, SOP_SUBMUL, SOP_ADD4, SOP_MUL4,
  SOP_MULMULADD, SOP_MULMULSUB
};
struct Slp {
  int n = 0, voff = 0, tape = 0, nconst = 0;
  int np = 0, poff = 0;  // parameters at tape slots [poff, poff + np)
  std::vector<int> ins;  // 6 per instruction: input[0..3], op, output
  std::vector<C> consts;
  std::vector<int> outputs;
};

static inline DD dd_div(DD a, DD b) {  // long division: three quotient digits
  double q1 = a.hi / b.hi;
  DD r = a - b * dd(q1);
  double q2 = r.hi / b.hi;
  r = r - b * dd(q2);
  double q3 = r.hi / b.hi;
  double s1, e1;
  quick_two_sum(q1, q2, s1, e1);
  return DD{s1, e1} + dd(q3);
}
static inline C s_neg(C a) { return -a; }
static inline CDD s_neg(CDD a) { return CDD{DD{-a.re.hi, -a.re.lo}, DD{-a.im.hi, -a.im.lo}}; }
static inline C s_div(C a, C b) { return div_fast(a, b); }  // op_div = div_fast
static inline CDD s_div(CDD a, CDD b) {
  DD d = b.re * b.re + b.im * b.im;
  return CDD{dd_div(a.re * b.re + a.im * b.im, d), dd_div(a.im * b.re - a.re * b.im, d)};
}
static inline C s_sqrt(C a) {
  std::complex<double> r = std::sqrt(std::complex<double>(a.re, a.im));
  return C{r.real(), r.imag()};
}
static inline CDD s_sqrt(CDD a) {  // FP64 root, then one Newton step in double-double
  C s = s_sqrt(round_c(a));
  if (s.re == 0.0 && s.im == 0.0) return cdd(s);
  CDD sd = cdd(s);
  C r = round_c(a - sd * sd);
  return sd + cdd(div_fast(r, C{2.0 * s.re, 2.0 * s.im}));
}
static inline bool s_zero(C a) { return a.re == 0.0 && a.im == 0.0; }
static inline bool s_zero(CDD a) { return a.re.hi == 0.0 && a.im.hi == 0.0; }
template <class S>
static S s_inv(S a) {
  return s_div(one_like(a), a);
}
template <class S>
static S s_pow(S a, int p) {  // power_by_squaring, inverted for p < 0 (op_pow_int)
  unsigned q = p < 0 ? (unsigned)(-p) : (unsigned)p;
  S r = one_like(a), b = a;
  bool first = true;
  while (q) {
    if (q & 1u) {
      r = first ? b : r * b;
      first = false;
    }
    q >>= 1;
    if (q) b = b * b;
  }
  return p < 0 ? s_inv(r) : r;
}
static inline C s_scale(C a, int k) { return a * (double)k; }
template <class S>
static S slp_value(int op, const S* v, int p) {
  switch (op) {
    case SOP_CB: return v[0] * v[0] * v[0];
    case SOP_INV: return s_inv(v[0]);
    case SOP_INV_NOT_ZERO: return s_zero(v[0]) ? v[0] : s_inv(v[0]);
    case SOP_INVSQR: { S i = s_inv(v[0]); return i * i; }
    case SOP_NEG: return s_neg(v[0]);
    case SOP_SQR: return v[0] * v[0];
    case SOP_SQRT: return s_sqrt(v[0]);
    case SOP_IDENTITY: return v[0];
    case SOP_ADD: return v[0] + v[1];
    case SOP_DIV: return s_div(v[0], v[1]);
    case SOP_MUL: return v[0] * v[1];
    case SOP_SUB: return v[0] - v[1];
    case SOP_POW_INT: return s_pow(v[0], p);
    case SOP_ADD3: return v[0] + v[1] + v[2];
    case SOP_MUL3: return v[0] * v[1] * v[2];
    case SOP_MULADD: return v[0] * v[1] + v[2];
    case SOP_MULSUB: return v[0] * v[1] - v[2];
    case SOP_SUBMUL: return v[2] - v[0] * v[1];
    case SOP_ADD4: return v[0] + v[1] + v[2] + v[3];
    case SOP_MUL4: return v[0] * v[1] * v[2] * v[3];
    case SOP_MULMULADD: return v[0] * v[1] + v[2] * v[3];
    case SOP_MULMULSUB: return v[0] * v[1] - v[2] * v[3];
  }
  return zero_like(v[0]);
}
static int slp_arity(int op) {
  if (op >= SOP_CB && op <= SOP_IDENTITY) return 1;
  if (op >= SOP_ADD && op <= SOP_POW) return 2;
  if (op >= SOP_ADD3 && op <= SOP_SUBMUL) return 3;
  if (op >= SOP_ADD4) return 4;
  return 0;
}
// all tape values at x (arithmetic S); pv: the parameters' values (np of them, may be null
// without parameters)
template <class S>
static void slp_tape(const Slp& P, const S* x, std::vector<S>& t, const C* pv = nullptr) {
  t.assign(P.tape, zero_like(x[0]));
  for (int k = 0; k < P.nconst; ++k) t[k] = promote(P.consts[k], x[0]);
  for (int j = 0; j < P.n; ++j) t[P.voff + j] = x[j];
  for (int k = 0; k < P.np; ++k) t[P.poff + k] = promote(pv[k], x[0]);
  for (size_t q = 0; q + 5 < P.ins.size(); q += 6) {
    int op = P.ins[q + 4];
    if (op == SOP_STOP) break;
    S v[4];
    int a = slp_arity(op);
    for (int r = 0; r < a; ++r)
      if (!(op == SOP_POW_INT && r == 1)) v[r] = t[P.ins[q + r]];
    t[P.ins[q + 5]] = slp_value(op, v, P.ins[q + 1]);
  }
}
// derivative of an op's output from its inputs' values v, output value c and input tangents d
static C slp_tangent(int op, const C* v, C c, const C* d, int p) {
  switch (op) {
    case SOP_CB: return s_scale(v[0] * v[0], 3) * d[0];
    case SOP_INV: return s_neg(c * c * d[0]);
    case SOP_INV_NOT_ZERO: return s_zero(v[0]) ? d[0] : s_neg(c * c * d[0]);
    case SOP_INVSQR: return s_neg(s_scale(c * s_inv(v[0]), 2) * d[0]);
    case SOP_NEG: return s_neg(d[0]);
    case SOP_SQR: return s_scale(v[0] * d[0], 2);
    case SOP_SQRT: return s_div(d[0], s_scale(c, 2));
    case SOP_IDENTITY: return d[0];
    case SOP_ADD: return d[0] + d[1];
    case SOP_DIV: return s_div(d[0] - c * d[1], v[1]);
    case SOP_MUL: return d[0] * v[1] + v[0] * d[1];
    case SOP_SUB: return d[0] - d[1];
    case SOP_POW_INT: return p == 0 ? cx(0.0) : s_scale(s_pow(v[0], p - 1), p) * d[0];
    case SOP_ADD3: return d[0] + d[1] + d[2];
    case SOP_MUL3: return d[0] * v[1] * v[2] + v[0] * d[1] * v[2] + v[0] * v[1] * d[2];
    case SOP_MULADD: return d[0] * v[1] + v[0] * d[1] + d[2];
    case SOP_MULSUB: return d[0] * v[1] + v[0] * d[1] - d[2];
    case SOP_SUBMUL: return d[2] - (d[0] * v[1] + v[0] * d[1]);
    case SOP_ADD4: return d[0] + d[1] + d[2] + d[3];
    case SOP_MUL4:
      return d[0] * v[1] * v[2] * v[3] + v[0] * d[1] * v[2] * v[3] + v[0] * v[1] * d[2] * v[3] +
             v[0] * v[1] * v[2] * d[3];
    case SOP_MULMULADD: return d[0] * v[1] + v[0] * d[1] + d[2] * v[3] + v[2] * d[3];
    case SOP_MULMULSUB: return d[0] * v[1] + v[0] * d[1] - (d[2] * v[3] + v[2] * d[3]);
  }
  return cx(0.0);
}
// F(x) and its Jacobian (column-major m×n), one forward-mode sweep per variable
static void slp_eval_jac(const Slp& P, const C* x, C* u, C* U, const C* pv = nullptr) {
  std::vector<C> t, dt;
  slp_tape(P, x, t, pv);
  for (int i = 0; i < P.n; ++i) u[i] = t[P.outputs[i]];
  for (int j = 0; j < P.n; ++j) {
    dt.assign(P.tape, cx(0.0));
    dt[P.voff + j] = cx(1.0);
    for (size_t q = 0; q + 5 < P.ins.size(); q += 6) {
      int op = P.ins[q + 4];
      if (op == SOP_STOP) break;
      C v[4], d[4];
      int a = slp_arity(op);
      for (int r = 0; r < a; ++r)
        if (!(op == SOP_POW_INT && r == 1)) {
          v[r] = t[P.ins[q + r]];
          d[r] = dt[P.ins[q + r]];
        }
      dt[P.ins[q + 5]] = slp_tangent(op, v, t[P.ins[q + 5]], d, P.ins[q + 1]);
    }
    for (int i = 0; i < P.n; ++i) U[(size_t)j * P.n + i] = dt[P.outputs[i]];
  }
}
// truncated series (orders 0..K) of the ops
static void ser_mul(const C* a, const C* b, C* c, int K) {
  for (int k = 0; k <= K; ++k) {
    C s = cx(0.0);
    for (int j = 0; j <= k; ++j) s = s + a[j] * b[k - j];
    c[k] = s;
  }
}
static void ser_inv(const C* a, C* c, int K) {  // c_0 = 1/a_0, c_k = -(Σ_{j≥1} a_j c_{k-j}) c_0
  c[0] = s_inv(a[0]);
  for (int k = 1; k <= K; ++k) {
    C s = cx(0.0);
    for (int j = 1; j <= k; ++j) s = s + a[j] * c[k - j];
    c[k] = s_neg(s) * c[0];
  }
}
static void ser_pow(const C* a, int p, C* c, int K) {
  int q = p < 0 ? -p : p;
  std::vector<C> r(K + 1, cx(0.0)), b(a, a + K + 1), tmp(K + 1);
  r[0] = cx(1.0);
  while (q) {
    if (q & 1) {
      ser_mul(r.data(), b.data(), tmp.data(), K);
      r = tmp;
    }
    q >>= 1;
    if (q) {
      ser_mul(b.data(), b.data(), tmp.data(), K);
      b = tmp;
    }
  }
  if (p < 0)
    ser_inv(r.data(), c, K);
  else
    for (int k = 0; k <= K; ++k) c[k] = r[k];
}
// pv, dv_p: the parameters' values and their first-order coefficients (parameter homotopy:
// p(t + s) = p(t) + s (p - q)); null without parameters
static void slp_taylor(const Slp& P, int K, const C* tx, int nx, C* dv, const C* pv = nullptr,
                       const C* dpv = nullptr) {
  const int L = K + 1, n = P.n;
  std::vector<C> t((size_t)P.tape * L, cx(0.0));
  auto at = [&](int slot) { return &t[(size_t)slot * L]; };
  for (int k = 0; k < P.nconst; ++k) at(k)[0] = P.consts[k];
  for (int j = 0; j < n; ++j)
    for (int k = 0; k < L; ++k) at(P.voff + j)[k] = k < nx ? tx[(size_t)k * n + j] : cx(0.0);
  for (int k = 0; k < P.np; ++k) {
    at(P.poff + k)[0] = pv[k];
    if (L > 1) at(P.poff + k)[1] = dpv[k];
  }
  std::vector<C> a(L), b(L), c(L), e(L);
  for (size_t q = 0; q + 5 < P.ins.size(); q += 6) {
    int op = P.ins[q + 4];
    if (op == SOP_STOP) break;
    const C* v[4] = {nullptr, nullptr, nullptr, nullptr};
    int ar = slp_arity(op);
    for (int r = 0; r < ar; ++r)
      if (!(op == SOP_POW_INT && r == 1)) v[r] = at(P.ins[q + r]);
    C* o = at(P.ins[q + 5]);
    auto add = [&](const C* x, const C* y, C* z, double sy) {
      for (int k = 0; k < L; ++k) z[k] = x[k] + y[k] * sy;
    };
    switch (op) {
      case SOP_IDENTITY: for (int k = 0; k < L; ++k) o[k] = v[0][k]; break;
      case SOP_NEG: for (int k = 0; k < L; ++k) o[k] = s_neg(v[0][k]); break;
      case SOP_ADD: add(v[0], v[1], o, 1.0); break;
      case SOP_SUB: add(v[0], v[1], o, -1.0); break;
      case SOP_MUL: ser_mul(v[0], v[1], o, K); break;
      case SOP_SQR: ser_mul(v[0], v[0], o, K); break;
      case SOP_CB: ser_mul(v[0], v[0], a.data(), K); ser_mul(a.data(), v[0], o, K); break;
      case SOP_INV: ser_inv(v[0], o, K); break;
      case SOP_INV_NOT_ZERO:
        if (s_zero(v[0][0])) for (int k = 0; k < L; ++k) o[k] = v[0][k];
        else ser_inv(v[0], o, K);
        break;
      case SOP_INVSQR: ser_inv(v[0], a.data(), K); ser_mul(a.data(), a.data(), o, K); break;
      case SOP_POW_INT: ser_pow(v[0], P.ins[q + 1], o, K); break;
      case SOP_DIV:  // c_0 = a_0/b_0, c_k = (a_k - Σ_{j≥1} b_j c_{k-j}) / b_0
        o[0] = s_div(v[0][0], v[1][0]);
        for (int k = 1; k <= K; ++k) {
          C s = v[0][k];
          for (int j = 1; j <= k; ++j) s = s - v[1][j] * o[k - j];
          o[k] = s_div(s, v[1][0]);
        }
        break;
      case SOP_SQRT:  // c_0 = √a_0, c_k = (a_k - Σ_{j=1..k-1} c_j c_{k-j}) / (2 c_0)
        o[0] = s_sqrt(v[0][0]);
        for (int k = 1; k <= K; ++k) {
          C s = v[0][k];
          for (int j = 1; j <= k - 1; ++j) s = s - o[j] * o[k - j];
          o[k] = s_div(s, s_scale(o[0], 2));
        }
        break;
      case SOP_ADD3: add(v[0], v[1], a.data(), 1.0); add(a.data(), v[2], o, 1.0); break;
      case SOP_MUL3: ser_mul(v[0], v[1], a.data(), K); ser_mul(a.data(), v[2], o, K); break;
      case SOP_MULADD: ser_mul(v[0], v[1], a.data(), K); add(a.data(), v[2], o, 1.0); break;
      case SOP_MULSUB: ser_mul(v[0], v[1], a.data(), K); add(a.data(), v[2], o, -1.0); break;
      case SOP_SUBMUL: ser_mul(v[0], v[1], a.data(), K); add(v[2], a.data(), o, -1.0); break;
      case SOP_ADD4:
        add(v[0], v[1], a.data(), 1.0); add(a.data(), v[2], b.data(), 1.0); add(b.data(), v[3], o, 1.0);
        break;
      case SOP_MUL4:
        ser_mul(v[0], v[1], a.data(), K); ser_mul(a.data(), v[2], b.data(), K); ser_mul(b.data(), v[3], o, K);
        break;
      case SOP_MULMULADD: ser_mul(v[0], v[1], a.data(), K); ser_mul(v[2], v[3], b.data(), K); add(a.data(), b.data(), o, 1.0); break;
      case SOP_MULMULSUB: ser_mul(v[0], v[1], a.data(), K); ser_mul(v[2], v[3], b.data(), K); add(a.data(), b.data(), o, -1.0); break;
    }
  }
  for (int k = 0; k < L; ++k)
    for (int i = 0; i < n; ++i) dv[(size_t)k * n + i] = at(P.outputs[i])[k];
}

// power table pw[j*(D+1)+k] = x_j^k
template <class S>
static S smul(S a, S b) {
  return a * b;
}
static inline C one_like(C) { return cx(1.0); }
static inline CDD one_like(CDD) { return cdd(cx(1.0)); }
static inline C zero_like(C) { return cx(0.0); }
static inline CDD zero_like(CDD) { return cdd(cx(0.0)); }
static inline C promote(C c, C) { return c; }
static inline CDD promote(C c, CDD) { return cdd(c); }

template <class S>
static void power_table(const System& F, const S* x, std::vector<S>& pw) {
  int D = F.maxdeg;
  pw.resize((size_t)F.n * (D + 1));
  for (int j = 0; j < F.n; ++j) {
    S p = one_like(x[j]);
    pw[(size_t)j * (D + 1)] = p;
    for (int k = 1; k <= D; ++k) {
      p = p * x[j];
      pw[(size_t)j * (D + 1) + k] = p;
    }
  }
}

// F(x) in arithmetic S (C or CDD)
template <class S>
static void sys_eval(const System& F, const S* x, S* u) {
  if (F.slp) {
    std::vector<S> t;
    slp_tape(*F.slp, x, t);
    for (int i = 0; i < F.m; ++i) u[i] = t[F.slp->outputs[i]];
    return;
  }
  std::vector<S> pw;
  power_table(F, x, pw);
  int D = F.maxdeg;
  S z = zero_like(x[0]);
  for (int i = 0; i < F.m; ++i) u[i] = z;
  for (const Term& T : F.terms) {
    S v = promote(T.coef, z);
    for (auto& ve : T.vars) v = v * pw[(size_t)ve.first * (D + 1) + ve.second];
    u[T.eq] = u[T.eq] + v;
  }
}

// F(x) and its Jacobian U (column-major m×n)
static void sys_eval_jac(const System& F, const C* x, C* u, C* U) {
  if (F.slp) return slp_eval_jac(*F.slp, x, u, U);
  std::vector<C> pw;
  power_table(F, x, pw);
  int D = F.maxdeg;
  for (int i = 0; i < F.m; ++i) u[i] = cx(0.0);
  for (int i = 0; i < F.m * F.n; ++i) U[i] = cx(0.0);
  for (const Term& T : F.terms) {
    C v = T.coef;
    for (auto& ve : T.vars) v = v * pw[(size_t)ve.first * (D + 1) + ve.second];
    u[T.eq] = u[T.eq] + v;
    for (size_t a = 0; a < T.vars.size(); ++a) {
      int j = T.vars[a].first, e = T.vars[a].second;
      C d = T.coef * (double)e;
      for (size_t b = 0; b < T.vars.size(); ++b) {
        int l = T.vars[b].first, el = T.vars[b].second;
        int ee = (b == a) ? el - 1 : el;
        if (ee > 0) d = d * pw[(size_t)l * (D + 1) + ee];
      }
      U[(size_t)j * F.m + T.eq] = U[(size_t)j * F.m + T.eq] + d;
    }
  }
}

// Truncated Taylor series: coefficients 0..K of F(x(ε)), x(ε)=Σ_{k<nx} tx[k] ε^k.
// Restates the semantics of taylor!(u, Val(K), F, tx) with all orders assigned
// (src/model_kit/taylor.jl:607-737, instruction_interpreter.jl:446-491).
static void series_mul(const C* a, const C* b, C* c, int K) {
  for (int k = 0; k <= K; ++k) {
    C s = cx(0.0);
    for (int j = 0; j <= k; ++j) s = s + a[j] * b[k - j];
    c[k] = s;
  }
}
static void sys_taylor(const System& F, int K, const C* tx, int nx, C* dv /* (K+1)×m */) {
  if (F.slp) return slp_taylor(*F.slp, K, tx, nx, dv);
  int n = F.n, D = F.maxdeg, L = K + 1;
  std::vector<C> ps((size_t)n * (D + 1) * L, cx(0.0));
  std::vector<C> tmp(L);
  for (int j = 0; j < n; ++j) {
    C* p0 = &ps[((size_t)j * (D + 1) + 0) * L];
    p0[0] = cx(1.0);
    C xs[8];
    for (int k = 0; k < L; ++k) xs[k] = (k < nx) ? tx[(size_t)k * n + j] : cx(0.0);
    for (int e = 1; e <= D; ++e) {
      C* pe = &ps[((size_t)j * (D + 1) + e) * L];
      series_mul(&ps[((size_t)j * (D + 1) + e - 1) * L], xs, pe, K);
    }
  }
  for (int i = 0; i < L * F.m; ++i) dv[i] = cx(0.0);
  std::vector<C> acc(L), nxt(L);
  for (const Term& T : F.terms) {
    for (int k = 0; k < L; ++k) acc[k] = cx(0.0);
    acc[0] = T.coef;
    for (auto& ve : T.vars) {
      series_mul(acc.data(), &ps[((size_t)ve.first * (D + 1) + ve.second) * L], nxt.data(), K);
      acc.swap(nxt);
    }
    for (int k = 0; k < L; ++k) dv[(size_t)k * F.m + T.eq] = dv[(size_t)k * F.m + T.eq] + acc[k];
  }
}

// src/homotopies/straight_line_homotopy.jl: H(x,t) = γ t G(x) + (1-t) F(x);
// toric (src/homotopies/toric_homotopy.jl): H(x,t) = F(x; u·t^w), u = F's coefficients, w per term
struct Homotopy {
  System G, F;
  C gamma;
  int n, m;
  bool toric = false;
  // parameter homotopy (src/homotopies/parameter_homotopy.jl:3-44): H(x, t) = F(x; t p + (1-t) q)
  // with F.slp a program with parameters
  bool param = false;
  std::vector<C> pp, pq;
  std::vector<double> w;     // weights of the current path (F's term order)
  mutable System Ft;         // F with the coefficients u·t^w at t = tc_t
  mutable std::vector<double> tpow;
  mutable double tc_t = NaN;
};

// tp! (parameter_homotopy.jl:64-87): the parameters at t and their t-derivative p - q
static void param_at(const Homotopy& H, C t, std::vector<C>& pv, std::vector<C>& dp) {
  const size_t m = H.pp.size();
  pv.resize(m);
  dp.resize(m);
  for (size_t k = 0; k < m; ++k) {
    if (t.im == 0.0) {
      const double s = t.re, r = 1.0 - t.re;
      pv[k] = C{s * H.pp[k].re + r * H.pq[k].re, s * H.pp[k].im + r * H.pq[k].im};
    } else {
      pv[k] = t * H.pp[k] + (cx(1.0) - t) * H.pq[k];
    }
    dp[k] = H.pp[k] - H.pq[k];
  }
}
template <class S>
static void param_eval(const Homotopy& H, const S* x, C t, S* u) {
  std::vector<C> pv, dp;
  param_at(H, t, pv, dp);
  std::vector<S> tape;
  slp_tape(*H.F.slp, x, tape, pv.data());
  for (int i = 0; i < H.m; ++i) u[i] = tape[H.F.slp->outputs[i]];
}

// coeffs! (toric_homotopy.jl:147-180) for real t ≥ 0
static const System& toric_sys(const Homotopy& H, double t) {
  if (!(t == H.tc_t)) {
    H.tpow.resize(H.F.terms.size());
    for (size_t k = 0; k < H.F.terms.size(); ++k) {
      double w = H.w[k];
      double p = (t == 0.0) ? (w == 0.0 ? 1.0 : 0.0) : std::exp(w * std::log(t));
      H.tpow[k] = p;
      H.Ft.terms[k].coef = H.F.terms[k].coef * p;
    }
    H.tc_t = t;
  }
  return H.Ft;
}

// :96-104
static void H_eval(const Homotopy& H, const C* x, C t, C* u) {
  if (H.param) return param_eval(H, x, t, u);  // evaluate!(u, H.F, x, H.pt) (:89-92)
  if (H.toric) {
    sys_eval(toric_sys(H, t.re), x, u);
    return;
  }
  std::vector<C> g(H.m), f(H.m);
  sys_eval(H.G, x, g.data());
  sys_eval(H.F, x, f.data());
  C ts = H.gamma * t, tt = cx(1.0) - t;
  for (int i = 0; i < H.m; ++i) u[i] = ts * g[i] + tt * f[i];
}
// :81-94 (DD residual rounded to F64 on store)
static void H_eval_dd(const Homotopy& H, const CDD* x, C t, C* u) {
  if (H.param) {
    std::vector<CDD> f(H.m);
    param_eval(H, x, t, f.data());
    for (int i = 0; i < H.m; ++i) u[i] = round_c(f[i]);
    return;
  }
  if (H.toric) {
    std::vector<CDD> f(H.m);
    sys_eval(toric_sys(H, t.re), x, f.data());
    for (int i = 0; i < H.m; ++i) u[i] = round_c(f[i]);
    return;
  }
  std::vector<CDD> g(H.m), f(H.m);
  sys_eval(H.G, x, g.data());
  sys_eval(H.F, x, f.data());
  CDD ts = cdd(H.gamma * t), tt = cdd(cx(1.0) - t);
  for (int i = 0; i < H.m; ++i) u[i] = round_c(ts * g[i] + tt * f[i]);
}
// :106-124
static void H_eval_jac(const Homotopy& H, const C* x, C t, C* u, C* U) {
  if (H.param) {  // evaluate_and_jacobian!(u, U, H.F, x, H.pt) (:94-97)
    std::vector<C> pv, dp;
    param_at(H, t, pv, dp);
    return slp_eval_jac(*H.F.slp, x, u, U, pv.data());
  }
  if (H.toric) {
    sys_eval_jac(toric_sys(H, t.re), x, u, U);
    return;
  }
  int m = H.m, n = H.n;
  std::vector<C> g(m), f(m), Gj((size_t)m * n), Fj((size_t)m * n);
  sys_eval_jac(H.G, x, g.data(), Gj.data());
  sys_eval_jac(H.F, x, f.data(), Fj.data());
  C ts = H.gamma * t, tt = cx(1.0) - t;
  for (int i = 0; i < m; ++i) u[i] = ts * g[i] + tt * f[i];
  for (size_t k = 0; k < (size_t)m * n; ++k) U[k] = ts * Gj[k] + tt * Fj[k];
}
// :130-137  taylor!(u, Val(1), H, x, t) = γ G(x) - F(x);
// toric (toric_homotopy.jl:133-146, 255-257): F(x; ċ), ċ = w·c/t (t = 0: u where w == 1)
static void H_taylor1(const Homotopy& H, const C* x, C t, C* u) {
  if (H.param) {  // taylor!(u, Val(1), H.F, x, tp!(H, t)): order 1 of F(x; p(t + s))
    std::vector<C> pv, dp, dv((size_t)2 * H.m);
    param_at(H, t, pv, dp);
    slp_taylor(*H.F.slp, 1, x, 1, dv.data(), pv.data(), dp.data());
    for (int i = 0; i < H.m; ++i) u[i] = dv[(size_t)H.m + i];
    return;
  }
  if (H.toric) {
    const System& Fc = toric_sys(H, t.re);
    System Fd = Fc;
    for (size_t k = 0; k < Fd.terms.size(); ++k) {
      double w = H.w[k];
      if (t.re == 0.0)
        Fd.terms[k].coef = (w == 1.0) ? H.F.terms[k].coef : cx(0.0);
      else
        Fd.terms[k].coef = (w * Fc.terms[k].coef) * (1.0 / t.re);
    }
    sys_eval(Fd, x, u);
    return;
  }
  std::vector<C> g(H.m), f(H.m);
  sys_eval(H.G, x, g.data());
  sys_eval(H.F, x, f.data());
  for (int i = 0; i < H.m; ++i) u[i] = H.gamma * g[i] - f[i];
}
// :138-154  taylor!(u, Val(K), H, tx, t), tx holds K vectors (orders 0..K-1)
static void H_taylorK(const Homotopy& H, int K, const C* tx, C t, C* u) {
  int m = H.m;
  if (H.param) {  // taylor!(u, Val(K), H.F, tx, tp!(H, t)) (:98-101): order K of F(x(s); p(t + s))
    std::vector<C> pv, dp, dv((size_t)(K + 1) * m);
    param_at(H, t, pv, dp);
    slp_taylor(*H.F.slp, K, tx, K, dv.data(), pv.data(), dp.data());
    for (int i = 0; i < m; ++i) u[i] = dv[(size_t)K * m + i];
    return;
  }
  if (H.toric) {
    // taylor_coeffs! (toric_homotopy.jl:199-253): c^(j) = u·tw_j, tw_0 = t^w,
    // tw_1 = w tw_0/t, tw_2 = (w-1)/2 tw_1/t, tw_3 = (w-2) tw_2/t/3; u_K = Σ_j [ε^(K-j)] F(x(ε); c^(j))
    const double tr = t.re;
    toric_sys(H, tr);
    for (int i = 0; i < m; ++i) u[i] = cx(0.0);
    std::vector<C> dv((size_t)(K + 1) * m);
    for (int j = 0; j <= K; ++j) {
      System Fj = H.F;
      for (size_t k = 0; k < Fj.terms.size(); ++k) {
        double w = H.w[k], tw[4];
        if (tr == 0.0) {
          tw[0] = w < 1e-12 ? 1.0 : 0.0;
          tw[1] = (tw[0] == 0.0 && std::fabs(w - 1.0) <= 0x1p-26 * std::max(std::fabs(w), 1.0)) ? 1.0 : 0.0;
          tw[2] = tw[3] = 0.0;
        } else {
          double ti = 1.0 / tr;
          tw[0] = H.tpow[k];
          tw[1] = w * tw[0] * ti;
          tw[2] = 0.5 * (w - 1) * tw[1] * ti;
          tw[3] = (w - 2) * tw[2] * ti / 3;
        }
        Fj.terms[k].coef = H.F.terms[k].coef * tw[j];
      }
      sys_taylor(Fj, K, tx, K, dv.data());
      for (int i = 0; i < m; ++i) u[i] = u[i] + dv[(size_t)(K - j) * m + i];
    }
    return;
  }
  std::vector<C> dg((size_t)(K + 1) * m), df((size_t)(K + 1) * m);
  sys_taylor(H.G, K, tx, K, dg.data());
  sys_taylor(H.F, K, tx, K, df.data());
  for (int i = 0; i < m; ++i) {
    C start = H.gamma * (dg[(size_t)(K - 1) * m + i] + t * dg[(size_t)K * m + i]);
    C target = (cx(1.0) - t) * df[(size_t)K * m + i] - df[(size_t)(K - 1) * m + i];
    u[i] = start + target;
  }
}

// ---------------------------------------------------------------------------------------
// Norms (src/norm.jl)
// ---------------------------------------------------------------------------------------
// :194-213
static double inf_norm_v(const C* x, int n) {
  double dmax = abs2(x[0]);
  for (int i = 1; i < n; ++i) dmax = max_fast(dmax, abs2(x[i]));
  double d = std::sqrt(dmax);
  if (std::isinf(d)) {
    dmax = cabs(x[0]);
    for (int i = 1; i < n; ++i) dmax = jmax(dmax, cabs(x[i]));
    return dmax;
  }
  return d;
}
// :150-169 (the overflow branch compares abs of the first entry with abs2 of the rest)
static double inf_dist(const C* x, const C* y, int n) {
  double dmax = abs2(x[0] - y[0]);
  for (int i = 1; i < n; ++i) dmax = max_fast(dmax, abs2(x[i] - y[i]));
  double d = std::sqrt(dmax);
  if (std::isinf(d)) {
    dmax = cabs(x[0] - y[0]);
    for (int i = 1; i < n; ++i) dmax = jmax(dmax, abs2(x[i] - y[i]));
    return dmax;
  }
  return d;
}
// :214-234 (w == nullptr gives InfNorm)
static double wnorm(const C* x, const double* w, int n) {
  if (!w) return inf_norm_v(x, n);
  double dmax = abs2(x[0] / w[0]);
  for (int i = 1; i < n; ++i) dmax = max_fast(dmax, abs2(x[i] / w[i]));
  double d = std::sqrt(dmax);
  if (std::isinf(d)) {
    dmax = cabs(x[0] / w[0]);
    for (int i = 1; i < n; ++i) dmax = jmax(dmax, cabs(x[i] / w[i]));
    return dmax;
  }
  return d;
}
// :170-192
static double wdist(const C* x, const C* y, const double* w, int n) {
  std::vector<C> d(n);
  for (int i = 0; i < n; ++i) d[i] = x[i] - y[i];
  return wnorm(d.data(), w, n);
}

struct WeightedNorm {  // :36-40, :65-69
  std::vector<double> w;
  double scale_min = 1e-4, scale_abs_min = 1e-6, scale_max = std::ldexp(1.0, 511);
  int n = 0;
  double operator()(const C* x) const { return wnorm(x, w.data(), n); }
  double dist(const C* x, const C* y) const { return wdist(x, y, w.data(), n); }
  void init(const C* x) {  // :101-113
    double point_norm = inf_norm_v(x, n);
    for (int i = 0; i < n; ++i) {
      double wi = fast_abs(x[i]);
      if (wi < scale_min * point_norm)
        wi = scale_min * point_norm;
      else if (wi > scale_max * point_norm)
        wi = scale_max * point_norm;
      w[i] = jmax(wi, scale_abs_min);
    }
  }
  void update(const C* x) {  // :122-136
    double norm_x = (*this)(x);
    for (int i = 0; i < n; ++i) {
      double wi = (fast_abs(x[i]) + w[i]) / 2;
      if (wi < scale_min * norm_x)
        wi = scale_min * norm_x;
      else if (wi > scale_max * norm_x)
        wi = scale_max * norm_x;
      if (std::isfinite(wi)) w[i] = jmax(wi, scale_abs_min);
    }
  }
};

// ---------------------------------------------------------------------------------------
// Linear algebra (src/linear_algebra.jl), square case
// ---------------------------------------------------------------------------------------
struct MW {
  int n = 0;
  std::vector<C> A, LU;  // column-major
  std::vector<int> ipiv;
  std::vector<double> row_scaling;
  bool factorized = false, scaled = false;
  // stats (Jacobian :809-815)
  long factorizations = 0, ldivs = 0;
  C& a(int i, int j) { return A[(size_t)j * n + i]; }
  C& lu(int i, int j) { return LU[(size_t)j * n + i]; }
  void resize(int nn) {
    n = nn;
    A.assign((size_t)n * n, cx(0.0));
    LU.assign((size_t)n * n, cx(0.0));
    ipiv.assign(n, 0);
    row_scaling.assign(n, 1.0);
  }
};

// :88-98
static void updated(MW& W) {
  W.factorized = false;
  W.scaled = false;
  W.LU = W.A;
}

// :130-184 right-looking partial-pivot LU, pivot by max abs2, naive complex division
static void lu_factor(std::vector<C>& Av, std::vector<int>& ipiv, int n) {
  auto A = [&](int i, int j) -> C& { return Av[(size_t)j * n + i]; };
  for (int k = 0; k < n; ++k) {
    int kp = k;
    double amax = abs2(A(k, k));
    for (int i = k + 1; i < n; ++i) {
      double absi = abs2(A(i, k));
      if (absi > amax) {
        kp = i;
        amax = absi;
      }
    }
    ipiv[k] = kp;
    if (amax != 0.0) {  // !iszero(amax); NaN != 0
      if (k != kp) {
        for (int i = 0; i < n; ++i) std::swap(A(k, i), A(kp, i));
      }
      C Akk = A(k, k);
      for (int i = k + 1; i < n; ++i) A(i, k) = div_fast(A(i, k), Akk);
    }
    for (int j = k + 1; j < n; ++j) {
      C Akj = A(k, j);
      for (int i = k + 1; i < n; ++i) A(i, j) = A(i, j) - A(i, k) * Akj;
    }
  }
}

// :254-263
static void factorize(MW& W) {
  lu_factor(W.LU, W.ipiv, W.n);
  W.factorized = true;
}

// :268-316
static void lu_ldiv(MW& W, C* x) {
  int n = W.n;
  for (int i = 0; i < n; ++i)
    if (i != W.ipiv[i]) std::swap(x[i], x[W.ipiv[i]]);
  for (int j = 0; j < n; ++j) {  // ldiv_unit_lower!
    C xj = x[j];
    for (int i = j + 1; i < n; ++i) x[i] = x[i] - W.lu(i, j) * xj;
  }
  for (int j = n - 1; j >= 0; --j) {  // ldiv_upper!
    C xj = div_fast(x[j], W.lu(j, j));
    x[j] = xj;
    for (int i = 0; i < j; ++i) x[i] = x[i] - W.lu(i, j) * xj;
  }
}
// :318-354
static void lu_ldiv_adj(MW& W, C* x) {
  int n = W.n;
  for (int j = 0; j < n; ++j) {  // ldiv_adj_upper!
    C z = x[j];
    for (int i = 0; i < j; ++i) z = z - conj(W.lu(i, j)) * x[i];
    x[j] = div_fast(z, conj(W.lu(j, j)));
  }
  for (int j = n - 1; j >= 0; --j) {  // ldiv_adj_unit_lower!
    C z = x[j];
    for (int i = n - 1; i >= j + 1; --i) z = z - conj(W.lu(i, j)) * x[i];
    x[j] = z;
  }
  for (int i = n - 1; i >= 0; --i)  // _inverse_ipiv!
    if (i != W.ipiv[i]) std::swap(x[i], x[W.ipiv[i]]);
}

// :389-408  LA.ldiv!(x, WS, b)
static void ws_ldiv(MW& W, C* x, const C* b) {
  int n = W.n;
  if (n == 1) {
    x[0] = cdiv(b[0], W.A[0]);
    return;
  }
  if (!W.factorized) factorize(W);
  if (W.scaled) {
    for (int i = 0; i < n; ++i) x[i] = W.row_scaling[i] * b[i];
  } else {
    for (int i = 0; i < n; ++i) x[i] = b[i];
  }
  lu_ldiv(W, x);
}

// :432-459
static void skeel_row_scaling(double* d, const C* A, int n, const double* c,
                              double scaling_threshold = -30.0) {
  for (int i = 0; i < n; ++i) d[i] = 0.0;
  for (int j = 0; j < n; ++j) {
    double cj = c[j];
    for (int i = 0; i < n; ++i) d[i] += fast_abs(A[(size_t)j * n + i]) * cj;
  }
  double m = d[0];
  for (int i = 1; i < n; ++i) m = jmax(m, d[i]);  // maximum(d)
  double s = scaling_threshold + m;
  for (int i = 0; i < n; ++i) {
    int e = 0;
    std::frexp(d[i], &e);
    if (!std::isfinite(d[i])) e = 0;  // Julia frexp(Inf/NaN) exponent is 0
    if (e < s)
      d[i] = 1.0;
    else
      d[i] = std::exp2(-e);
  }
}
// :489-497
static void apply_row_scaling(MW& W) {
  for (int j = 0; j < W.n; ++j)
    for (int i = 0; i < W.n; ++i) W.lu(i, j) = W.lu(i, j) * W.row_scaling[i];
  W.scaled = true;
}

// :833-862  ldiv!(x, J, b[, norm::WeightedNorm])
static void jac_ldiv(MW& W, C* x, const C* b, const double* weights) {
  if (weights && !W.factorized) {
    skeel_row_scaling(W.row_scaling.data(), W.A.data(), W.n, weights);
    apply_row_scaling(W);
  }
  W.factorizations += !W.factorized;
  W.ldivs += 1;
  ws_ldiv(W, x, b);
}

// :528-544 mixed-precision (DD residual) refinement step
static double mp_refine_step(MW& W, C* x, const C* b, const double* w) {
  int n = W.n;
  std::vector<CDD> xb(n), rb(n);
  std::vector<C> r(n), dx(n);
  for (int i = 0; i < n; ++i) xb[i] = cdd(x[i]);
  for (int i = 0; i < n; ++i) rb[i] = cdd(cx(0.0));
  for (int j = 0; j < n; ++j)
    for (int i = 0; i < n; ++i) rb[i] = rb[i] + cdd(W.a(i, j)) * xb[j];
  for (int i = 0; i < n; ++i) rb[i] = rb[i] - cdd(b[i]);
  for (int i = 0; i < n; ++i) r[i] = round_c(rb[i]);
  ws_ldiv(W, dx.data(), r.data());
  for (int i = 0; i < n; ++i) x[i] = x[i] - dx[i];
  return wnorm(dx.data(), w, n) / wnorm(x, w, n);
}
// :553-567 fixed-precision refinement step
static double fp_refine_step(MW& W, C* x, const C* b, const double* w) {
  int n = W.n;
  std::vector<C> r(n, cx(0.0)), dx(n);
  for (int j = 0; j < n; ++j) {
    C xj = x[j];
    for (int i = 0; i < n; ++i) r[i] = r[i] + W.a(i, j) * xj;
  }
  for (int i = 0; i < n; ++i) r[i] = r[i] - b[i];
  ws_ldiv(W, dx.data(), r.data());
  for (int i = 0; i < n; ++i) x[i] = x[i] - dx[i];
  return wnorm(dx.data(), w, n) / wnorm(x, w, n);
}
// :864-885
static double iterative_refinement(MW& W, C* x, const C* b, const double* w, double tol,
                                   int max_iters) {
  W.ldivs += 1;
  double delta = mp_refine_step(W, x, b, w);
  for (int i = 2; i <= max_iters; ++i) {
    W.ldivs += 1;
    double dp = mp_refine_step(W, x, b, w);
    if (dp < tol) return dp;
    if (dp > 0.5 * delta) return dp;
    delta = dp;
  }
  return delta;
}

// :598-682 Higham's 1-norm estimator of ‖diag(d_r)⁻¹ A⁻¹ diag(d_l)⁻¹‖∞
static double inverse_inf_norm_est(MW& W, const double* d_l, const double* d_r) {
  if (!W.factorized) factorize(W);
  const double* rs = W.scaled ? W.row_scaling.data() : nullptr;
  int n = W.n;
  std::vector<C> y(n);
  std::vector<double> x(n);
  for (int i = 0; i < n; ++i) x[i] = 1.0 / n;
  if (d_r)
    for (int i = 0; i < n; ++i) x[i] /= d_r[i];
  for (int i = 0; i < n; ++i) y[i] = cx(x[i]);
  lu_ldiv_adj(W, y.data());
  if (d_l)
    for (int i = 0; i < n; ++i) y[i] = y[i] / d_l[i];
  if (rs)
    for (int i = 0; i < n; ++i) y[i] = y[i] * rs[i];
  double g = 0.0;
  for (int i = 0; i < n; ++i) g += fast_abs(y[i]);
  for (int i = 0; i < n; ++i) y[i] = y[i] / fast_abs(y[i]);
  if (d_l)
    for (int i = 0; i < n; ++i) y[i] = y[i] / d_l[i];
  if (rs)
    for (int i = 0; i < n; ++i) y[i] = y[i] / rs[i];
  lu_ldiv(W, y.data());
  for (int i = 0; i < n; ++i) x[i] = d_r ? y[i].re / d_r[i] : y[i].re;
  int k = 2;
  while (true) {
    int j = 0;
    double mx = std::fabs(x[0]);
    for (int i = 1; i < n; ++i) {
      double ai = std::fabs(x[i]);
      if (ai > mx) {
        j = i;
        mx = ai;
      }
    }
    for (int i = 0; i < n; ++i) x[i] = 0.0;
    x[j] = 1.0;
    if (d_r)
      for (int i = 0; i < n; ++i) x[i] /= d_r[i];
    for (int i = 0; i < n; ++i) y[i] = cx(x[i]);
    lu_ldiv_adj(W, y.data());
    if (d_l)
      for (int i = 0; i < n; ++i) y[i] = y[i] / d_l[i];
    if (rs)
      for (int i = 0; i < n; ++i) y[i] = y[i] * rs[i];
    double gbar = g;
    g = 0.0;
    for (int i = 0; i < n; ++i) g += fast_abs(y[i]);
    if (g <= gbar) {
      g = gbar;
      break;
    }
    for (int i = 0; i < n; ++i) y[i] = y[i] / fast_abs(y[i]);
    if (d_l)
      for (int i = 0; i < n; ++i) y[i] = y[i] / d_l[i];
    if (rs)
      for (int i = 0; i < n; ++i) y[i] = y[i] / rs[i];
    lu_ldiv(W, y.data());
    for (int i = 0; i < n; ++i) x[i] = d_r ? y[i].re / d_r[i] : y[i].re;
    k += 1;
    double xinf = 0.0;
    for (int i = 0; i < n; ++i) xinf = jmax(xinf, std::fabs(x[i]));
    if (x[j] == xinf || k > 2) break;
  }
  return nanmin(g, INF);
}
// :684-707
static double inf_norm_mat(MW& W, const double* d_l, const double* d_r) {
  double nrm = -INF;
  int n = W.n;
  for (int i = 0; i < n; ++i) {
    double ni = 0.0;
    for (int j = 0; j < n; ++j) ni += d_r ? fast_abs(W.a(i, j)) * d_r[j] : fast_abs(W.a(i, j));
    if (d_l) ni *= d_l[i];
    nrm = max_fast(nrm, ni);  // @fastmath max
  }
  return nrm;
}
// :745-774
static double ws_cond(MW& W, const double* d_l, const double* d_r) {
  if (W.n == 1) {
    double a = cabs(W.A[0]);
    if (!d_l && !d_r) return 1.0 / a;
    if (!d_l) return 1.0 / (a * d_r[0]);
    if (!d_r) return 1.0 / (d_l[0] * a);
    return 1.0 / (d_l[0] * a * d_r[0]);
  }
  return inverse_inf_norm_est(W, d_l, d_r) * inf_norm_mat(W, d_l, d_r);
}

// numerical rank with rtol (one-sided Jacobi SVD); restates LA.rank(J, rtol=1e-14)
// used by the invalid-start branch of init! (src/tracker.jl:711-737)
static int rank_rtol(const C* A0, int n, double rtol) {
  std::vector<C> A(A0, A0 + (size_t)n * n);
  for (int sweep = 0; sweep < 60; ++sweep) {
    bool rotated = false;
    for (int p = 0; p < n - 1; ++p)
      for (int q = p + 1; q < n; ++q) {
        double alpha = 0, beta = 0;
        C g = cx(0.0);
        for (int i = 0; i < n; ++i) {
          C ap = A[(size_t)p * n + i], aq = A[(size_t)q * n + i];
          alpha += abs2(ap);
          beta += abs2(aq);
          g = g + conj(ap) * aq;
        }
        double ag = cabs(g);
        if (ag == 0.0 || ag <= 1e-15 * std::sqrt(alpha * beta)) continue;
        rotated = true;
        double zeta = (beta - alpha) / (2.0 * ag);
        double tt = (zeta >= 0 ? 1.0 : -1.0) / (std::fabs(zeta) + std::sqrt(1.0 + zeta * zeta));
        double c = 1.0 / std::sqrt(1.0 + tt * tt), s = c * tt;
        C ph = g / ag;  // e^{iφ}
        for (int i = 0; i < n; ++i) {
          C ap = A[(size_t)p * n + i], aq = A[(size_t)q * n + i];
          A[(size_t)p * n + i] = c * ap - s * (conj(ph) * aq);
          A[(size_t)q * n + i] = s * (ph * ap) + c * aq;
        }
      }
    if (!rotated) break;
  }
  std::vector<double> sv(n);
  double smax = 0;
  for (int j = 0; j < n; ++j) {
    double s = 0;
    for (int i = 0; i < n; ++i) s += abs2(A[(size_t)j * n + i]);
    sv[j] = std::sqrt(s);
    smax = std::max(smax, sv[j]);
  }
  int r = 0;
  for (int j = 0; j < n; ++j)
    if (sv[j] > rtol * smax) ++r;
  return r;
}

// ---------------------------------------------------------------------------------------
// Options (src/tracker.jl:45-140, src/endgame_tracker.jl:47-72)
// ---------------------------------------------------------------------------------------
struct TrackerParameters {
  double a = 0.125, beta_a = 1.0, beta_omega_p = 3.0, beta_tau = 0.4, strict_beta_tau = 0.3;
  int min_newton_iters = 2;
};
struct TrackerOptions {
  int max_steps = 10000;
  double max_step_size = INF, max_initial_step_size = INF;
  bool extended_precision = true;
  double min_step_size = 1e-48, min_rel_step_size = 0.0, terminate_cond = 1e13;
  TrackerParameters p;
};
struct EndgameOptions {
  double endgame_start = 0.1;
  int max_endgame_steps = 2000, max_endgame_extended_steps = 400;
  double min_cond = 1e6, min_cond_growth = 1e4, min_coord_growth = 100.0;
  bool zero_is_at_infinity = false, at_infinity_check = true, only_nonsingular = false;
  double singular_min_accuracy = 1e-6;
  int max_winding_number = 6;
  double val_finite_tol = 0.05, val_at_infinity_tol = 0.01;
  double sing_cond = 1e14, sing_accuracy = 1e-12, scaling_threshold = -30.0;
  int refine_steps = 3;
};

// TrackerCode (src/tracker.jl:164-178)
enum TC {
  TC_tracking = 0,
  TC_success,
  TC_terminated_max_steps,
  TC_terminated_accuracy_limit,
  TC_terminated_ill_conditioned,
  TC_terminated_invalid_startvalue,
  TC_terminated_invalid_startvalue_singular_jacobian,
  TC_terminated_step_size_too_small,
  TC_terminated_unknown
};
// EndgameTrackerCode (src/endgame_tracker.jl:100-117)
enum EC {
  EC_tracking = 0,
  EC_success,
  EC_at_infinity,
  EC_at_zero,
  EC_terminated_accuracy_limit,
  EC_terminated_invalid_startvalue,
  EC_terminated_invalid_startvalue_singular_jacobian,
  EC_terminated_ill_conditioned,
  EC_terminated_max_steps,
  EC_terminated_max_extended_steps,
  EC_terminated_max_winding_number,
  EC_terminated_step_size_too_small,
  EC_terminated_unknown,
  EC_post_check_failed,
  EC_excess_solution,
  EC_polyhedral_failed
};
// :119-139
static int ec_from_tc(int c) {
  switch (c) {
    case TC_success: return EC_success;
    case TC_terminated_max_steps: return EC_terminated_max_steps;
    case TC_terminated_accuracy_limit: return EC_terminated_accuracy_limit;
    case TC_terminated_ill_conditioned: return EC_terminated_ill_conditioned;
    case TC_terminated_invalid_startvalue: return EC_terminated_invalid_startvalue;
    case TC_terminated_invalid_startvalue_singular_jacobian:
      return EC_terminated_invalid_startvalue_singular_jacobian;
    case TC_terminated_step_size_too_small: return EC_terminated_step_size_too_small;
    case TC_terminated_unknown: return EC_terminated_unknown;
    default: return EC_tracking;
  }
}

// ---------------------------------------------------------------------------------------
// SegmentStepper (src/utils.jl:300-394)
// ---------------------------------------------------------------------------------------
struct SegmentStepper {
  C start, target;
  double abs_D = 0;
  bool forward = true;
  double s = 0, sp = 0;
  void init(C st, C tg) {
    start = st;
    target = tg;
    abs_D = cabs(tg - st);
    forward = cabs(st) < cabs(tg);
    s = sp = forward ? 0.0 : abs_D;
  }
  bool is_done() const { return forward ? s == abs_D : s == 0.0; }
  void step_success() { s = sp; }
  void propose(double ds) { sp = forward ? jmin(s + ds, abs_D) : jmax(s - ds, 0.0); }
  double dist_to_target() const { return forward ? abs_D - s : s; }
  double Ds() const { return forward ? sp - s : s - sp; }
  C t_at(double ss) const {
    if (forward) {
      if (ss == 0.0) return start;
      if (ss == abs_D) return target;
      return start + (ss / abs_D) * (target - start);
    } else {
      if (ss == abs_D) return start;
      if (ss == 0.0) return target;
      return target + (ss / abs_D) * (start - target);
    }
  }
  C t() const { return t_at(s); }
  C tp() const { return t_at(sp); }
  C Dt() const { return forward ? ((sp - s) / abs_D) * (target - start) : ((s - sp) / abs_D) * (target - start); }
};

// ---------------------------------------------------------------------------------------
// Predictor (src/predictor.jl)
// ---------------------------------------------------------------------------------------
enum { PADE21 = 0, HERMITE = 1 };

static C t_to_s_plane(C t, int m) {  // :338-351 (branch = 0)
  double r = fast_abs(t);
  if (t.im == 0.0 && t.re > 0) return cx(nthroot(r, m));
  double th = std::atan2(t.im, t.re);
  th = std::fmod(th, 2 * M_PI);
  if (th < 0) th += 2 * M_PI;  // mod2pi
  return nthroot(r, m) * cis(th / m);
}

// :354-371 (samples y[0..n) values, yd[0..n) derivatives)
static void cubic_hermite(C* xh, const C* y0, const C* yd0, C t0, const C* y1, const C* yd1, C t1, C t,
                          int n) {
  if (t0.im == 0.0 && t1.im == 0.0 && t.im == 0.0) {
    double T0 = t0.re, T1 = t1.re, T = t.re;
    double s = (T - T0) / (T1 - T0);
    double h00 = (1 + 2 * s) * ((1 - s) * (1 - s));
    double h10 = (T - T0) * ((1 - s) * (1 - s));
    double h01 = (s * s) * (3 - 2 * s);
    double h11 = (T - T0) * s * (s - 1);
    for (int i = 0; i < n; ++i) xh[i] = h00 * y0[i] + h10 * yd0[i] + h01 * y1[i] + h11 * yd1[i];
  } else {
    C s = cdiv(t - t0, t1 - t0);
    C one = cx(1.0), oms = one - s;
    C h00 = (one + 2.0 * s) * (oms * oms);
    C h10 = (t - t0) * (oms * oms);
    C h01 = (s * s) * (cx(3.0) - 2.0 * s);
    C h11 = (t - t0) * s * (s - one);
    for (int i = 0; i < n; ++i) xh[i] = h00 * y0[i] + h10 * yd0[i] + h01 * y1[i] + h11 * yd1[i];
  }
}

struct Predictor {  // :72-103
  int method = PADE21, order = 4;
  double trust_region = INF, local_error = INF, cond_H_xd = INF;
  std::vector<C> tx;  // 4 vectors: x, x¹, x², x³ (orders 0..3), stored contiguously
  C t = cx(NaN, 0), prev_t = cx(NaN, 0);
  double tx_norm[4] = {0, 0, 0, 0};
  std::vector<C> xtemp, u, prev_tx1;  // prev_tx1: 2 vectors
  int winding_number = 1;
  C s = cx(NaN, 0), prev_s = cx(NaN, 0);
  int n = 0;
  C* x0() { return &tx[0]; }
  C* x1() { return &tx[n]; }
  C* x2() { return &tx[2 * n]; }
  C* x3() { return &tx[3 * n]; }
  void resize(int nn, int m) {
    n = nn;
    tx.assign(4 * (size_t)n, cx(0.0));
    xtemp.assign(n, cx(0.0));
    u.assign(m, cx(0.0));
    prev_tx1.assign(2 * (size_t)n, cx(0.0));
  }
  void init() {  // :124-133
    cond_H_xd = 1.0;
    winding_number = 1;
    t = prev_t = cx(NaN, 0);
    s = prev_s = cx(NaN, 0);
    trust_region = local_error = NaN;
  }
};

// :158-284
static void predictor_update(Predictor& P, const Homotopy& H, const C* x, C t, MW& J,
                             const WeightedNorm& norm, const C* xhat) {
  int n = P.n, m = P.winding_number;
  for (int i = 0; i < n; ++i) {
    P.prev_tx1[i] = P.x0()[i];
    P.prev_tx1[n + i] = P.x1()[i];
  }
  P.prev_t = P.t;
  P.t = t;
  if (m > 1) {
    P.prev_s = P.s;
    P.s = t_to_s_plane(t, m);
  }
  if (!xhat) {
    P.local_error = NaN;
  } else {
    double Ds = fast_abs(t - P.prev_t);
    P.local_error = norm.dist(xhat, x) / std::pow(Ds, P.order);
  }
  for (int i = 0; i < n; ++i) P.x0()[i] = x[i];
  P.tx_norm[0] = norm(x);

  const double* w = norm.w.data();
  // ẋ = -H_x⁻¹ H_t
  H_taylor1(H, x, t, P.u.data());
  for (int i = 0; i < H.m; ++i) P.u[i] = -P.u[i];
  jac_ldiv(J, P.xtemp.data(), P.u.data(), nullptr);
  double delta = fp_refine_step(J, P.xtemp.data(), P.u.data(), w);
  P.cond_H_xd = delta / EPS;
  double tol1 = 1e-10;
  if (delta > tol1) iterative_refinement(J, P.xtemp.data(), P.u.data(), nullptr, tol1, 5);
  P.tx_norm[1] = norm(P.xtemp.data());
  for (int i = 0; i < n; ++i) P.x1()[i] = P.xtemp[i];
  if (m > 1) {
    P.method = HERMITE;
    P.order = 4;
    P.trust_region = P.tx_norm[0] / P.tx_norm[1];
    if (std::isnan(P.local_error)) P.local_error = std::pow(P.tx_norm[1] / P.tx_norm[0], 3);
    return;
  }
  H_taylorK(H, 2, P.tx.data(), t, P.u.data());
  for (int i = 0; i < H.m; ++i) P.u[i] = -P.u[i];
  jac_ldiv(J, P.xtemp.data(), P.u.data(), nullptr);
  double tol2 = 1e-10;
  if (delta > tol2) iterative_refinement(J, P.xtemp.data(), P.u.data(), w, tol2, 4);
  P.tx_norm[2] = norm(P.xtemp.data());
  for (int i = 0; i < n; ++i) P.x2()[i] = P.xtemp[i];

  H_taylorK(H, 3, P.tx.data(), t, P.u.data());
  for (int i = 0; i < H.m; ++i) P.u[i] = -P.u[i];
  jac_ldiv(J, P.xtemp.data(), P.u.data(), nullptr);
  double tol3 = 1e-4;
  if (delta > tol3) iterative_refinement(J, P.xtemp.data(), P.u.data(), w, tol3, 3);
  P.tx_norm[3] = norm(P.xtemp.data());
  for (int i = 0; i < n; ++i) P.x3()[i] = P.xtemp[i];

  double tau = INF;
  for (int i = 0; i < n; ++i) {
    double c1 = fast_abs(P.x1()[i]), c2 = fast_abs(P.x2()[i]), c3 = fast_abs(P.x3()[i]);
    double lam = jmax(1e-6, c1);
    c1 /= lam;
    c2 /= lam * lam;
    c3 /= lam * lam * lam;
    double tol = 1e-14 * jmax(c1, jmax(c2, c3));
    if (!((c1 <= tol && c2 <= tol && c3 <= tol) || c2 <= tol)) {
      double taui = (c2 / c3) / lam;
      if (taui < tau) tau = taui;
    }
  }
  if (!std::isfinite(tau)) tau = P.tx_norm[2] / P.tx_norm[3];
  if (!std::isfinite(tau)) {
    double mx = jmax(jmax(P.tx_norm[0], P.tx_norm[1]), jmax(P.tx_norm[2], P.tx_norm[3]));
    tau = P.tx_norm[0] / mx;
  }
  P.method = PADE21;
  P.order = 4;
  P.trust_region = tau;
  if (std::isnan(P.local_error)) {
    double it = 1.0 / tau;
    P.local_error = (it * it) * (it * it);
  }
}

// :286-329
static void predict(Predictor& P, C* xh, const C* x, C t, C Dt) {
  int n = P.n, m = P.winding_number;
  if (P.method == PADE21) {
    double lam = P.trust_region, lam2 = lam * lam, lam3 = lam * lam * lam;
    double tol = 1e-12;
    for (int i = 0; i < n; ++i) {
      C xi = P.x0()[i], x1 = P.x1()[i], x2 = P.x2()[i], x3 = P.x3()[i];
      double c = fast_abs(xi), c1 = fast_abs(x1), c2 = fast_abs(x2), c3 = fast_abs(x3);
      double a1 = c1 * lam, a2 = c2 * lam2, a3 = c3 * lam3;
      double tau = tol * std::sqrt(c * c + a1 * a1 + a2 * a2 + a3 * a3);
      if (c3 * lam3 <= tau || c2 * lam2 <= tau) {
        xh[i] = xi + Dt * (x1 + Dt * x2);
      } else {
        C di = cx(1.0) - cdiv(Dt * x3, x2);
        xh[i] = xi + Dt * (x1 + cdiv(Dt * x2, di));
      }
    }
  } else {
    C prev_s = t_to_s_plane(P.prev_t, m);
    C s = t_to_s_plane(t, m);
    C sp = t_to_s_plane(t + Dt, m);
    C prev_sm, sm;
    if (m == 2) {
      prev_sm = 2.0 * prev_s;
      sm = 2.0 * s;
    } else {
      prev_sm = (double)m * cpow_int(prev_s, m - 1);
      sm = (double)m * cpow_int(s, m - 1);
    }
    std::vector<C> py1(n), y1(n);
    for (int i = 0; i < n; ++i) {
      py1[i] = prev_sm * P.prev_tx1[n + i];
      y1[i] = sm * P.x1()[i];
    }
    cubic_hermite(xh, P.prev_tx1.data(), py1.data(), prev_s, P.x0(), y1.data(), s, sp, n);
  }
}

// ---------------------------------------------------------------------------------------
// Newton corrector (src/newton_corrector.jl)
// ---------------------------------------------------------------------------------------
enum NC { NEWT_CONVERGED = 0, NEWT_TERMINATED, NEWT_MAX_ITERS, NEWT_SINGULARITY };
struct NewtonResult {
  int code;
  double accuracy;
  int iters;
  double omega, theta, mu_low, norm_dx0;
};
struct Corrector {
  double a, h_a;
  std::vector<C> dx, r;
  std::vector<CDD> x_ext;
  void init(double aa, int n, int m) {
    a = aa;
    h_a = 2 * a * (std::sqrt(4 * a * a + 1) - 2 * a);
    dx.assign(n, cx(0.0));
    r.assign(m, cx(0.0));
    x_ext.assign(n, cdd(cx(0.0)));
  }
};

static void eval_dd(Corrector& NC, const Homotopy& H, const C* x, C t) {
  for (int i = 0; i < H.n; ++i) NC.x_ext[i] = cdd(x[i]);
  H_eval_dd(H, NC.x_ext.data(), t, NC.r.data());
}

// :55-78 (x̄ may alias x)
static double ext_refine_step(C* xbar, Corrector& NC, const Homotopy& H, const C* x, C t, MW& J,
                              const WeightedNorm& norm, bool simple_newton_step) {
  int n = H.n;
  H_eval_jac(H, x, t, NC.r.data(), J.A.data());
  eval_dd(NC, H, x, t);
  updated(J);
  jac_ldiv(J, NC.dx.data(), NC.r.data(), norm.w.data());
  iterative_refinement(J, NC.dx.data(), NC.r.data(), norm.w.data(), 1e-8, 3);
  for (int i = 0; i < n; ++i) xbar[i] = x[i] - NC.dx[i];
  if (simple_newton_step) {
    eval_dd(NC, H, xbar, t);
    jac_ldiv(J, NC.dx.data(), NC.r.data(), norm.w.data());
  }
  return norm(NC.dx.data());
}

// :80-205  (all iterates alias x̄)
static NewtonResult newton(C* xbar, Corrector& NC, const Homotopy& H, const C* x0, C t, MW& J,
                           const WeightedNorm& norm, double mu, double omega, bool extended_precision,
                           bool accurate_mu, bool first_correction) {
  int n = H.n;
  const double a = NC.a, h_a = NC.h_a;
  const double* w = norm.w.data();
  for (int i = 0; i < n; ++i) xbar[i] = x0[i];
  C* xi = xbar;
  double mu_low = NaN, theta = NaN, norm_dxi = NaN, norm_dxim1 = NaN, norm_dx0 = NaN;
  double abar = a;
  C* dx = NC.dx.data();
  C* r = NC.r.data();
  for (int i = 0; i <= 10; ++i) {
    H_eval_jac(H, xi, t, r, J.A.data());
    if (extended_precision) eval_dd(NC, H, xi, t);
    updated(J);
    jac_ldiv(J, dx, r, w);
    if (extended_precision) iterative_refinement(J, dx, r, w, abar * abar, 3);
    norm_dxi = norm(dx);
    if (std::isnan(norm_dxi)) {
      return NewtonResult{NEWT_SINGULARITY, norm(dx), i + 1, omega, theta, mu_low, norm_dx0};
    }
    for (int k = 0; k < n; ++k) xi[k] = xi[k] - dx[k];
    if (i == 0) norm_dx0 = norm_dxi;
    if (i == 1) omega = 2 * norm_dxi / (norm_dxim1 * norm_dxim1);
    if (i >= 1) theta = norm_dxi / norm_dxim1;
    if ((i >= 1 && theta > abar) || (i == 0 && !first_correction && 0.125 * norm_dx0 * omega > h_a)) {
      return NewtonResult{NEWT_TERMINATED, norm(dx), i + 1, omega, theta, mu_low, norm_dx0};
    } else if (omega * norm_dxi * norm_dxi < 2 * mu * std::sqrt(1 - 2 * h_a)) {
      H_eval_jac(H, xi, t, r, J.A.data());
      updated(J);
      if (extended_precision) {
        jac_ldiv(J, dx, r, nullptr);
        mu_low = norm(dx);
        eval_dd(NC, H, xi, t);
      }
      jac_ldiv(J, dx, r, nullptr);
      if (extended_precision) iterative_refinement(J, dx, r, w, abar * abar, 3);
      for (int k = 0; k < n; ++k) xi[k] = xi[k] - dx[k];
      double norm_dxi1 = norm(dx);
      if (std::isnan(norm_dxi1)) {
        return NewtonResult{NEWT_SINGULARITY, norm(dx), i + 1, omega, theta, mu_low, norm_dx0};
      } else if (norm_dxi1 > std::sqrt(norm_dxi)) {
        theta = norm_dxi1 / norm_dxi;
        return NewtonResult{NEWT_TERMINATED, norm_dxi1, i + 2, omega, theta, mu_low, norm_dx0};
      }
      if (norm_dxi1 > 2 * mu && extended_precision) {
        eval_dd(NC, H, xi, t);
        jac_ldiv(J, dx, r, nullptr);
        norm_dxi = norm_dxi1;
        mu = norm_dxi1 = norm(dx);
      } else if (norm_dxi1 > 2 * mu || accurate_mu) {
        H_eval(H, xi, t, r);
        jac_ldiv(J, dx, r, nullptr);
        mu = norm(dx);
      } else {
        mu = norm_dxi1;
      }
      if (i == 0) {
        double wbar = 2 * norm_dxi / (norm_dxi1 * norm_dxi1);
        if (wbar < omega)
          omega = wbar;
        else
          omega *= 0.25;
      }
      return NewtonResult{NEWT_CONVERGED, mu, i + 2, omega, theta, mu_low, norm_dx0};
    }
    norm_dxim1 = norm_dxi;
    if (i >= 1) abar *= abar;
  }
  return NewtonResult{NEWT_MAX_ITERS, mu, 11, omega, theta, mu_low, norm_dx0};
}

// :207-286 (x₁, x₂ alias x̄)
static void init_newton(bool& valid, double& omega_out, double& mu_out, C* xbar, Corrector& NC,
                        const Homotopy& H, const C* x0, C t, MW& J, const WeightedNorm& norm,
                        double a, bool extended_precision) {
  int n = H.n;
  C* dx = NC.dx.data();
  C* r = NC.r.data();
  const double* w = norm.w.data();
  H_eval_jac(H, x0, t, r, J.A.data());
  if (extended_precision) eval_dd(NC, H, x0, t);
  updated(J);
  jac_ldiv(J, dx, r, w);
  double v = norm(dx) + EPS;
  valid = false;
  double omega = NaN, mu = NaN;
  double eps_ = std::sqrt(v);
  for (int k = 1; k <= 3; ++k) {
    for (int i = 0; i < n; ++i) xbar[i] = x0[i] + cx(eps_ * w[i]);
    H_eval_jac(H, xbar, t, r, J.A.data());
    if (extended_precision) eval_dd(NC, H, xbar, t);
    updated(J);
    jac_ldiv(J, dx, r, w);
    for (int i = 0; i < n; ++i) xbar[i] = xbar[i] - dx[i];
    double norm_dx0 = norm(dx);
    if (extended_precision)
      eval_dd(NC, H, xbar, t);
    else
      H_eval(H, xbar, t, r);
    jac_ldiv(J, dx, r, w);
    for (int i = 0; i < n; ++i) xbar[i] = xbar[i] - dx[i];
    double norm_dx1 = norm(dx) + EPS;
    if (norm_dx1 < a * norm_dx0) {
      omega = 2 * norm_dx1 / (norm_dx0 * norm_dx0);
      mu = norm_dx1;
      if (omega * mu > std::pow(a, 7)) {
        NewtonResult rr = newton(xbar, NC, H, xbar, t, J, norm, std::pow(a, 7) / omega, omega,
                                 extended_precision, true, false);
        if (rr.code == NEWT_CONVERGED) {
          valid = true;
          omega = rr.omega;
          mu = rr.accuracy;
        } else {
          valid = false;
        }
      } else {
        valid = true;
        break;
      }
    } else {
      eps_ *= std::sqrt(eps_);
    }
  }
  omega_out = omega;
  mu_out = mu;
}

// ---------------------------------------------------------------------------------------
// Tracker (src/tracker.jl)
// ---------------------------------------------------------------------------------------
static inline double h_fn(double a) { return 2 * a * (std::sqrt(4 * a * a + 1) - 2 * a); }  // :517

struct Tracker {
  const Homotopy* H = nullptr;
  TrackerOptions opt;
  Predictor pred;
  Corrector corr;
  // state (:307-338)
  std::vector<C> x, xh, xb;
  SegmentStepper ss;
  double Ds_prev = 0, accuracy = 0, omega = 1, omega_prev = 1, mu = EPS, tau = INF, norm_dx0 = NaN;
  int trace_iters = 0;  // Newton iterations of the last step (step trace only)
  bool extended_prec = false, used_extended_prec = false, refined_extended_prec = false,
       keep_extended_prec = false, use_strict_beta_tau = false;
  WeightedNorm norm;
  MW J;
  int code = TC_tracking;
  long accepted_steps = 0, rejected_steps = 0, last_steps_failed = 0, ext_accepted_steps = 0,
       ext_rejected_steps = 0;
  int n = 0;

  void setup(const Homotopy& HH, const TrackerOptions& o) {
    H = &HH;
    opt = o;
    n = HH.n;
    x.assign(n, cx(0.0));
    xh.assign(n, cx(0.0));
    xb.assign(n, cx(0.0));
    norm.n = n;
    norm.w.assign(n, 1.0);
    J.resize(n);
    pred.resize(n, HH.m);
    corr.init(opt.p.a, n, HH.m);
    ss.init(cx(1.0), cx(0.0));
  }
  long steps() const { return accepted_steps + rejected_steps; }
  long ext_steps() const { return ext_accepted_steps + ext_rejected_steps; }
  bool last_step_failed() const { return last_steps_failed > 0; }
};

// :520-539
static double initial_step_size(Tracker& T) {
  double a = T.opt.p.beta_a * T.opt.p.a;
  int p = T.pred.order;
  double omega = T.omega;
  double e = T.pred.local_error;
  if (std::isinf(e)) e = 1e5;
  double tau = T.pred.trust_region;
  double Ds1 = nthroot((std::sqrt(1 + 2 * h_fn(a)) - 1) / (omega * e), p) / T.opt.p.beta_omega_p;
  double Ds2 = T.opt.p.beta_tau * tau;
  double Ds = nanmin(Ds1, Ds2);
  return jmin(jmin(Ds, T.opt.max_step_size), T.opt.max_initial_step_size);
}

// :541-588
static void update_stepsize(Tracker& T, const NewtonResult& res) {
  double a = T.opt.p.beta_a * T.opt.p.a;
  int p = T.pred.order;
  double omega = jclamp(T.omega + 2 * (T.omega - T.omega_prev), T.omega, 8 * T.omega);
  double tau = T.tau;
  double Ds;
  if (res.code == NEWT_CONVERGED) {
    double e = T.pred.local_error;
    double Ds1 = nthroot((std::sqrt(1 + 2 * h_fn(a)) - 1) / (omega * e), p) / T.opt.p.beta_omega_p;
    double Ds2 = T.opt.p.beta_tau * tau;
    if (T.use_strict_beta_tau || T.ss.dist_to_target() < Ds2) Ds2 = T.opt.p.strict_beta_tau * tau;
    Ds = jmin(nanmin(Ds1, Ds2), T.opt.max_step_size);
    if (T.use_strict_beta_tau && T.ss.dist_to_target() < Ds) Ds *= T.opt.p.strict_beta_tau;
    Ds = jmin(Ds, 10 * T.Ds_prev);
    if (T.last_step_failed()) Ds = jmin(Ds, T.Ds_prev);
  } else {
    int j = res.iters - 2;
    int N = (j >= 0 && j < 62) ? (1 << j) : 0;  // Julia: 1 << -1 == 0
    double Theta_j = nthroot(res.theta, N);
    double h_Theta_j = h_fn(Theta_j);
    double h_a = h_fn(0.5 * a);
    if (std::isnan(Theta_j) || res.code == NEWT_SINGULARITY || std::isnan(res.accuracy) ||
        res.iters == 1 || h_Theta_j < h_a) {
      Ds = 0.25 * T.ss.Ds();
    } else {
      Ds = nthroot((std::sqrt(1 + 2 * h_fn(0.5 * a)) - 1) / (std::sqrt(1 + 2 * h_fn(Theta_j)) - 1), p) *
           T.ss.Ds();
    }
  }
  T.ss.propose(Ds);
}

// :591-619
static void check_terminated(Tracker& T) {
  double tol_acc;
  if (T.extended_prec || !T.opt.extended_precision) {
    double a = T.opt.p.a;
    tol_acc = std::pow(a, (1 << T.opt.p.min_newton_iters) - 1) * h_fn(a);
  } else {
    tol_acc = INF;
  }
  C tp = T.ss.tp(), t = T.ss.t();
  double at = fast_abs(t);
  // 2eps(|t|): spacing of floats at |t|
  double eps_t = (at == 0.0) ? std::numeric_limits<double>::denorm_min()
                             : std::nextafter(at, INF) - at;
  if (std::isinf(at)) eps_t = NaN;
  if (T.ss.is_done()) {
    T.code = TC_success;
  } else if (T.steps() >= T.opt.max_steps) {
    T.code = TC_terminated_max_steps;
  } else if (T.omega * T.mu > tol_acc) {
    T.code = TC_terminated_accuracy_limit;
  } else if (T.ss.Ds() < T.opt.min_step_size) {
    T.code = TC_terminated_step_size_too_small;
  } else if (fast_abs(tp - t) <= 2 * eps_t) {
    T.code = TC_terminated_step_size_too_small;
  } else if (T.opt.min_rel_step_size > 0 && !(tp.re == T.ss.target.re && tp.im == T.ss.target.im) &&
             fast_abs(tp - t) < fast_abs(t) * T.opt.min_rel_step_size) {
    T.code = TC_terminated_step_size_too_small;
  }
}

// :788-813
static void use_extended_precision(Tracker& T) {
  if (!T.opt.extended_precision) return;
  if (T.extended_prec) return;
  T.extended_prec = true;
  T.used_extended_prec = true;
  double mu = T.mu;
  for (int i = 0; i < 2; ++i)
    mu = ext_refine_step(T.x.data(), T.corr, *T.H, T.x.data(), T.ss.t(), T.J, T.norm, false);
  T.mu = jmax(mu, EPS);
}
// :768-786
static void update_precision(Tracker& T, double mu_low) {
  if (!T.opt.extended_precision) return;
  double a = T.opt.p.a, mu = T.mu, omega = T.omega;
  if (T.extended_prec && !T.keep_extended_prec && !std::isnan(mu_low) && mu_low > mu) {
    if (mu_low * omega < std::pow(a, 7) * h_fn(a)) {
      T.extended_prec = false;
      T.mu = mu_low;
    }
  } else if (mu * omega > std::pow(a, 5) * h_fn(a)) {
    use_extended_precision(T);
  }
}
// :815-844
static double refine_current_solution(Tracker& T, double min_tol, int nsteps) {
  double mu = T.accuracy;
  C t = T.ss.t();
  double mub = ext_refine_step(T.xb.data(), T.corr, *T.H, T.x.data(), t, T.J, T.norm, false);
  if (mub < mu) {
    T.x = T.xb;
    mu = mub;
  }
  int k = 1;
  while (mu > min_tol && k <= nsteps) {
    mub = ext_refine_step(T.xb.data(), T.corr, *T.H, T.x.data(), t, T.J, T.norm, true);
    if (mub < mu) {
      T.x = T.xb;
      mu = mub;
    }
    k += 1;
  }
  return mu;
}

static void update_predictor(Tracker& T, const C* xhat) {  // :621-624
  predictor_update(T.pred, *T.H, T.x.data(), T.ss.t(), T.J, T.norm, xhat);
}

// :639-754
static bool tracker_init(Tracker& T, const C* x1, C t1, C t0, double omega_in = NaN, double mu_in = NaN,
                         double tau_in = INF, double max_initial_step_size = INF, bool keep_steps = false,
                         bool extended_precision = false) {
  int n = T.n;
  for (int i = 0; i < n; ++i) T.x[i] = x1[i];
  T.ss.init(t1, t0);
  T.Ds_prev = 0.0;
  T.accuracy = EPS;
  T.omega = 1.0;
  T.keep_extended_prec = false;
  T.use_strict_beta_tau = false;
  T.refined_extended_prec = false;  // a fresh Tracker per path (informational flag only)
  T.norm.init(T.x.data());
  T.J.factorizations = T.J.ldivs = 0;
  T.code = TC_tracking;
  if (!keep_steps) {
    T.accepted_steps = T.rejected_steps = 0;
    T.ext_accepted_steps = T.ext_rejected_steps = 0;
  }
  T.last_steps_failed = 0;
  C t = T.ss.t();
  bool valid;
  double omega = omega_in, mu = mu_in;
  if (std::isnan(omega) || std::isnan(mu)) {
    double a = T.opt.p.a;
    init_newton(valid, omega, mu, T.xb.data(), T.corr, *T.H, T.x.data(), t, T.J, T.norm, a,
                extended_precision);
    if (!valid && !extended_precision) {
      extended_precision = true;
      init_newton(valid, omega, mu, T.xb.data(), T.corr, *T.H, T.x.data(), t, T.J, T.norm, a, true);
    }
  } else {
    valid = true;
  }
  T.used_extended_prec = T.extended_prec = extended_precision;
  if (!std::isnan(omega)) T.omega = omega;
  if (valid) {
    T.accuracy = mu;
    T.mu = jmax(mu, EPS);
  } else {
    H_eval_jac(*T.H, T.x.data(), t, T.corr.r.data(), T.J.A.data());
    bool anynan = false;
    for (auto& z : T.J.A) anynan = anynan || isnanC(z);
    int corank = 0;
    if (anynan) {
      T.code = TC_terminated_invalid_startvalue;
      corank = 0;
    } else {
      corank = n - rank_rtol(T.J.A.data(), n, 1e-14);
    }
    T.code = corank > 0 ? TC_terminated_invalid_startvalue_singular_jacobian : TC_terminated_invalid_startvalue;
    return false;
  }
  T.tau = tau_in;
  H_eval_jac(*T.H, T.x.data(), t, T.corr.r.data(), T.J.A.data());
  updated(T.J);
  T.pred.init();
  update_predictor(T, nullptr);
  T.tau = T.pred.trust_region;
  double Ds = initial_step_size(T);
  Ds = jmax(jmin(Ds, max_initial_step_size), T.opt.min_step_size);
  T.ss.propose(Ds);
  T.omega_prev = T.omega;
  return T.code == TC_tracking;
}

// :756-766
static void tracker_init_t0(Tracker& T, C t0, double max_initial_step_size = INF) {
  T.code = TC_tracking;
  T.ss.init(T.ss.t(), t0);
  double Ds = initial_step_size(T);
  Ds = jmin(Ds, max_initial_step_size);
  T.ss.propose(Ds);
  T.Ds_prev = 0.0;
}

// Optional step trace of one path (test infrastructure: finding the first step where two
// trackers' decisions part). Per step, HCO_TRACE_FIELDS doubles: t (re, im), Δs tried, trust
// region, ω and μ before the step, accepted, Newton iterations, ‖x‖∞ after, next Δs, ω and
// accuracy after, extended precision, tracker code, endgame steps so far.
constexpr int HCO_TRACE_FIELDS = 15;
static bool tracker_step_impl(Tracker& T);
static thread_local std::vector<double>* tl_trace = nullptr;
static thread_local const long* tl_trace_eg = nullptr;
static int64_t g_trace_path = -1;  // 0-based path index to trace (-1: none)
static Slp g_slp;  // program of F for hco_track (hco_set_slp)
static bool g_slp_on = false;
static std::vector<C> g_param_p, g_param_q;  // parameter homotopy of g_slp (hco_set_slp_parameters)
static std::vector<double> g_trace;

// :851-926
static bool tracker_step(Tracker& T) {
  const double tr_t_re = T.ss.t().re, tr_t_im = T.ss.t().im, tr_ds = T.ss.Ds(), tr_tau = T.tau,
               tr_omega = T.omega, tr_mu = T.mu;
  bool ok = tracker_step_impl(T);
  if (tl_trace) {
    double nx = 0;
    for (const C& v : T.x) nx = std::max(nx, cabs(v));
    double rec[HCO_TRACE_FIELDS] = {tr_t_re, tr_t_im, tr_ds, tr_tau, tr_omega, tr_mu, (double)ok,
                                    (double)T.trace_iters, nx, T.ss.Ds(), T.omega, T.accuracy,
                                    (double)T.extended_prec, (double)T.code,
                                    tl_trace_eg ? (double)*tl_trace_eg : 0.0};
    tl_trace->insert(tl_trace->end(), rec, rec + HCO_TRACE_FIELDS);
  }
  return ok;
}

static bool tracker_step_impl(Tracker& T) {
  C t = T.ss.t(), Dt = T.ss.Dt(), tp = T.ss.tp();
  predict(T.pred, T.xh.data(), T.x.data(), t, Dt);
  T.norm.update(T.xh.data());
  NewtonResult res = newton(T.xb.data(), T.corr, *T.H, T.xh.data(), tp, T.J, T.norm, T.mu, T.omega,
                            T.extended_prec, false, T.accepted_steps == 0);
  if (res.code == NEWT_CONVERGED) {
    T.x = T.xb;
    T.Ds_prev = T.ss.Ds();
    T.ss.step_success();
    T.accuracy = res.accuracy;
    T.mu = jmax(res.accuracy, EPS);
    T.omega_prev = T.omega;
    T.omega = jmax(jmax(res.omega, 0.5 * T.omega), 0.1);
    update_precision(T, res.mu_low);
    if (T.ss.is_done() && T.opt.extended_precision && T.accuracy > 1e-14) {
      T.accuracy = refine_current_solution(T, 1e-14, 3);
      T.refined_extended_prec = true;
    }
    update_predictor(T, T.xh.data());
    T.tau = T.pred.trust_region;
    T.accepted_steps += 1;
    T.ext_accepted_steps += T.extended_prec;
    T.last_steps_failed = 0;
  } else {
    T.rejected_steps += 1;
    T.ext_rejected_steps += T.extended_prec;
    T.last_steps_failed += 1;
  }
  T.norm_dx0 = res.norm_dx0;
  T.trace_iters = res.iters;
  update_stepsize(T, res);
  check_terminated(T);
  return !T.last_step_failed();
}

// LA.cond(tracker, x, t, d_l, d_r) (src/tracker.jl:509-514)
static double tracker_cond(Tracker& T, const C* x, C t, const double* d_l, const double* d_r) {
  H_eval_jac(*T.H, x, t, T.corr.r.data(), T.J.A.data());
  updated(T.J);
  return ws_cond(T.J, d_l, d_r);
}

// ---------------------------------------------------------------------------------------
// Valuation (src/valuation.jl)
// ---------------------------------------------------------------------------------------
struct Valuation {
  int n = 0;
  std::vector<double> val_x, val_tx, Dval_x, Dval_tx;
  std::vector<double> nu2, nu1, vd2, vd1, lx2, lx1, lxd2, lxd1;
  double logt2 = NaN, logt1 = NaN;
  void resize(int nn) {
    n = nn;
    for (auto* v : {&val_x, &val_tx, &Dval_x, &Dval_tx, &nu2, &nu1, &vd2, &vd1, &lx2, &lx1, &lxd2, &lxd1})
      v->assign(n, 0.0);
  }
  void init() {  // :38-49
    resize(n);
    logt2 = logt1 = NaN;
  }
};
static inline double nu_f(C x, C xd, double t) {  // :52-61
  double xx = abs2(x);
  double mu = x.re * xd.re + x.im * xd.im;
  return t * (mu / xx);
}
static inline void nu_nu1(C x, C xd, C x2, double t, double& a, double& b) {  // :63-77
  double xx = abs2(x);
  double mu = x.re * xd.re + x.im * xd.im;
  double l = mu / xx;
  double mu1 = x.re * x2.re + xd.re * xd.re + x.im * x2.im + xd.im * xd.im;
  double l1 = mu1 / xx - 2 * l * l;
  a = t * l;
  b = t * l1 + l;
}
static inline double finite_diff(double nu, double s, double nu2, double s2, double nu1,
                                 double s1) {  // :138-141
  double D1 = s - s1, D2 = s - s2, D12 = s1 - s2;
  return (D2 * nu1) / (D12 * D1) - ((D12 + D2) * nu2) / (D12 * D2) - (D12 * nu) / (D1 * D2);
}
static void valuation_update(Valuation& V, Predictor& P, double t) {  // :82-124
  double logt = std::log(t);
  bool diff = P.winding_number > 1 && !std::isnan(V.logt2);
  for (int i = 0; i < V.n; ++i) {
    C xi = P.x0()[i], xdi = P.x1()[i], x2i = P.x2()[i], x3i = P.x3()[i];
    double logxi = std::log(fast_abs(xi));
    double logxdi = std::log(fast_abs(xdi));
    if (diff) {
      double nui = nu_f(xi, xdi, t);
      double Dnui = finite_diff(nui, logt, V.nu2[i], V.logt2, V.nu1[i], V.logt1);
      V.val_x[i] = nui;
      V.Dval_x[i] = Dnui;
      double val_xdi = finite_diff(logxdi, logt, V.lxd2[i], V.logt2, V.lxd1[i], V.logt1);
      double Dval_xdi = finite_diff(val_xdi, logt, V.vd2[i], V.logt2, V.vd1[i], V.logt1);
      V.val_tx[i] = val_xdi + 1;
      V.Dval_tx[i] = Dval_xdi;
    } else {
      double nui, nu1;
      nu_nu1(xi, xdi, 2.0 * x2i, t, nui, nu1);
      V.val_x[i] = nui;
      V.Dval_x[i] = t * nu1;
      double old = V.nu2[i];
      V.nu2[i] = nui;
      V.nu1[i] = old;
      double vxd;
      nu_nu1(xdi, 2.0 * x2i, 6.0 * x3i, t, vxd, nu1);
      V.val_tx[i] = vxd + 1;
      V.Dval_tx[i] = t * nu1;
    }
    double o = V.lx2[i];
    V.lx2[i] = logxi;
    V.lx1[i] = o;
    o = V.lxd2[i];
    V.lxd2[i] = logxdi;
    V.lxd1[i] = o;
  }
  V.logt1 = V.logt2;
  V.logt2 = logt;
}
// :143-173
static void at_infinity_tol(std::vector<double>& tols, const Valuation& V, double finite_tol,
                            bool zero_is_finite) {
  for (int i = 0; i < V.n; ++i) {
    double vx = V.val_x[i];
    double a1 = std::fabs(1.0 - V.val_tx[i] / vx), a2 = std::fabs(V.Dval_x[i] / vx),
           a3 = std::fabs(V.Dval_tx[i] / V.val_tx[i]);
    double e = jmax(jmax(a1, a2), a3);
    if (std::isnan(e)) {
      tols[i] = INF;
      continue;
    }
    if (vx + e < -finite_tol)
      tols[i] = e;
    else if (!zero_is_finite && vx - e > -finite_tol)
      tols[i] = e;
    else
      tols[i] = INF;
  }
}
// :175-205
static bool val_is_finite(const Valuation& V, double finite_tol, bool zero_is_finite, int max_wn) {
  double delta = 1.0 / max_wn;
  for (int i = 0; i < V.n; ++i) {
    double vx = V.val_x[i];
    if (std::fabs(vx) < finite_tol) {
      if (!(std::fabs(V.Dval_x[i]) < finite_tol) || V.val_tx[i] < 0.5 * delta) return false;
    } else if (zero_is_finite && vx > (delta - finite_tol)) {
      double a1 = std::fabs(1.0 - V.val_tx[i] / vx), a2 = std::fabs(V.Dval_x[i] / vx),
             a3 = std::fabs(V.Dval_tx[i] / V.val_tx[i]);
      double e = jmax(jmax(a1, a2), a3);
      if (!(e < finite_tol)) return false;
    } else {
      return false;
    }
  }
  return true;
}
// :207-228
static void estimate_winding_number(const Valuation& V, int max_wn, int& m, double& err_out) {
  m = 1;
  double min_err = INF;
  for (int k = 1; k <= max_wn; ++k) {
    double err = 0.0;
    for (int i = 0; i < V.n; ++i) {
      double mv = k * V.val_tx[i];
      double ei = std::fabs(std::nearbyint(mv) - mv);
      err = (ei > err) ? ei : err;
    }
    if (err < min_err) {
      m = k;
      min_err = err;
    }
  }
  err_out = min_err;
}

// ---------------------------------------------------------------------------------------
// EndgameTracker (src/endgame_tracker.jl)
// ---------------------------------------------------------------------------------------
struct EndgameTracker {
  Tracker T;
  EndgameOptions opt;
  // state (:177-215)
  int code = EC_tracking;
  bool singular_endgame = false;
  Valuation val;
  int winding_number = 0;  // 0 == nothing
  std::vector<C> solution;
  double accuracy = NaN, cond = 1.0;
  bool singular = false;
  long steps_eg = 0, ext_steps_eg_start = 0;
  bool jtz_failed[2] = {false, false};
  std::vector<C> last_point;
  double last_t = NaN;
  std::vector<double> row_scaling, col_scaling;
  std::vector<double> at_inf_starts, at_inf_tols, at_inf_abs_coords, at_inf_conds;
  std::vector<C> samples[3];  // each 2n: values then derivatives
  double sample_times[3] = {0, 0, 0}, sample_conds[3] = {0, 0, 0};
  double singular_start = NaN;
  long singular_steps = 0;
  std::vector<C> prediction, prev_prediction;
  int n = 0;

  void setup(const Homotopy& H, const TrackerOptions& to, const EndgameOptions& eo) {
    T.setup(H, to);
    opt = eo;
    n = H.n;
    val.resize(n);
    solution.assign(n, cx(NaN, NaN));
    last_point.assign(n, cx(0.0));
    row_scaling.assign(H.m, 0.0);
    col_scaling.assign(n, 0.0);
    at_inf_starts.assign(n, 0.0);
    at_inf_tols.assign(n, 0.0);
    at_inf_abs_coords.assign(n, 0.0);
    at_inf_conds.assign(n, 0.0);
    for (auto& s : samples) s.assign(2 * (size_t)n, cx(0.0));
    prediction.assign(n, cx(0.0));
    prev_prediction.assign(n, cx(0.0));
  }
};

// :260-294
static void eg_init(EndgameTracker& E, const C* x, double t1) {
  E.T.opt.min_rel_step_size = 0.0;
  tracker_init(E.T, x, cx(t1), cx(0.0));
  E.code = ec_from_tc(E.T.code);
  E.singular_endgame = false;
  E.jtz_failed[0] = E.jtz_failed[1] = false;
  E.val.init();
  E.winding_number = 0;
  for (auto& s : E.solution) s = cx(NaN, NaN);
  E.accuracy = NaN;
  E.cond = NaN;
  E.singular = false;
  E.steps_eg = 0;
  E.ext_steps_eg_start = std::numeric_limits<long>::max();
  for (auto& v : E.row_scaling) v = 1.0;
  for (auto& v : E.col_scaling) v = 1.0;
  for (auto& v : E.at_inf_starts) v = NaN;
  E.singular_steps = 0;
}

// :695-721
static void tracking_stopped(EndgameTracker& E) {
  Tracker& T = E.T;
  E.accuracy = T.accuracy;
  if (E.code == EC_success && E.accuracy > 1e-14) refine_current_solution(T, 1e-14, E.opt.refine_steps);
  E.solution = T.x;
  E.winding_number = 0;
  if (E.code == EC_success) {
    E.col_scaling = T.norm.w;
    skeel_row_scaling(E.row_scaling.data(), T.J.A.data(), E.n, E.col_scaling.data(), E.opt.scaling_threshold);
    E.cond = tracker_cond(T, E.solution.data(), cx(0.0), E.row_scaling.data(), E.col_scaling.data());
    E.singular = E.cond > E.opt.sing_cond || E.accuracy > E.opt.sing_accuracy;
  }
}

// :402-422
static bool check_finite(EndgameTracker& E) {
  if (!val_is_finite(E.val, E.opt.val_finite_tol, !E.opt.zero_is_at_infinity, E.opt.max_winding_number))
    return false;
  int m;
  double merr;
  estimate_winding_number(E.val, E.opt.max_winding_number, m, merr);
  if (merr < E.opt.val_finite_tol) {
    if (m == 1 && !E.jtz_failed[0]) return false;
    E.winding_number = m;
    return true;
  }
  return false;
}

// :424-499
static bool check_at_infinity(EndgameTracker& E) {
  if (!E.opt.at_infinity_check) return false;
  Tracker& T = E.T;
  at_infinity_tol(E.at_inf_tols, E.val, E.opt.val_finite_tol, !E.opt.zero_is_at_infinity);
  double kappa = NaN;
  double t = T.ss.t().re;
  for (int i = 0; i < E.n; ++i) {
    double toli = E.at_inf_tols[i];
    if (toli < E.opt.val_at_infinity_tol) {
      if (std::isnan(E.at_inf_starts[i])) {
        bool allnan = true;
        for (double v : E.at_inf_starts) allnan = allnan && std::isnan(v);
        if (allnan) {
          E.col_scaling = T.norm.w;
          skeel_row_scaling(E.row_scaling.data(), T.J.A.data(), E.n, E.col_scaling.data(),
                            E.opt.scaling_threshold);
        }
        kappa = ws_cond(T.J, E.row_scaling.data(), E.col_scaling.data());
        E.at_inf_conds[i] = kappa;
        E.at_inf_abs_coords[i] = fast_abs(T.x[i]);
        E.at_inf_starts[i] = t;
      } else {
        if (std::isnan(kappa)) kappa = ws_cond(T.J, E.row_scaling.data(), E.col_scaling.data());
        double vi = E.val.val_x[i];
        bool at_zero = E.val.val_x[i] > 0;
        double cond_growth = kappa / E.at_inf_conds[i];
        double coord_growth = at_zero ? E.at_inf_abs_coords[i] / fast_abs(T.x[i])
                                      : fast_abs(T.x[i]) / E.at_inf_abs_coords[i];
        double lim = jclamp(std::pow(0.25, 4 * vi), 20.0, E.opt.min_coord_growth);
        if (coord_growth > lim &&
            (cond_growth > E.opt.min_cond_growth || kappa > jmax(1e8, E.opt.min_cond))) {
          E.code = at_zero ? EC_at_zero : EC_at_infinity;
          return true;
        }
      }
    } else if (!std::isnan(E.at_inf_starts[i])) {
      E.at_inf_starts[i] = NaN;
    }
  }
  return false;
}

// :630-662
static void add_sample(EndgameTracker& E, double t) {
  Tracker& T = E.T;
  int m = E.winding_number;
  double s = nthroot(t, m);
  double mu = m * std::pow(s, m - 1);
  double kappa = ws_cond(T.J, E.row_scaling.data(), E.col_scaling.data());
  int n = E.n;
  if (E.singular_steps <= 2) {
    auto& tyk = E.samples[E.singular_steps];
    for (int i = 0; i < n; ++i) {
      tyk[i] = T.pred.x0()[i];
      tyk[n + i] = mu * T.pred.x1()[i];
    }
    E.sample_times[E.singular_steps] = s;
    E.sample_conds[E.singular_steps] = kappa;
  } else {
    std::swap(E.samples[0], E.samples[1]);
    std::swap(E.samples[1], E.samples[2]);
    E.sample_times[0] = E.sample_times[1];
    E.sample_conds[0] = E.sample_conds[1];
    E.sample_times[1] = E.sample_times[2];
    E.sample_conds[1] = E.sample_conds[2];
    auto& ty3 = E.samples[2];
    for (int i = 0; i < n; ++i) {
      ty3[i] = T.pred.x0()[i];
      ty3[n + i] = mu * T.pred.x1()[i];
    }
    E.sample_times[2] = s;
    E.sample_conds[2] = kappa;
  }
}

// :664-693
static double predict_endpoint(EndgameTracker& E) {
  if (E.singular_steps < 2) return INF;
  int n = E.n;
  if (E.singular_steps == 2) {
    cubic_hermite(E.prediction.data(), E.samples[0].data(), E.samples[0].data() + n, cx(E.sample_times[0]),
                  E.samples[1].data(), E.samples[1].data() + n, cx(E.sample_times[1]), cx(0.0), n);
  }
  E.prev_prediction = E.prediction;
  cubic_hermite(E.prediction.data(), E.samples[1].data(), E.samples[1].data() + n, cx(E.sample_times[1]),
                E.samples[2].data(), E.samples[2].data() + n, cx(E.sample_times[2]), cx(0.0), n);
  double p = E.sample_times[2] / E.sample_times[1];
  double err = inf_dist(E.prediction.data(), E.prev_prediction.data(), n) / std::fabs((p * p) * (p * p) - 1);
  double norm_s = inf_norm_v(E.prediction.data(), n);
  if (norm_s > 1e-8) err /= norm_s;
  return err;
}

// :501-524
static void switch_to_singular(EndgameTracker& E) {
  Tracker& T = E.T;
  E.singular_endgame = true;
  double t = T.ss.t().re;
  E.singular_start = t;
  bool allone = true;
  for (double v : E.row_scaling) allone = allone && (v == 1.0);
  if (allone) {
    E.col_scaling = T.norm.w;
    skeel_row_scaling(E.row_scaling.data(), T.J.A.data(), E.n, E.col_scaling.data(), E.opt.scaling_threshold);
  }
  add_sample(E, t);
  E.singular_steps = 0;
  T.pred.winding_number = E.winding_number;
  E.at_inf_conds[0] = E.sample_conds[0];
  T.keep_extended_prec = true;
}
// :525-530
static void switch_to_regular(EndgameTracker& E) {
  E.singular_endgame = false;
  E.T.pred.winding_number = 1;
  tracker_init_t0(E.T, cx(0.0));
}

// :533-628
static int singular_endgame_step(EndgameTracker& E) {
  Tracker& T = E.T;
  double lambda = 0.25;
  double t = T.ss.t().re;
  tracker_init_t0(T, cx(lambda * t));
  bool max_steps = false;
  while (T.code == TC_tracking) {
    tracker_step(T);
    if ((E.steps_eg += 1) >= E.opt.max_endgame_steps) {
      E.code = EC_terminated_max_steps;
      max_steps = true;
      break;
    } else if (T.ext_steps() - E.ext_steps_eg_start > E.opt.max_endgame_extended_steps) {
      E.code = EC_terminated_max_extended_steps;
      max_steps = true;
      break;
    }
  }
  E.singular_steps += 1;
  if (!max_steps) {
    if (T.code != TC_success) {
      E.code = ec_from_tc(T.code);
      tracking_stopped(E);
      return E.code;
    }
    valuation_update(E.val, T.pred, lambda * t);
    int mh;
    double mh_err;
    estimate_winding_number(E.val, E.opt.max_winding_number, mh, mh_err);
    if (mh != E.winding_number || mh_err > 0.1) {
      switch_to_regular(E);
      return E.code;
    }
    add_sample(E, lambda * t);
    if (E.singular_steps < 2) return E.code;
    double acc = predict_endpoint(E);
    if (E.singular_steps == 2) {
      E.accuracy = acc;
      E.solution = E.prediction;
      return E.code;
    } else if (acc < E.accuracy && E.accuracy > 1e-12) {
      E.accuracy = acc;
      E.solution = E.prediction;
      return E.code;
    }
  }
  // @label prediction
  int m = E.winding_number;
  double kappa = E.sample_conds[2];
  double zero_cond = 1.0 / (m + 1);
  for (int i = 0; i < E.n; ++i) {
    // Bool * x is a strong zero in Julia: false * NaN == 0
    E.solution[i] = (E.val.val_x[i] < zero_cond) ? E.prediction[i] : cx(0.0);
  }
  double kappa0 = tracker_cond(T, E.solution.data(), cx(0.0), E.row_scaling.data(), E.col_scaling.data());
  double J0_norm = inf_norm_mat(T.J, E.row_scaling.data(), nullptr);
  if (E.accuracy < E.opt.singular_min_accuracy &&
      (((m > 1 && kappa > E.opt.min_cond && nanmax(kappa0, 1.0 / J0_norm) > kappa) || (m == 1 && kappa0 > 1e12)) ||
       max_steps || (E.n == 1 && 1.0 / J0_norm < E.opt.min_cond))) {
    E.cond = jmax(kappa0, 1.0 / J0_norm);
    E.singular = true;
    return (E.code = EC_success);
  } else if (!max_steps) {
    switch_to_regular(E);
    return E.code;
  }
  return E.code;
}

// :329-399
static int eg_step(EndgameTracker& E) {
  Tracker& T = E.T;
  if (E.steps_eg >= E.opt.max_endgame_steps) {
    return (E.code = EC_terminated_max_steps);
  } else if (T.ext_steps() - E.ext_steps_eg_start > E.opt.max_endgame_extended_steps) {
    bool allfin = true;
    for (auto& s : E.solution) allfin = allfin && !isnanC(s);
    if (allfin && E.winding_number != 0 && E.accuracy < E.opt.singular_min_accuracy) {
      E.cond = tracker_cond(T, E.solution.data(), cx(0.0), E.row_scaling.data(), E.col_scaling.data());
      E.singular = true;
      return (E.code = EC_success);
    }
    return (E.code = EC_terminated_max_extended_steps);
  }
  E.last_point = T.x;
  E.last_t = T.ss.t().re;
  if (E.singular_endgame) return singular_endgame_step(E);
  C tp = T.ss.tp();
  bool is_jump_to_zero = (tp.re == 0.0 && tp.im == 0.0);
  bool step_success = tracker_step(T);
  E.code = ec_from_tc(T.code);
  if (E.code != EC_tracking) {
    tracking_stopped(E);
    return E.code;
  }
  E.jtz_failed[0] = E.jtz_failed[1];
  E.jtz_failed[1] = is_jump_to_zero;
  double t = T.ss.t().re;
  if (!(t <= E.opt.endgame_start)) return E.code;
  if (E.steps_eg == 0) E.ext_steps_eg_start = T.ext_steps();
  E.steps_eg += 1;
  if (!step_success) return E.code;
  valuation_update(E.val, T.pred, t);
  if (check_finite(E)) {
    switch_to_singular(E);
    return E.code;
  } else if (check_at_infinity(E)) {
    return E.code;
  }
  return E.code;
}

}  // namespace hco

// =========================================================================================
// C interface for the test harness (ctypes)
// =========================================================================================
using namespace hco;

extern "C" {

// Option block shared with the harness; field meaning follows TrackerOptions /
// TrackerParameters / EndgameOptions (src/tracker.jl:45-140, src/endgame_tracker.jl:47-72).
struct hco_options {
  int32_t max_steps;
  int32_t extended_precision;
  double max_step_size, max_initial_step_size, min_step_size, min_rel_step_size, terminate_cond;
  double a, beta_a, beta_omega_p, beta_tau, strict_beta_tau;
  int32_t min_newton_iters;
  // endgame
  int32_t max_endgame_steps, max_endgame_extended_steps, max_winding_number;
  int32_t zero_is_at_infinity, at_infinity_check, only_nonsingular, refine_steps;
  double endgame_start, min_cond, min_cond_growth, min_coord_growth, singular_min_accuracy;
  double val_finite_tol, val_at_infinity_tol, sing_cond, sing_accuracy, scaling_threshold;
};

// Per-path record, mirrors PathResult (src/path_result.jl:76-98) / TrackerResult (src/tracker.jl:235-247)
struct hco_path_result {
  int32_t return_code;
  int32_t winding_number;  // 0 == nothing
  double t_re, t_im;
  double accuracy, residual, cond, omega, mu, tau;
  int32_t singular, extended_precision, extended_precision_used, _pad;
  int64_t accepted_steps, rejected_steps, steps_eg, path_number;
  double last_t;
};

void hco_default_options(hco_options* o) {
  TrackerOptions t;
  EndgameOptions e;
  o->max_steps = t.max_steps;
  o->extended_precision = t.extended_precision;
  o->max_step_size = t.max_step_size;
  o->max_initial_step_size = t.max_initial_step_size;
  o->min_step_size = t.min_step_size;
  o->min_rel_step_size = t.min_rel_step_size;
  o->terminate_cond = t.terminate_cond;
  o->a = t.p.a;
  o->beta_a = t.p.beta_a;
  o->beta_omega_p = t.p.beta_omega_p;
  o->beta_tau = t.p.beta_tau;
  o->strict_beta_tau = t.p.strict_beta_tau;
  o->min_newton_iters = t.p.min_newton_iters;
  o->max_endgame_steps = e.max_endgame_steps;
  o->max_endgame_extended_steps = e.max_endgame_extended_steps;
  o->max_winding_number = e.max_winding_number;
  o->zero_is_at_infinity = e.zero_is_at_infinity;
  o->at_infinity_check = e.at_infinity_check;
  o->only_nonsingular = e.only_nonsingular;
  o->refine_steps = e.refine_steps;
  o->endgame_start = e.endgame_start;
  o->min_cond = e.min_cond;
  o->min_cond_growth = e.min_cond_growth;
  o->min_coord_growth = e.min_coord_growth;
  o->singular_min_accuracy = e.singular_min_accuracy;
  o->val_finite_tol = e.val_finite_tol;
  o->val_at_infinity_tol = e.val_at_infinity_tol;
  o->sing_cond = e.sing_cond;
  o->sing_accuracy = e.sing_accuracy;
  o->scaling_threshold = e.scaling_threshold;
}

static void to_opts(const hco_options* o, TrackerOptions& t, EndgameOptions& e) {
  t.max_steps = o->max_steps;
  t.extended_precision = o->extended_precision != 0;
  t.max_step_size = o->max_step_size;
  t.max_initial_step_size = o->max_initial_step_size;
  t.min_step_size = o->min_step_size;
  t.min_rel_step_size = o->min_rel_step_size;
  t.terminate_cond = o->terminate_cond;
  t.p.a = o->a;
  t.p.beta_a = o->beta_a;
  t.p.beta_omega_p = o->beta_omega_p;
  t.p.beta_tau = o->beta_tau;
  t.p.strict_beta_tau = o->strict_beta_tau;
  t.p.min_newton_iters = o->min_newton_iters;
  e.max_endgame_steps = o->max_endgame_steps;
  e.max_endgame_extended_steps = o->max_endgame_extended_steps;
  e.max_winding_number = o->max_winding_number;
  e.zero_is_at_infinity = o->zero_is_at_infinity != 0;
  e.at_infinity_check = o->at_infinity_check != 0;
  e.only_nonsingular = o->only_nonsingular != 0;
  e.refine_steps = o->refine_steps;
  e.endgame_start = o->endgame_start;
  e.min_cond = o->min_cond;
  e.min_cond_growth = o->min_cond_growth;
  e.min_coord_growth = o->min_coord_growth;
  e.singular_min_accuracy = o->singular_min_accuracy;
  e.val_finite_tol = o->val_finite_tol;
  e.val_at_infinity_tol = o->val_at_infinity_tol;
  e.sing_cond = o->sing_cond;
  e.sing_accuracy = o->sing_accuracy;
  e.scaling_threshold = o->scaling_threshold;
}

// Track npaths start solutions.
//   mode 1: EndgameTracker from t1 to 0 → PathResult semantics (src/endgame_tracker.jl:902-914)
//   mode 0: Tracker from t1 to t0         → TrackerResult semantics (src/tracker.jl:1023-1026)
// Systems: terms (eq, exps n per term row-major, coef re/im). out_x: npaths×n complex;
// out_val (may be null): npaths×n valuation val_x; out_last (may be null): last_path_point.
int hco_track(int n, int nG, const int32_t* G_eq, const int32_t* G_exps, const double* G_coef, int nF,
              const int32_t* F_eq, const int32_t* F_exps, const double* F_coef, double gamma_re, double gamma_im,
              int64_t npaths, const double* starts, int mode, double t1_re, double t1_im, double t0_re,
              double t0_im, const hco_options* opts, int nthreads, hco_path_result* out, double* out_x,
              double* out_val, double* out_last) {
  Homotopy H;
  H.n = n;
  H.m = n;
  H.G = make_system(n, n, nG, G_eq, G_exps, G_coef);
  H.F = make_system(n, n, nF, F_eq, F_exps, F_coef);
  if (g_slp_on) {
    if (g_slp.n != n) return 1;
    H.F.slp = &g_slp;
    if (g_slp.np > 0) {
      H.param = true;
      H.pp = g_param_p;
      H.pq = g_param_q;
    }
  }
  H.gamma = C{gamma_re, gamma_im};
  TrackerOptions to;
  EndgameOptions eo;
  to_opts(opts, to, eo);
  if (nthreads <= 0) nthreads = (int)std::max(1u, std::thread::hardware_concurrency());
  if (npaths < nthreads) nthreads = (int)std::max<int64_t>(1, npaths);
  std::atomic<int64_t> next(0);
  auto worker = [&]() {
    EndgameTracker E;
    E.setup(H, to, eo);
    std::vector<C> x0(n), r(n);
    while (true) {
      int64_t k = next.fetch_add(1);
      if (k >= npaths) break;
      for (int i = 0; i < n; ++i) x0[i] = C{starts[(k * n + i) * 2], starts[(k * n + i) * 2 + 1]};
      hco_path_result& R = out[k];
      std::memset(&R, 0, sizeof(R));
      R.path_number = k + 1;
      tl_trace = k == g_trace_path ? &g_trace : nullptr;
      tl_trace_eg = &E.steps_eg;
      if (tl_trace) tl_trace->clear();
      if (mode == 1) {
        eg_init(E, x0.data(), t1_re);
        while (E.code == EC_tracking) eg_step(E);
        Tracker& T = E.T;
        const C* xs;
        double t;
        if (E.code == EC_success) {
          t = 0.0;
          xs = E.solution.data();
        } else {
          t = T.ss.t().re;
          xs = T.x.data();
        }
        H_eval(H, xs, cx(t), r.data());
        R.return_code = E.code;
        R.t_re = t;
        R.t_im = 0;
        R.residual = inf_norm_v(r.data(), n);
        R.accuracy = E.accuracy;
        R.cond = E.cond;
        R.singular = E.singular;
        R.winding_number = E.winding_number;
        R.omega = T.omega;
        R.mu = T.mu;
        R.tau = T.tau;
        R.extended_precision = T.extended_prec;
        R.extended_precision_used = T.used_extended_prec;
        R.accepted_steps = T.accepted_steps;
        R.rejected_steps = T.rejected_steps;
        R.steps_eg = E.steps_eg;
        R.last_t = E.last_t;
        for (int i = 0; i < n; ++i) {
          out_x[(k * n + i) * 2] = xs[i].re;
          out_x[(k * n + i) * 2 + 1] = xs[i].im;
          if (out_val) out_val[k * n + i] = E.val.val_x[i];
          if (out_last) {
            out_last[(k * n + i) * 2] = E.last_point[i].re;
            out_last[(k * n + i) * 2 + 1] = E.last_point[i].im;
          }
        }
      } else {
        Tracker& T = E.T;
        tracker_init(T, x0.data(), C{t1_re, t1_im}, C{t0_re, t0_im});
        while (T.code == TC_tracking) tracker_step(T);
        C t = T.ss.t();
        R.return_code = T.code;
        R.t_re = t.re;
        R.t_im = t.im;
        R.accuracy = T.accuracy;
        R.omega = T.omega;
        R.mu = T.mu;
        R.tau = T.tau;
        R.extended_precision = T.extended_prec || T.refined_extended_prec;
        R.extended_precision_used = T.used_extended_prec || T.refined_extended_prec;
        R.accepted_steps = T.accepted_steps;
        R.rejected_steps = T.rejected_steps;
        H_eval(H, T.x.data(), t, r.data());
        R.residual = inf_norm_v(r.data(), n);
        // valuation estimate at the end point (src/valuation.jl:82-124), used by the
        // valuation known-answer tests
        Valuation V;
        V.resize(n);
        V.init();
        if (T.code != TC_terminated_invalid_startvalue &&
            T.code != TC_terminated_invalid_startvalue_singular_jacobian)
          valuation_update(V, T.pred, t.re);
        for (int i = 0; i < n; ++i) {
          out_x[(k * n + i) * 2] = T.x[i].re;
          out_x[(k * n + i) * 2 + 1] = T.x[i].im;
          if (out_val) {
            out_val[k * n + i] = V.val_x[i];
          }
          if (out_last) {  // val_tẋ for the valuation tests
            out_last[(k * n + i) * 2] = V.val_tx[i];
            out_last[(k * n + i) * 2 + 1] = 0.0;
          }
        }
      }
    }
  };
  std::vector<std::thread> th;
  for (int i = 0; i < nthreads; ++i) th.emplace_back(worker);
  for (auto& t : th) t.join();
  return 0;
}

// Toric homotopy tracking of the polyhedral method (PolyhedralTracker's toric stage,
// src/polyhedral.jl:439-484): path k tracks starts[k] from t1[k] to t0[k] with the weights of
// row rows[k] (weights: nrows × nF, F's term order) and init!'s ω/μ keywords (NaN: init_newton).
int hco_track_toric(int n, int nF, const int32_t* F_eq, const int32_t* F_exps, const double* F_coef, int nrows,
                    const double* weights, int64_t npaths, const double* starts, const int32_t* rows,
                    const double* t1, const double* t0, const double* omega, const double* mu,
                    const hco_options* opts, int nthreads, hco_path_result* out, double* out_x) {
  Homotopy H0;
  H0.n = H0.m = n;
  H0.F = make_system(n, n, nF, F_eq, F_exps, F_coef);
  H0.G = make_system(n, n, 0, nullptr, nullptr, nullptr);
  H0.gamma = cx(1.0);
  H0.toric = true;
  H0.Ft = H0.F;
  (void)nrows;
  TrackerOptions to;
  EndgameOptions eo;
  to_opts(opts, to, eo);
  if (nthreads <= 0) nthreads = (int)std::max(1u, std::thread::hardware_concurrency());
  if (npaths < nthreads) nthreads = (int)std::max<int64_t>(1, npaths);
  std::atomic<int64_t> next(0);
  auto worker = [&]() {
    Homotopy H = H0;
    Tracker T;
    T.setup(H, to);
    std::vector<C> x0(n), r(n);
    while (true) {
      int64_t k = next.fetch_add(1);
      if (k >= npaths) break;
      for (int i = 0; i < n; ++i) x0[i] = C{starts[(k * n + i) * 2], starts[(k * n + i) * 2 + 1]};
      H.w.assign(weights + (size_t)rows[k] * nF, weights + (size_t)(rows[k] + 1) * nF);
      H.tc_t = NaN;
      tracker_init(T, x0.data(), cx(t1[k]), cx(t0[k]), omega ? omega[k] : NaN, mu ? mu[k] : NaN);
      while (T.code == TC_tracking) tracker_step(T);
      C t = T.ss.t();
      hco_path_result& R = out[k];
      std::memset(&R, 0, sizeof(R));
      R.path_number = k + 1;
      R.return_code = T.code;
      R.t_re = t.re;
      R.t_im = t.im;
      R.accuracy = T.accuracy;
      R.omega = T.omega;
      R.mu = T.mu;
      R.tau = T.tau;
      R.extended_precision = T.extended_prec || T.refined_extended_prec;
      R.extended_precision_used = T.used_extended_prec || T.refined_extended_prec;
      R.accepted_steps = T.accepted_steps;
      R.rejected_steps = T.rejected_steps;
      H_eval(H, T.x.data(), t, r.data());
      R.residual = inf_norm_v(r.data(), n);
      for (int i = 0; i < n; ++i) {
        out_x[(k * n + i) * 2] = T.x[i].re;
        out_x[(k * n + i) * 2 + 1] = T.x[i].im;
      }
    }
  };
  std::vector<std::thread> th;
  for (int i = 0; i < nthreads; ++i) th.emplace_back(worker);
  for (auto& t : th) t.join();
  return 0;
}

// --- unit-level entry points for the known-answer tests ---------------------------------

// LU + ldiv (src/linear_algebra.jl:389-408), A column-major n×n complex, b n complex
int hco_ldiv(int n, const double* A, const double* b, double* x) {
  MW W;
  W.resize(n);
  for (int i = 0; i < n * n; ++i) W.A[i] = C{A[2 * i], A[2 * i + 1]};
  updated(W);
  std::vector<C> bb(n), xx(n);
  for (int i = 0; i < n; ++i) bb[i] = C{b[2 * i], b[2 * i + 1]};
  ws_ldiv(W, xx.data(), bb.data());
  for (int i = 0; i < n; ++i) {
    x[2 * i] = xx[i].re;
    x[2 * i + 1] = xx[i].im;
  }
  return 0;
}
// inverse_inf_norm_est / cond with optional d_l, d_r (src/linear_algebra.jl:585-774)
int hco_inverse_inf_norm_est(int n, const double* A, const double* d_l, const double* d_r, double* est,
                             double* cond) {
  MW W;
  W.resize(n);
  for (int i = 0; i < n * n; ++i) W.A[i] = C{A[2 * i], A[2 * i + 1]};
  updated(W);
  *est = inverse_inf_norm_est(W, d_l, d_r);
  *cond = ws_cond(W, d_l, d_r);
  return 0;
}
// DD ops on pairs (src/DoubleDouble.jl): op 0 add, 1 sub, 2 mul
int hco_dd_op(int op, const double* a, const double* b, double* c) {
  DD x{a[0], a[1]}, y{b[0], b[1]}, z;
  if (op == 0)
    z = x + y;
  else if (op == 1)
    z = x - y;
  else
    z = x * y;
  c[0] = z.hi;
  c[1] = z.lo;
  return 0;
}
// weighted / unweighted ∞-norm (src/norm.jl:194-234); w may be null
double hco_norm(int n, const double* x, const double* w) {
  std::vector<C> v(n);
  for (int i = 0; i < n; ++i) v[i] = C{x[2 * i], x[2 * i + 1]};
  return wnorm(v.data(), w, n);
}
// evaluate the homotopy (plain, DD, Jacobian, taylor K) for the model-kit tests.
// kind 0: H(x,t); 1: DD H(x,t); 2: Jacobian (out n*n); 3..5: taylor K=1..3 with tx (K vectors)
int hco_homotopy_eval(int n, int nG, const int32_t* G_eq, const int32_t* G_exps, const double* G_coef, int nF,
                      const int32_t* F_eq, const int32_t* F_exps, const double* F_coef, double gamma_re,
                      double gamma_im, int kind, const double* x, double t_re, double t_im, double* out) {
  Homotopy H;
  H.n = H.m = n;
  H.G = make_system(n, n, nG, G_eq, G_exps, G_coef);
  H.F = make_system(n, n, nF, F_eq, F_exps, F_coef);
  if (g_slp_on) {
    if (g_slp.n != n) return 1;
    H.F.slp = &g_slp;
    if (g_slp.np > 0) {
      H.param = true;
      H.pp = g_param_p;
      H.pq = g_param_q;
    }
  }
  H.gamma = C{gamma_re, gamma_im};
  C t{t_re, t_im};
  int nx = (kind >= 4) ? kind - 2 : 1;
  std::vector<C> xv((size_t)nx * n), u(n), U((size_t)n * n);
  for (size_t i = 0; i < xv.size(); ++i) xv[i] = C{x[2 * i], x[2 * i + 1]};
  if (kind == 0) {
    H_eval(H, xv.data(), t, u.data());
  } else if (kind == 1) {
    std::vector<CDD> xd(n);
    for (int i = 0; i < n; ++i) xd[i] = cdd(xv[i]);
    H_eval_dd(H, xd.data(), t, u.data());
  } else if (kind == 2) {
    H_eval_jac(H, xv.data(), t, u.data(), U.data());
    for (int i = 0; i < n * n; ++i) {
      out[2 * i] = U[i].re;
      out[2 * i + 1] = U[i].im;
    }
    return 0;
  } else if (kind == 3) {
    H_taylor1(H, xv.data(), t, u.data());
  } else {
    H_taylorK(H, kind - 2, xv.data(), t, u.data());
  }
  for (int i = 0; i < n; ++i) {
    out[2 * i] = u[i].re;
    out[2 * i + 1] = u[i].im;
  }
  return 0;
}

// F as a straight-line program for the following hco_track calls (instr: 6 ints per
// instruction — input[0..3], op, output; consts re/im; tape layout as in include/hcgpu.h's
// hc_slp); ninstr < 0 switches back to term tables.
void hco_set_slp(int n, int ninstr, const int32_t* instr, int nconst, const double* consts, int voff, int tape,
                 const int32_t* outputs) {
  if (ninstr < 0) {
    g_slp_on = false;
    return;
  }
  g_slp = Slp();
  g_slp.n = n;
  g_slp.voff = voff;
  g_slp.tape = tape;
  g_slp.nconst = nconst;
  g_slp.ins.assign(instr, instr + 6 * (size_t)ninstr);
  for (int k = 0; k < nconst; ++k) g_slp.consts.push_back(C{consts[2 * k], consts[2 * k + 1]});
  g_slp.outputs.assign(outputs, outputs + n);
  g_slp_on = true;
}

// The program of hco_set_slp as F(x; p) with np parameters at tape slots [poff, poff + np),
// tracked as the parameter homotopy F(x; t p + (1 - t) q); p, q: np complex values each.
void hco_set_slp_parameters(int np, int poff, const double* p, const double* q) {
  g_slp.np = np;
  g_slp.poff = poff;
  g_param_p.assign(np, cx(0.0));
  g_param_q.assign(np, cx(0.0));
  for (int k = 0; k < np; ++k) {
    g_param_p[k] = C{p[2 * k], p[2 * k + 1]};
    g_param_q[k] = C{q[2 * k], q[2 * k + 1]};
  }
}

// Step trace of one path of the next hco_track call (path: 0-based index, -1 = off); the
// records (HCO_TRACE_FIELDS doubles each) are read with hco_get_trace.
void hco_set_trace(int64_t path) { g_trace_path = path; }
int64_t hco_get_trace(double* out, int64_t max_records) {
  int64_t nrec = (int64_t)(g_trace.size() / HCO_TRACE_FIELDS);
  int64_t m = std::min(nrec, max_records);
  if (out && m > 0) std::memcpy(out, g_trace.data(), (size_t)m * HCO_TRACE_FIELDS * sizeof(double));
  return nrec;
}

}  // extern "C"
