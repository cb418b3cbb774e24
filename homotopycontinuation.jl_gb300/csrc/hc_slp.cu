// hc_slp.cu — straight-line programs (ModelKit's InstructionSequence) turned into CUDA C and
// compiled with NVRTC for the device at hand, together with the tracking kernel.
//
// The reference compiles a system's instruction sequence into Julia functions
// (src/model_kit/compiled_system_homotopy.jl:178-243) and caches compiled systems by hash
// (:39-57). Here the program is first lowered (3- and 4-ary ops split into binary ones, every
// op with only constant inputs folded on the host, instructions that feed no output dropped)
// and then written out four ways, each a straight-line function whose tape values are local
// variables (registers):
//   eval_v<T>   F(x) in arithmetic T (complex FP64, or double-double for the extended-precision
//               residual); every lane of the warp runs the whole program, lane i keeps F_i;
//   eval_vt<T>  F(x) and, in lane j, the derivatives along e_j — forward-mode differentiation,
//               so lane j ends with column j of the Jacobian (complex FP64, or FP32 for the
//               mixed-precision tracker's Jacobian);
//   seriesK     the truncated Taylor series of F along x(s) = Σ_{k<K} tx_k s^k, orders K-1
//               and K, for K = 1, 2, 3 (the taylor! of the predictor, src/model_kit/taylor.jl),
//               with the series rules of ModelKit's ops (products by convolution, inverse,
//               quotient and square root by their recurrences).
// Every lane computing the same values costs nothing extra on the FP64 pipe (a warp-wide FP64
// instruction occupies it for the same time however many lanes are active), and keeps the
// evaluator free of shared-memory tables.
#include <nvrtc.h>
#include <sys/stat.h>
#include <unistd.h>

#include <chrono>
#include <complex>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <map>
#include <mutex>
#include <sstream>

#include "hc_slp.h"
#include "hc_jit_headers.inc"  // generated by the build: kJitHeaderNames / kJitHeaderSources

namespace hcd {
namespace {

using cplx = std::complex<double>;

int op_arity(int op) {
  switch (op) {
    case HC_OP_STOP:
      return 0;
    case HC_OP_CB: case HC_OP_ACOS: case HC_OP_ASIN: case HC_OP_COS: case HC_OP_COSH: case HC_OP_EXP:
    case HC_OP_INV: case HC_OP_INV_NOT_ZERO: case HC_OP_INVSQR: case HC_OP_NEG: case HC_OP_SIN:
    case HC_OP_SINH: case HC_OP_SQR: case HC_OP_SQRT: case HC_OP_TAN: case HC_OP_TANH: case HC_OP_IDENTITY:
      return 1;
    case HC_OP_ADD: case HC_OP_DIV: case HC_OP_MUL: case HC_OP_SUB: case HC_OP_POW_INT: case HC_OP_POW:
      return 2;
    case HC_OP_ADD3: case HC_OP_MUL3: case HC_OP_MULADD: case HC_OP_MULSUB: case HC_OP_SUBMUL:
      return 3;
    case HC_OP_ADD4: case HC_OP_MUL4: case HC_OP_MULMULADD: case HC_OP_MULMULSUB:
      return 4;
    default:
      return -1;
  }
}
bool op_supported(int op) {
  switch (op) {
    case HC_OP_ACOS: case HC_OP_ASIN: case HC_OP_COS: case HC_OP_COSH: case HC_OP_EXP: case HC_OP_SIN:
    case HC_OP_SINH: case HC_OP_TAN: case HC_OP_TANH: case HC_OP_POW:
      return false;
    default:
      return op_arity(op) >= 0;
  }
}

// ---- lowered program
enum LOp { L_ADD, L_SUB, L_MUL, L_DIV, L_NEG, L_SQR, L_INV, L_INVNZ, L_SQRT, L_POWI };
struct Ref {
  int kind = -1;  // 0 constant, 1 variable idx, 2 temporary idx, 3 parameter idx
  int idx = 0;
  cplx c;
};
struct LIns {
  int op;
  Ref a, b;
  int p;  // exponent of L_POWI
};

// host arithmetic of constant folding, with the evaluators' formulas
cplx h_div(cplx a, cplx b) {
  double d = b.real() * b.real() + b.imag() * b.imag();
  return cplx((a.real() * b.real() + a.imag() * b.imag()) / d, (a.imag() * b.real() - a.real() * b.imag()) / d);
}
cplx h_pow(cplx a, int p) {
  bool neg = p < 0;
  unsigned q = neg ? (unsigned)(-p) : (unsigned)p;
  cplx r(1.0, 0.0), b = a;
  bool first = true;
  while (q) {
    if (q & 1u) {
      r = first ? b : r * b;
      first = false;
    }
    q >>= 1;
    if (q) b = b * b;
  }
  return neg ? h_div(cplx(1.0, 0.0), r) : r;
}

struct Lowered {
  int n = 0, np = 0;
  std::vector<LIns> ins;    // temporaries 0..ins.size()-1
  std::vector<Ref> out;     // per equation
  std::vector<char> live;   // per temporary: reaches an output
  std::vector<char> usedvar, usedpar;
};

struct Lowerer {
  Lowered L;
  Ref cst(cplx c) {
    Ref r;
    r.kind = 0;
    r.c = c;
    return r;
  }
  Ref emit(int op, Ref a, Ref b = Ref(), int p = 0) {
    L.ins.push_back(LIns{op, a, b, p});
    Ref r;
    r.kind = 2;
    r.idx = (int)L.ins.size() - 1;
    return r;
  }
  Ref bin(int op, Ref a, Ref b) {
    if (a.kind == 0 && b.kind == 0) {
      switch (op) {
        case L_ADD: return cst(a.c + b.c);
        case L_SUB: return cst(a.c - b.c);
        case L_MUL: return cst(a.c * b.c);
        case L_DIV: return cst(h_div(a.c, b.c));
      }
    }
    return emit(op, a, b);
  }
  Ref un(int op, Ref a, int p = 0) {
    if (a.kind == 0) {
      switch (op) {
        case L_NEG: return cst(-a.c);
        case L_SQR: return cst(a.c * a.c);
        case L_INV: return cst(h_div(cplx(1.0, 0.0), a.c));
        case L_INVNZ: return cst(a.c == cplx(0.0, 0.0) ? a.c : h_div(cplx(1.0, 0.0), a.c));
        case L_SQRT: return cst(std::sqrt(a.c));
        case L_POWI: return cst(h_pow(a.c, p));
      }
    }
    return emit(op, a, Ref(), p);
  }
  // ModelKit op (operations.jl:183-248) on lowered operands
  Ref op(int o, const Ref* v, int p) {
    switch (o) {
      case HC_OP_CB: return bin(L_MUL, un(L_SQR, v[0]), v[0]);
      case HC_OP_INV: return un(L_INV, v[0]);
      case HC_OP_INV_NOT_ZERO: return un(L_INVNZ, v[0]);
      case HC_OP_INVSQR: return un(L_SQR, un(L_INV, v[0]));
      case HC_OP_NEG: return un(L_NEG, v[0]);
      case HC_OP_SQR: return un(L_SQR, v[0]);
      case HC_OP_SQRT: return un(L_SQRT, v[0]);
      case HC_OP_IDENTITY: return v[0];
      case HC_OP_ADD: return bin(L_ADD, v[0], v[1]);
      case HC_OP_DIV: return bin(L_DIV, v[0], v[1]);
      case HC_OP_MUL: return bin(L_MUL, v[0], v[1]);
      case HC_OP_SUB: return bin(L_SUB, v[0], v[1]);
      case HC_OP_POW_INT:
        if (p == 0) return cst(cplx(1.0, 0.0));
        if (p == 1) return v[0];
        return un(L_POWI, v[0], p);
      case HC_OP_ADD3: return bin(L_ADD, bin(L_ADD, v[0], v[1]), v[2]);
      case HC_OP_MUL3: return bin(L_MUL, bin(L_MUL, v[0], v[1]), v[2]);
      case HC_OP_MULADD: return bin(L_ADD, bin(L_MUL, v[0], v[1]), v[2]);
      case HC_OP_MULSUB: return bin(L_SUB, bin(L_MUL, v[0], v[1]), v[2]);
      case HC_OP_SUBMUL: return bin(L_SUB, v[2], bin(L_MUL, v[0], v[1]));
      case HC_OP_ADD4: return bin(L_ADD, bin(L_ADD, bin(L_ADD, v[0], v[1]), v[2]), v[3]);
      case HC_OP_MUL4: return bin(L_MUL, bin(L_MUL, bin(L_MUL, v[0], v[1]), v[2]), v[3]);
      case HC_OP_MULMULADD: return bin(L_ADD, bin(L_MUL, v[0], v[1]), bin(L_MUL, v[2], v[3]));
      case HC_OP_MULMULSUB: return bin(L_SUB, bin(L_MUL, v[0], v[1]), bin(L_MUL, v[2], v[3]));
    }
    return Ref();
  }
};

Lowered lower(const SlpProgram& P) {
  Lowerer W;
  W.L.n = P.n;
  W.L.np = P.np;
  std::vector<Ref> slot(P.tape);
  for (int k = 0; k < P.nconst; ++k) slot[k] = W.cst(cplx(P.consts[2 * k], P.consts[2 * k + 1]));
  for (int j = 0; j < P.n; ++j) {
    slot[P.voff + j].kind = 1;
    slot[P.voff + j].idx = j;
  }
  for (int k = 0; k < P.np; ++k) {
    slot[P.poff + k].kind = 3;
    slot[P.poff + k].idx = k;
  }
  for (const hc_instruction& I : P.instr) {
    if (I.op == HC_OP_STOP) break;
    int a = op_arity(I.op);
    Ref v[4];
    for (int q = 0; q < a; ++q)
      if (!(I.op == HC_OP_POW_INT && q == 1)) v[q] = slot[I.input[q]];
    slot[I.output] = W.op(I.op, v, I.op == HC_OP_POW_INT ? I.input[1] : 0);
  }
  for (int i = 0; i < P.n; ++i) W.L.out.push_back(slot[P.outputs[i]]);
  // temporaries that reach an output
  Lowered& L = W.L;
  L.live.assign(L.ins.size(), 0);
  L.usedvar.assign(P.n, 0);
  L.usedpar.assign(P.np, 0);
  auto mark = [&](const Ref& r) {
    if (r.kind == 2) L.live[r.idx] = 1;
    if (r.kind == 1) L.usedvar[r.idx] = 1;
    if (r.kind == 3) L.usedpar[r.idx] = 1;
  };
  for (const Ref& r : L.out) mark(r);
  for (int k = (int)L.ins.size() - 1; k >= 0; --k)
    if (L.live[k]) {
      mark(L.ins[k].a);
      mark(L.ins[k].b);
    }
  return W.L;
}

// ---- emission
std::string num(double v) {
  char b[40];
  snprintf(b, sizeof b, "%.17g", v);
  std::string s(b);
  if (s.find_first_of(".eEn") == std::string::npos) s += ".0";  // a double literal, not an int
  if (s == "inf") return "__longlong_as_double(0x7ff0000000000000LL)";
  if (s == "-inf") return "__longlong_as_double(0xfff0000000000000LL)";
  if (s == "nan" || s == "-nan") return "__longlong_as_double(0x7ff8000000000000LL)";
  return s;
}
std::string kc(const char* T, cplx c) { return std::string("kc<") + T + ">(" + num(c.real()) + ", " + num(c.imag()) + ")"; }

// values (and tangents) in a template over T
std::string emit_eval(const Lowered& L, bool tangent) {
  std::ostringstream o;
  const int n = L.n;
  auto val = [&](const Ref& r) -> std::string {
    if (r.kind == 0) return kc("T", r.c);
    if (r.kind == 1) return "x" + std::to_string(r.idx);
    if (r.kind == 3) return "p" + std::to_string(r.idx);
    return "t" + std::to_string(r.idx);
  };
  std::vector<char> hasd(L.ins.size(), 0);
  auto hast = [&](const Ref& r) { return r.kind == 1 || (r.kind == 2 && hasd[r.idx]); };
  auto der = [&](const Ref& r) -> std::string {
    if (r.kind == 1) return "dx" + std::to_string(r.idx);
    return "u" + std::to_string(r.idx);
  };
  // pq: the parameter homotopy's p (entries 0..np-1) and q (np..2np-1); t: where it is
  // evaluated (both unused without parameters)
  o << "template <class T>\n__device__ __forceinline__ void " << (tangent ? "eval_vt" : "eval_v")
    << "(const c64* __restrict__ xv, const c64* __restrict__ pq, c64 t, int lane, T& Fi"
    << (tangent ? ", T* col" : "") << ") {\n";
  for (int j = 0; j < n; ++j)
    if (L.usedvar[j]) {
      o << "  const T x" << j << " = var<T>(xv[" << j << "]);\n";
      if (tangent) o << "  const T dx" << j << " = unit<T>(lane == " << j << ");\n";
    }
  for (int k = 0; k < L.np; ++k)
    if (L.usedpar[k])
      o << "  const T p" << k << " = var<T>(param_at(pq[" << k << "], pq[" << L.np + k << "], t));\n";
  for (size_t k = 0; k < L.ins.size(); ++k) {
    if (!L.live[k]) continue;
    const LIns& I = L.ins[k];
    std::string a = val(I.a), b = I.b.kind >= 0 ? val(I.b) : "", t = "t" + std::to_string(k);
    std::string e;
    switch (I.op) {
      case L_ADD: e = a + " + " + b; break;
      case L_SUB: e = a + " - " + b; break;
      case L_MUL: e = a + " * " + b; break;
      case L_DIV: e = "sdiv(" + a + ", " + b + ")"; break;
      case L_NEG: e = "-" + a; break;
      case L_SQR: e = a + " * " + a; break;
      case L_INV: e = "sinv(" + a + ")"; break;
      case L_INVNZ: e = "is_zero(" + a + ") ? " + a + " : sinv(" + a + ")"; break;
      case L_SQRT: e = "ssqrt(" + a + ")"; break;
      case L_POWI: e = "spow(" + a + ", " + std::to_string(I.p) + ")"; break;
    }
    o << "  const T " << t << " = " << e << ";\n";
    if (!tangent) continue;
    bool ha = hast(I.a), hb = I.b.kind >= 0 && hast(I.b);
    if (!ha && !hb) continue;
    hasd[k] = 1;
    std::string da = ha ? der(I.a) : "", db = hb ? der(I.b) : "", d;
    switch (I.op) {
      case L_ADD: d = ha && hb ? da + " + " + db : (ha ? da : db); break;
      case L_SUB: d = ha && hb ? da + " - " + db : (ha ? da : "-" + db); break;
      case L_MUL:
        d = ha && hb ? da + " * " + b + " + " + a + " * " + db : (ha ? da + " * " + b : a + " * " + db);
        break;
      case L_DIV:
        d = ha && hb ? "sdiv(" + da + " - " + t + " * " + db + ", " + b + ")"
                     : (ha ? "sdiv(" + da + ", " + b + ")" : "-sdiv(" + t + " * " + db + ", " + b + ")");
        break;
      case L_NEG: d = "-" + da; break;
      case L_SQR: d = "smul(" + a + " * " + da + ", 2)"; break;
      case L_INV: d = "-(" + t + " * " + t + " * " + da + ")"; break;
      case L_INVNZ: d = "is_zero(" + a + ") ? " + da + " : -(" + t + " * " + t + " * " + da + ")"; break;
      case L_SQRT: d = "sdiv(" + da + ", smul(" + t + ", 2))"; break;
      case L_POWI: d = "smul(spow(" + a + ", " + std::to_string(I.p - 1) + "), " + std::to_string(I.p) + ") * " + da; break;
    }
    o << "  const T u" << k << " = " << d << ";\n";
  }
  o << "  Fi = kc<T>(0.0, 0.0);\n";
  for (int i = 0; i < n; ++i) o << "  if (lane == " << i << ") Fi = " << val(L.out[i]) << ";\n";
  if (tangent)
    for (int i = 0; i < n; ++i)
      o << "  col[" << i << "] = " << (hast(L.out[i]) ? der(L.out[i]) : std::string("kc<T>(0.0, 0.0)")) << ";\n";
  o << "}\n";
  return o.str();
}

// Taylor series of order K (FP64): orders K-1 and K of F (order 0 twice for K = 1)
std::string emit_series(const Lowered& L, int K) {
  std::ostringstream o;
  const int n = L.n;
  int hidden = 0;
  // a series value: name prefix and its highest order that is not structurally zero
  struct S {
    int kind;  // 0 constant, 1 named series
    cplx c;
    std::string name;
    int mz;
  };
  std::vector<S> tmp(L.ins.size());
  auto ser = [&](const Ref& r) -> S {
    if (r.kind == 0) return S{0, r.c, "", 0};
    if (r.kind == 1) return S{1, cplx(), "x" + std::to_string(r.idx), K - 1};
    if (r.kind == 3) return S{1, cplx(), "p" + std::to_string(r.idx), 1};  // p(t + s) = p(t) + s (p - q)
    return tmp[r.idx];
  };
  auto at = [&](const S& s, int q) -> std::string {  // order q or "" when zero
    if (s.kind == 0) return q == 0 ? kc("c64", s.c) : "";
    return q <= s.mz ? s.name + "_" + std::to_string(q) : "";
  };
  auto decl = [&](const std::string& name, int q, const std::string& e) {
    o << "  const c64 " << name << "_" << q << " = " << (e.empty() ? "kc<c64>(0.0, 0.0)" : e) << ";\n";
  };
  auto sum = [](const std::vector<std::string>& terms) {
    std::string e;
    for (const std::string& t : terms) e += (e.empty() ? "" : " + ") + t;
    return e;
  };
  auto mul = [&](const S& a, const S& b, const std::string& name) -> S {
    S r{1, cplx(), name, std::min(K, a.mz + b.mz)};
    for (int q = 0; q <= r.mz; ++q) {
      std::vector<std::string> terms;
      for (int j = 0; j <= q; ++j) {
        std::string x = at(a, j), y = at(b, q - j);
        if (!x.empty() && !y.empty()) terms.push_back(x + " * " + y);
      }
      decl(name, q, sum(terms));
    }
    return r;
  };
  auto fresh = [&]() { return "h" + std::to_string(hidden++); };
  o << "__device__ __forceinline__ void series" << K
    << "(const c64* __restrict__ tx0, const c64* __restrict__ tx1, const c64* __restrict__ tx2, "
       "const c64* __restrict__ pq, c64 t, int lane, c64& Flo, c64& Fhi) {\n";
  for (int j = 0; j < n; ++j)
    if (L.usedvar[j])
      for (int q = 0; q < K; ++q) o << "  const c64 x" << j << "_" << q << " = tx" << q << "[" << j << "];\n";
  for (int k = 0; k < L.np; ++k)
    if (L.usedpar[k]) {
      o << "  const c64 p" << k << "_0 = param_at(pq[" << k << "], pq[" << L.np + k << "], t);\n";
      o << "  const c64 p" << k << "_1 = pq[" << k << "] - pq[" << L.np + k << "];\n";
    }
  for (size_t k = 0; k < L.ins.size(); ++k) {
    if (!L.live[k]) continue;
    const LIns& I = L.ins[k];
    S a = ser(I.a), b = I.b.kind >= 0 ? ser(I.b) : S{0, cplx(), "", 0};
    std::string name = "s" + std::to_string(k);
    S r{1, cplx(), name, 0};
    switch (I.op) {
      case L_ADD:
      case L_SUB: {
        r.mz = std::max(a.mz, b.mz);
        for (int q = 0; q <= r.mz; ++q) {
          std::string x = at(a, q), y = at(b, q), e;
          if (!x.empty() && !y.empty())
            e = x + (I.op == L_ADD ? " + " : " - ") + y;
          else if (!x.empty())
            e = x;
          else if (!y.empty())
            e = I.op == L_ADD ? y : "-" + y;
          decl(name, q, e);
        }
        break;
      }
      case L_NEG:
        r.mz = a.mz;
        for (int q = 0; q <= r.mz; ++q) decl(name, q, at(a, q).empty() ? "" : "-" + at(a, q));
        break;
      case L_MUL: r = mul(a, b, name); break;
      case L_SQR: r = mul(a, a, name); break;
      case L_POWI: {
        int p = I.p < 0 ? -I.p : I.p;
        S acc{0, cplx(1.0, 0.0), "", 0}, base = a;
        bool first = true;
        while (p) {
          if (p & 1) {
            acc = first ? base : mul(acc, base, fresh());
            first = false;
          }
          p >>= 1;
          if (p) base = mul(base, base, fresh());
        }
        if (I.p > 0) {
          r = acc;  // alias the last product
          if (r.kind == 1 && r.name != name) {
            for (int q = 0; q <= r.mz; ++q) decl(name, q, at(r, q));
            r.name = name;
          }
          break;
        }
        a = acc;  // x^p = 1 / x^|p|: the inverse below
      }
        // fall through
      case L_INV: {
        // c_0 = 1/a_0, c_q = -(Σ_{j=1..q} a_j c_{q-j}) c_0
        r.mz = a.mz >= 1 ? K : 0;
        decl(name, 0, "sinv(" + at(a, 0) + ")");
        for (int q = 1; q <= r.mz; ++q) {
          std::vector<std::string> terms;
          for (int j = 1; j <= q; ++j)
            if (!at(a, j).empty()) terms.push_back(at(a, j) + " * " + name + "_" + std::to_string(q - j));
          decl(name, q, terms.empty() ? "" : "-(" + sum(terms) + ") * " + name + "_0");
        }
        break;
      }
      case L_INVNZ: {
        // a_0 == 0: the series of a itself (op_inv_not_zero), else its inverse
        std::string z = name + "_z";
        o << "  const bool " << z << " = is_zero(" << at(a, 0) << ");\n";
        std::string iv = name + "_i";
        r.mz = a.mz >= 1 ? K : 0;
        decl(iv, 0, "sinv(" + at(a, 0) + ")");
        for (int q = 1; q <= r.mz; ++q) {
          std::vector<std::string> terms;
          for (int j = 1; j <= q; ++j)
            if (!at(a, j).empty()) terms.push_back(at(a, j) + " * " + iv + "_" + std::to_string(q - j));
          decl(iv, q, terms.empty() ? "" : "-(" + sum(terms) + ") * " + iv + "_0");
        }
        for (int q = 0; q <= r.mz; ++q) {
          std::string x = at(a, q);
          decl(name, q, z + " ? " + (x.empty() ? std::string("kc<c64>(0.0, 0.0)") : x) + " : " + iv + "_" + std::to_string(q));
        }
        break;
      }
      case L_DIV: {
        if (b.kind == 0) {  // by a constant
          r.mz = a.mz;
          decl(name, 0, "sdiv(" + at(a, 0) + ", " + kc("c64", b.c) + ")");
          for (int q = 1; q <= r.mz; ++q)
            decl(name, q, at(a, q).empty() ? "" : "sdiv(" + at(a, q) + ", " + kc("c64", b.c) + ")");
          break;
        }
        // c_0 = a_0/b_0, c_q = (a_q - Σ_{j=1..q} b_j c_{q-j}) / b_0
        r.mz = K;
        std::string ib = name + "_ib";
        o << "  const c64 " << ib << " = sinv(" << at(b, 0) << ");\n";
        decl(name, 0, "sdiv(" + (at(a, 0).empty() ? std::string("kc<c64>(0.0, 0.0)") : at(a, 0)) + ", " + at(b, 0) + ")");
        for (int q = 1; q <= K; ++q) {
          std::vector<std::string> terms;
          for (int j = 1; j <= q; ++j)
            if (!at(b, j).empty()) terms.push_back(at(b, j) + " * " + name + "_" + std::to_string(q - j));
          std::string x = at(a, q);
          std::string e = (x.empty() ? std::string("kc<c64>(0.0, 0.0)") : x) + (terms.empty() ? "" : " - (" + sum(terms) + ")");
          decl(name, q, "(" + e + ") * " + ib);
        }
        break;
      }
      case L_SQRT: {
        // c_0 = √a_0, c_q = (a_q - Σ_{j=1..q-1} c_j c_{q-j}) / (2 c_0)
        r.mz = a.mz >= 1 ? K : 0;
        decl(name, 0, "ssqrt(" + at(a, 0) + ")");
        std::string i2 = name + "_i2";
        if (r.mz >= 1) o << "  const c64 " << i2 << " = sinv(smul(" << name << "_0, 2));\n";
        for (int q = 1; q <= r.mz; ++q) {
          std::vector<std::string> terms;
          for (int j = 1; j <= q - 1; ++j) terms.push_back(name + "_" + std::to_string(j) + " * " + name + "_" + std::to_string(q - j));
          std::string x = at(a, q);
          std::string e = (x.empty() ? std::string("kc<c64>(0.0, 0.0)") : x) + (terms.empty() ? "" : " - (" + sum(terms) + ")");
          decl(name, q, "(" + e + ") * " + i2);
        }
        break;
      }
    }
    tmp[k] = r;
  }
  // straight-line homotopy: orders K-1 and K of F (order 0 twice for K = 1: the t-derivative
  // is γG - F); parameter homotopy: orders K-1 and K of F(x(s); p(t + s)), whose order K is
  // the homotopy's
  const int lo = (K == 1 && L.np == 0) ? 0 : K - 1, hi = (K == 1 && L.np == 0) ? 0 : K;
  o << "  Flo = Fhi = kc<c64>(0.0, 0.0);\n";
  for (int i = 0; i < n; ++i) {
    S s = ser(L.out[i]);
    std::string x = at(s, lo), y = at(s, hi);
    o << "  if (lane == " << i << ") { Flo = " << (x.empty() ? std::string("kc<c64>(0.0, 0.0)") : x)
      << "; Fhi = " << (y.empty() ? std::string("kc<c64>(0.0, 0.0)") : y) << "; }\n";
  }
  o << "}\n";
  return o.str();
}

}  // namespace

int slp_validate(const hc_slp* F, const int32_t* degrees, const double* scaling, int nparams, int poff,
                 SlpProgram& P, std::string& err) {
  if (!F || (nparams == 0 && (!degrees || !scaling))) {
    err = "null argument";
    return HC_ERR_INVALID_ARG;
  }
  if (nparams < 0 || nparams > 1024) {
    err = "need 0 <= nparameters <= 1024";
    return HC_ERR_INVALID_ARG;
  }
  const int n = F->n;
  if (n < 1 || n > 32) {
    err = "need 1 <= n <= 32";
    return HC_ERR_UNSUPPORTED;
  }
  if (F->ninstructions < 0 || F->nconstants < 0 || F->tape_size < 0 || (F->ninstructions > 0 && !F->instructions) ||
      (F->nconstants > 0 && !F->constants) || !F->outputs) {
    err = "bad program arrays";
    return HC_ERR_INVALID_ARG;
  }
  if (F->ninstructions > 200000) {
    err = "program longer than 200,000 instructions";
    return HC_ERR_TOO_LARGE;
  }
  const int tape = F->tape_size, voff = F->variables_offset, nc = F->nconstants;
  if (nc > tape || voff < nc || voff + n > tape) {
    err = "constants must occupy slots [0, nconstants) and variables [variables_offset, +n) within the tape";
    return HC_ERR_INVALID_ARG;
  }
  for (int k = 0; k < 2 * nc; ++k)
    if (!std::isfinite(F->constants[k])) {
      err = "constants must be finite";
      return HC_ERR_INVALID_ARG;
    }
  if (nparams > 0 && (poff < nc || poff + nparams > tape || (poff < voff + n && poff + nparams > voff))) {
    err = "parameters must occupy slots [parameters_offset, +nparameters) within the tape, apart from the "
          "constants and variables";
    return HC_ERR_INVALID_ARG;
  }
  std::vector<char> written(tape, 0), fixed(tape, 0);
  for (int k = 0; k < nc; ++k) written[k] = fixed[k] = 1;
  for (int j = 0; j < n; ++j) written[voff + j] = fixed[voff + j] = 1;
  for (int k = 0; k < nparams; ++k) written[poff + k] = fixed[poff + k] = 1;
  P.instr.clear();
  for (int k = 0; k < F->ninstructions; ++k) {
    const hc_instruction& I = F->instructions[k];
    if (I.op == HC_OP_STOP) break;
    int a = op_arity(I.op);
    if (a < 0) {
      err = "instruction " + std::to_string(k) + ": unknown op " + std::to_string(I.op);
      return HC_ERR_INVALID_ARG;
    }
    if (!op_supported(I.op)) {
      err = "instruction " + std::to_string(k) + ": op " + std::to_string(I.op) +
            " (transcendental or real power) is not supported by the GPU evaluator";
      return HC_ERR_UNSUPPORTED;
    }
    for (int q = 0; q < a; ++q) {
      if (I.op == HC_OP_POW_INT && q == 1) {
        if (I.input[1] < -64 || I.input[1] > 64) {
          err = "instruction " + std::to_string(k) + ": POW_INT exponent outside [-64, 64]";
          return HC_ERR_UNSUPPORTED;
        }
        continue;
      }
      int s = I.input[q];
      if (s < 0 || s >= tape || !written[s]) {
        err = "instruction " + std::to_string(k) + ": input slot " + std::to_string(s) + " is not written before it is read";
        return HC_ERR_INVALID_ARG;
      }
    }
    // slots are written in order and may be written again (ModelKit compacts its tapes,
    // src/model_kit/instruction_sequence.jl:354-381); constants, variables and parameters stay
    // fixed
    if (I.output < 0 || I.output >= tape || fixed[I.output]) {
      err = "instruction " + std::to_string(k) + ": output slot " + std::to_string(I.output) +
            " is out of range or a constant, variable or parameter";
      return HC_ERR_INVALID_ARG;
    }
    written[I.output] = 1;
    P.instr.push_back(I);
  }
  for (int i = 0; i < n; ++i) {
    int s = F->outputs[i];
    if (s < 0 || s >= tape || !written[s]) {
      err = "output " + std::to_string(i) + ": slot " + std::to_string(s) + " is never written";
      return HC_ERR_INVALID_ARG;
    }
  }
  if (nparams == 0)
    for (int i = 0; i < n; ++i)
      if (degrees[i] < 1 || degrees[i] > 64 || !std::isfinite(scaling[i])) {
        err = "start system: degrees must lie in [1, 64] and scalings be finite";
        return HC_ERR_INVALID_ARG;
      }
  P.n = n;
  P.nconst = nc;
  P.voff = voff;
  P.tape = tape;
  P.np = nparams;
  P.poff = nparams > 0 ? poff : 0;
  P.consts.assign(F->constants, F->constants + 2 * nc);
  P.outputs.assign(F->outputs, F->outputs + n);
  if (nparams == 0) {
    P.degrees.assign(degrees, degrees + n);
    P.scaling.assign(scaling, scaling + n);
  } else {  // no start system
    P.degrees.assign(n, 1);
    P.scaling.assign(n, 1.0);
  }
  return HC_OK;
}

std::string slp_codegen(const SlpProgram& P) {
  Lowered L = lower(P);
  std::ostringstream o;
  o << "// generated from a straight-line program (n = " << P.n << ", " << P.np << " parameters, "
    << P.instr.size() << " instructions, " << L.ins.size() << " lowered operations)\n";
  o << "#include \"hc_slp_ops.cuh\"\nnamespace hcslp {\nconstexpr int NV = " << P.n << ";\n";
  o << "constexpr int NP = " << P.np << ";  // > 0: parameter homotopy F(x; t p + (1 - t) q)\n";
  o << "__constant__ int slp_degree[NV] = {";
  for (int i = 0; i < P.n; ++i) o << (i ? ", " : "") << P.degrees[i];
  o << "};\n__constant__ double slp_scaling[NV] = {";
  for (int i = 0; i < P.n; ++i) o << (i ? ", " : "") << num(P.scaling[i]);
  o << "};\n";
  o << emit_eval(L, false) << emit_eval(L, true);
  for (int K = 1; K <= 3; ++K) o << emit_series(L, K);
  o << "}  // namespace hcslp\n#define HC_SLP 1\n#include \"hc_track_kernel.cuh\"\n";
  return o.str();
}

// ---- NVRTC build, caches
namespace {

uint64_t fnv1a(const std::string& s, uint64_t h = 1469598103934665603ULL) {
  for (unsigned char c : s) {
    h ^= c;
    h *= 1099511628211ULL;
  }
  return h;
}

std::string cache_dir() {
  const char* e = getenv("HCGPU_CACHE");
  if (e && *e) return e;
  const char* home = getenv("HOME");
  return std::string(home && *home ? home : "/tmp") + "/.cache/hcgpu";
}

void mkdirs(const std::string& d) {
  std::string cur;
  for (size_t i = 0; i < d.size(); ++i) {
    cur += d[i];
    if (d[i] == '/' && cur.size() > 1) mkdir(cur.c_str(), 0755);
  }
  mkdir(d.c_str(), 0755);
}

std::mutex g_slp_mu;
std::map<uint64_t, SlpModule> g_slp_modules;  // key: source and options hash

}  // namespace

int slp_build(const std::string& source, bool mixed, SlpModule& out, std::string& err) {
  int dev = 0, major = 0, minor = 0;
  cudaError_t ce = cudaGetDevice(&dev);
  if (ce == cudaSuccess) ce = cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, dev);
  if (ce == cudaSuccess) ce = cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, dev);
  if (ce != cudaSuccess) {
    err = std::string("device query: ") + cudaGetErrorString(ce);
    return HC_ERR_CUDA;
  }
  // sm_XYa: the architecture-specific target of this device (the library itself is built for sm_103a)
  std::string arch = "--gpu-architecture=sm_" + std::to_string(major) + std::to_string(minor) + "a";
  std::vector<std::string> opts = {arch, "-std=c++17", "-default-device", "-diag-suppress=39,177",
                                   "-DHC_NVRTC_KERNEL=1"};
  const char* kname = mixed ? "hcd::track_kernel<true>" : "hcd::track_kernel<false>";
  std::string key_text = source + "\n" + kname;
  for (const std::string& s : opts) key_text += "\n" + s;
  for (int i = 0; i < kJitHeaderCount; ++i) key_text += kJitHeaderSources[i];
  int nv_major = 0, nv_minor = 0;
  nvrtcVersion(&nv_major, &nv_minor);
  key_text += "nvrtc " + std::to_string(nv_major) + "." + std::to_string(nv_minor);
  const uint64_t key = fnv1a(key_text);
  std::lock_guard<std::mutex> g(g_slp_mu);
  auto it = g_slp_modules.find(key);
  if (it != g_slp_modules.end()) {
    out = it->second;
    return HC_OK;
  }
  char hex[17];
  snprintf(hex, sizeof hex, "%016llx", (unsigned long long)key);
  const std::string dir = cache_dir(), path = dir + "/slp_" + hex + ".cubin", names_path = path + ".name";
  std::string cubin, lowered;
  bool cached = false;
  {
    std::ifstream f(path, std::ios::binary), fn(names_path);
    if (f && fn) {
      std::stringstream ss;
      ss << f.rdbuf();
      cubin = ss.str();
      std::getline(fn, lowered);
      cached = !cubin.empty() && !lowered.empty();
    }
  }
  double secs = 0;
  if (!cached) {
    auto t0 = std::chrono::steady_clock::now();
    nvrtcProgram prog;
    nvrtcResult r = nvrtcCreateProgram(&prog, source.c_str(), "hc_slp_system.cu", kJitHeaderCount, kJitHeaderSources,
                                       kJitHeaderNames);
    if (r != NVRTC_SUCCESS) {
      err = std::string("nvrtcCreateProgram: ") + nvrtcGetErrorString(r);
      return HC_ERR_COMPILE;
    }
    nvrtcAddNameExpression(prog, kname);
    std::vector<const char*> copts;
    for (const std::string& s : opts) copts.push_back(s.c_str());
    r = nvrtcCompileProgram(prog, (int)copts.size(), copts.data());
    if (r != NVRTC_SUCCESS) {
      size_t ls = 0;
      nvrtcGetProgramLogSize(prog, &ls);
      std::string log(ls, '\0');
      if (ls) nvrtcGetProgramLog(prog, &log[0]);
      nvrtcDestroyProgram(&prog);
      err = "NVRTC: " + log.substr(0, 4000);
      return HC_ERR_COMPILE;
    }
    size_t cs = 0;
    nvrtcGetCUBINSize(prog, &cs);
    cubin.assign(cs, '\0');
    nvrtcGetCUBIN(prog, &cubin[0]);
    const char* ln = nullptr;
    nvrtcGetLoweredName(prog, kname, &ln);
    lowered = ln ? ln : "";
    nvrtcDestroyProgram(&prog);
    secs = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    // on-disk cache (best effort; written to a temporary name, then renamed)
    mkdirs(dir);
    std::string tmp = path + ".tmp" + std::to_string(getpid());
    {
      std::ofstream f(tmp, std::ios::binary);
      f.write(cubin.data(), (std::streamsize)cubin.size());
    }
    {
      std::ofstream fn(names_path + ".tmp" + std::to_string(getpid()));
      fn << lowered << "\n";
    }
    rename((names_path + ".tmp" + std::to_string(getpid())).c_str(), names_path.c_str());
    rename(tmp.c_str(), path.c_str());
  }
  SlpModule M;
  ce = cudaLibraryLoadData(&M.lib, cubin.data(), nullptr, nullptr, 0, nullptr, nullptr, 0);
  if (ce != cudaSuccess) {
    err = std::string("cudaLibraryLoadData: ") + cudaGetErrorString(ce);
    return HC_ERR_CUDA;
  }
  ce = cudaLibraryGetKernel(&M.kernel, M.lib, lowered.c_str());
  if (ce != cudaSuccess) {
    err = std::string("cudaLibraryGetKernel: ") + cudaGetErrorString(ce);
    cudaLibraryUnload(M.lib);
    return HC_ERR_CUDA;
  }
  M.cubin_bytes = cubin.size();
  M.compile_seconds = secs;
  M.from_cache = cached;
  g_slp_modules[key] = M;  // kept for the life of the process (shared by all handles)
  out = M;
  return HC_OK;
}

}  // namespace hcd
