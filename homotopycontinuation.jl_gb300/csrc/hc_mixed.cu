// hc_mixed.cu — fine mixed cells of a lifted point configuration (host code).
//
// The polyhedral start system (src/polyhedral.jl:7-49) needs the mixed cells of a fine mixed
// subdivision of the supports A_1..A_n under an integer lifting ω; the reference takes them from
// MixedSubdivisions.jl (outside the reference tree). This is an independent implementation of
// the published definition: a mixed cell picks one edge {a_i, b_i} of every support such that
// some inner normal (γ, 1) attains min_{a ∈ A_i} ⟨a, γ⟩ + ω(a) exactly at a_i and b_i for every i.
//
//   1. lower edges of every lifted support (one LP per point pair),
//   2. a relation table: pairs of lower edges of two supports that one normal can select
//      together (one LP per pair),
//   3. depth-first search over the supports, edges filtered by the table and every partial
//      choice checked by an LP; a full choice fixes γ by n linear equations, and the cell is
//      kept when every other lifted point lies strictly above its face.
//
// Each LP is "max s : A_eq γ = b_eq, A_ub γ + s ≤ b_ub, s ≤ 1" (strict feasibility when s > 0).
// The equalities are eliminated (γ = γ₀ + N z) and the remaining problem is solved through its
// dual, min hᵀy + y₀ subject to Gᵀy = 0, 1ᵀy + y₀ = 1, y, y₀ ≥ 0 (G = A_ub N, h = b_ub − A_ub γ₀),
// a standard-form LP with d + 1 rows, by the two-phase simplex method with Bland's rule.
#include <algorithm>
#include <array>
#include <atomic>
#include <cmath>
#include <cstdint>
#include <cstring>
#include <limits>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "../../include/hcgpu.h"

namespace {

constexpr double kTol = 1e-9;
// An LP margin or a cell's slack in (−kFeas, kFeas) is taken for zero: the lifting is not
// generic (a lower face holds more than two points of a support, or two normal cones only
// touch), and the caller draws another one. Exact margins are rationals whose denominators are
// subdeterminants of the small integer exponent differences, far above kFeas in magnitude.
constexpr double kFeas = 1e-7;

// Gaussian elimination of A_eq (k × n, row-major): particular solution γ₀ and null-space
// basis N (n × d, column-major). Returns false when the rows are dependent.
bool eliminate(int n, int k, const std::vector<double>& Aeq, const std::vector<double>& beq, std::vector<double>& g0,
               std::vector<double>& N, int& d) {
  std::vector<double> M((size_t)k * (n + 1));
  for (int i = 0; i < k; ++i) {
    for (int j = 0; j < n; ++j) M[(size_t)i * (n + 1) + j] = Aeq[(size_t)i * n + j];
    M[(size_t)i * (n + 1) + n] = beq[i];
  }
  std::vector<int> pivcol;
  int row = 0;
  for (int c = 0; c < n && row < k; ++c) {
    int best = -1;
    double bv = 1e-9;
    for (int r = row; r < k; ++r)
      if (std::fabs(M[(size_t)r * (n + 1) + c]) > bv) {
        bv = std::fabs(M[(size_t)r * (n + 1) + c]);
        best = r;
      }
    if (best < 0) continue;
    if (best != row)
      for (int j = 0; j <= n; ++j) std::swap(M[(size_t)best * (n + 1) + j], M[(size_t)row * (n + 1) + j]);
    double p = M[(size_t)row * (n + 1) + c];
    for (int j = 0; j <= n; ++j) M[(size_t)row * (n + 1) + j] /= p;
    for (int r = 0; r < k; ++r)
      if (r != row) {
        double f = M[(size_t)r * (n + 1) + c];
        if (f != 0.0)
          for (int j = 0; j <= n; ++j) M[(size_t)r * (n + 1) + j] -= f * M[(size_t)row * (n + 1) + j];
      }
    pivcol.push_back(c);
    ++row;
  }
  if (row < k) return false;
  std::vector<char> isp(n, 0);
  for (int c : pivcol) isp[c] = 1;
  d = n - k;
  g0.assign(n, 0.0);
  for (int i = 0; i < k; ++i) g0[pivcol[i]] = M[(size_t)i * (n + 1) + n];
  N.assign((size_t)n * d, 0.0);
  int col = 0;
  for (int f = 0; f < n; ++f) {
    if (isp[f]) continue;
    N[(size_t)col * n + f] = 1.0;
    for (int i = 0; i < k; ++i) N[(size_t)col * n + pivcol[i]] = -M[(size_t)i * (n + 1) + f];
    ++col;
  }
  return true;
}

// min cᵀx s.t. A x = b, x ≥ 0 for b ≥ 0 (rows × cols, row-major); two-phase simplex with
// Bland's rule. Returns the optimum (the problems solved here are feasible and bounded).
double simplex_min(int rows, int cols, const std::vector<double>& A, const std::vector<double>& b,
                   const std::vector<double>& c) {
  // tableau columns: cols structural, rows artificial, rhs
  const int W = cols + rows + 1;
  std::vector<double> T((size_t)(rows + 1) * W, 0.0);
  std::vector<int> basis(rows);
  for (int i = 0; i < rows; ++i) {
    for (int j = 0; j < cols; ++j) T[(size_t)i * W + j] = A[(size_t)i * cols + j];
    T[(size_t)i * W + cols + i] = 1.0;
    T[(size_t)i * W + W - 1] = b[i];
    basis[i] = cols + i;
  }
  auto pivot = [&](int pr, int pc) {
    double p = T[(size_t)pr * W + pc];
    for (int j = 0; j < W; ++j) T[(size_t)pr * W + j] /= p;
    for (int r = 0; r <= rows; ++r) {
      if (r == pr) continue;
      double f = T[(size_t)r * W + pc];
      if (f != 0.0)
        for (int j = 0; j < W; ++j) T[(size_t)r * W + j] -= f * T[(size_t)pr * W + j];
    }
    basis[pr] = pc;
  };
  auto run = [&](int ncand) {
    for (int it = 0; it < 50000; ++it) {
      int pc = -1;
      for (int j = 0; j < ncand; ++j)
        if (T[(size_t)rows * W + j] < -kTol) {
          pc = j;
          break;
        }
      if (pc < 0) return true;
      int pr = -1;
      double best = std::numeric_limits<double>::infinity();
      for (int r = 0; r < rows; ++r) {
        double a = T[(size_t)r * W + pc];
        if (a > kTol) {
          double q = T[(size_t)r * W + W - 1] / a;
          if (q < best - 1e-12 || (q <= best + 1e-12 && pr >= 0 && basis[r] < basis[pr])) {
            best = q;
            pr = r;
          }
        }
      }
      if (pr < 0) return false;  // unbounded
      pivot(pr, pc);
    }
    return true;
  };
  // phase 1: minimise the sum of the artificials (reduced costs of the structural columns)
  for (int j = 0; j < W; ++j) T[(size_t)rows * W + j] = 0.0;
  for (int i = 0; i < rows; ++i)
    for (int j = 0; j < cols; ++j) T[(size_t)rows * W + j] -= T[(size_t)i * W + j];
  for (int i = 0; i < rows; ++i) T[(size_t)rows * W + W - 1] -= T[(size_t)i * W + W - 1];
  run(cols);
  // drive artificials at level zero out of the basis where a structural pivot exists
  for (int r = 0; r < rows; ++r)
    if (basis[r] >= cols)
      for (int j = 0; j < cols; ++j)
        if (std::fabs(T[(size_t)r * W + j]) > kTol) {
          pivot(r, j);
          break;
        }
  // phase 2: objective row from c (artificials never enter)
  for (int j = 0; j < W; ++j) T[(size_t)rows * W + j] = 0.0;
  for (int j = 0; j < cols; ++j) T[(size_t)rows * W + j] = c[j];
  for (int r = 0; r < rows; ++r) {
    int bj = basis[r];
    double cb = bj < cols ? c[bj] : 0.0;
    if (cb != 0.0)
      for (int j = 0; j < W; ++j) T[(size_t)rows * W + j] -= cb * T[(size_t)r * W + j];
  }
  if (!run(cols)) return -std::numeric_limits<double>::infinity();
  return -T[(size_t)rows * W + W - 1];
}

// max s : A_eq γ = b_eq, A_ub γ + s ≤ b_ub, s ≤ 1 (see the file comment); −inf if the
// equalities are dependent.
double lp_margin(int n, const std::vector<double>& Aeq, const std::vector<double>& beq, const std::vector<double>& Aub,
                 const std::vector<double>& bub) {
  const int k = (int)beq.size(), r = (int)bub.size();
  std::vector<double> g0, N;
  int d = 0;
  if (!eliminate(n, k, Aeq, beq, g0, N, d)) return -std::numeric_limits<double>::infinity();
  std::vector<double> h(r), G((size_t)r * d);
  for (int i = 0; i < r; ++i) {
    double acc = bub[i];
    for (int j = 0; j < n; ++j) acc -= Aub[(size_t)i * n + j] * g0[j];
    h[i] = acc;
    for (int c = 0; c < d; ++c) {
      double g = 0.0;
      for (int j = 0; j < n; ++j) g += Aub[(size_t)i * n + j] * N[(size_t)c * n + j];
      G[(size_t)i * d + c] = g;
    }
  }
  if (d == 0) {
    double s = 1.0;
    for (double v : h) s = std::min(s, v);
    return s;
  }
  // dual: rows Gᵀy = 0 (d) and 1ᵀy + y0 = 1; columns y (r), y0
  const int rows = d + 1, cols = r + 1;
  std::vector<double> A((size_t)rows * cols, 0.0), b(rows, 0.0), c(cols);
  for (int c2 = 0; c2 < d; ++c2)
    for (int i = 0; i < r; ++i) A[(size_t)c2 * cols + i] = G[(size_t)i * d + c2];
  for (int i = 0; i < r; ++i) A[(size_t)d * cols + i] = 1.0;
  A[(size_t)d * cols + r] = 1.0;
  b[d] = 1.0;
  for (int i = 0; i < r; ++i) c[i] = h[i];
  c[r] = 1.0;
  return simplex_min(rows, cols, A, b, c);
}

struct Edge {
  int p, q;
  std::vector<double> eq;   // a_p − a_q
  double eqb;               // ω_q − ω_p
  std::vector<double> ub;   // rows a_p − a_c (c ≠ p, q)
  std::vector<double> ubb;  // ω_c − ω_p
};

long long det_bareiss(int n, std::vector<long long> M) {
  __int128 prev = 1;
  std::vector<__int128> A(M.begin(), M.end());
  int sign = 1;
  for (int k = 0; k < n - 1; ++k) {
    if (A[(size_t)k * n + k] == 0) {
      int s = -1;
      for (int r = k + 1; r < n; ++r)
        if (A[(size_t)r * n + k] != 0) {
          s = r;
          break;
        }
      if (s < 0) return 0;
      for (int j = 0; j < n; ++j) std::swap(A[(size_t)k * n + j], A[(size_t)s * n + j]);
      sign = -sign;
    }
    for (int i = k + 1; i < n; ++i)
      for (int j = k + 1; j < n; ++j)
        A[(size_t)i * n + j] = (A[(size_t)i * n + j] * A[(size_t)k * n + k] - A[(size_t)i * n + k] * A[(size_t)k * n + j]) / prev;
    prev = A[(size_t)k * n + k];
  }
  __int128 dt = A[(size_t)(n - 1) * n + (n - 1)] * sign;
  return (long long)(dt < 0 ? -dt : dt);
}

struct Cell {
  std::vector<int> idx;  // 2n
  std::vector<double> normal, beta;
  long long volume;
};

struct Search {
  int n;
  const std::vector<std::vector<std::vector<int>>>* pts;  // [support][point][coordinate]
  const std::vector<std::vector<long long>>* lift;
  std::vector<std::vector<Edge>> edges;
  std::vector<int> order;
  std::vector<std::vector<std::vector<char>>> compat;  // [a][b][x * |E_b| + y], a < b in search order
  std::mutex mu;
  std::vector<Cell> cells;
  std::atomic<bool> degenerate{false};

  // feasible (1), infeasible (0); a margin near zero marks the lifting as not generic
  int classify(double margin) {
    if (margin > kFeas) return 1;
    if (margin < -kFeas || std::isinf(margin)) return 0;
    degenerate = true;
    return 0;
  }

  void rec(int depth, std::vector<int>& pick, std::vector<double>& Aeq, std::vector<double>& beq,
           std::vector<double>& Aub, std::vector<double>& bub) {
    if (degenerate.load(std::memory_order_relaxed)) return;
    if (depth == n) {
      leaf(pick, Aeq, beq, Aub, bub);
      return;
    }
    const int i = order[depth];
    const std::vector<Edge>& E = edges[i];
    for (int y = 0; y < (int)E.size(); ++y) {
      bool ok = true;
      for (int a = 0; a < depth && ok; ++a) ok = compat[a][depth][(size_t)pick[a] * E.size() + y] != 0;
      if (!ok) continue;
      const Edge& e = E[y];
      size_t ke = Aeq.size(), kb = beq.size(), ku = Aub.size(), kub = bub.size();
      Aeq.insert(Aeq.end(), e.eq.begin(), e.eq.end());
      beq.push_back(e.eqb);
      Aub.insert(Aub.end(), e.ub.begin(), e.ub.end());
      bub.insert(bub.end(), e.ubb.begin(), e.ubb.end());
      bool feasible = true;
      if (depth >= 2 && depth + 1 < n) feasible = classify(lp_margin(n, Aeq, beq, Aub, bub)) != 0;
      if (feasible) {
        pick[depth] = y;
        rec(depth + 1, pick, Aeq, beq, Aub, bub);
      }
      Aeq.resize(ke);
      beq.resize(kb);
      Aub.resize(ku);
      bub.resize(kub);
    }
  }

  void leaf(const std::vector<int>& pick, const std::vector<double>& Aeq, const std::vector<double>& beq,
            const std::vector<double>& Aub, const std::vector<double>& bub) {
    std::vector<long long> M((size_t)n * n);
    for (int r = 0; r < n; ++r)
      for (int j = 0; j < n; ++j) M[(size_t)r * n + j] = (long long)std::llround(Aeq[(size_t)r * n + j]);
    long long vol = det_bareiss(n, M);
    if (vol == 0) return;
    std::vector<double> g, N;
    int d = 0;
    if (!eliminate(n, n, Aeq, beq, g, N, d)) return;
    // the slacks are rationals with denominator |det| = vol: |slack| ≥ 1/vol unless zero
    const double eps = std::min(kFeas, 0.25 / (double)vol);
    double smin = std::numeric_limits<double>::infinity();
    for (size_t r = 0; r < bub.size(); ++r) {
      double acc = bub[r];
      for (int j = 0; j < n; ++j) acc -= Aub[r * n + j] * g[j];
      smin = std::min(smin, acc);
    }
    if (smin < -eps) return;
    if (smin <= eps) {
      degenerate = true;
      return;
    }
    Cell c;
    c.idx.assign(2 * n, 0);
    c.beta.assign(n, 0.0);
    for (int depth = 0; depth < n; ++depth) {
      int i = order[depth];
      const Edge& e = edges[i][pick[depth]];
      c.idx[2 * i] = e.p;
      c.idx[2 * i + 1] = e.q;
      double b = (double)(*lift)[i][e.p];
      for (int j = 0; j < n; ++j) b += (double)(*pts)[i][e.p][j] * g[j];
      c.beta[i] = b;
    }
    c.normal = g;
    c.volume = vol;
    std::lock_guard<std::mutex> lk(mu);
    cells.push_back(std::move(c));
  }
};

template <class F>
void parallel_for(int count, F&& f) {
  unsigned hw = std::max(1u, std::thread::hardware_concurrency());
  int nt = (int)std::min<unsigned>(hw, (unsigned)std::max(1, count));
  std::atomic<int> next(0);
  std::vector<std::thread> th;
  for (int t = 0; t < nt; ++t)
    th.emplace_back([&]() {
      for (int k = next.fetch_add(1); k < count; k = next.fetch_add(1)) f(k);
    });
  for (auto& t : th) t.join();
}

}  // namespace

// the library's error slot (hc_last_error(NULL)), defined in hc_capi.cu
int hc_library_fail(int code, const char* msg);
static int mixed_fail(int code, const char* msg) { return hc_library_fail(code, msg); }

extern "C" {

int hc_mixed_cells(int n, const int32_t* nterms, const int32_t* points, const int64_t* lifting, int64_t max_cells,
                   int32_t* out_indices, double* out_normals, double* out_beta, int64_t* out_volumes,
                   int64_t* out_ncells) {
  if (n < 1 || n > 32 || !nterms || !points || !lifting || !out_ncells)
    return mixed_fail(HC_ERR_INVALID_ARG, "hc_mixed_cells: bad arguments");
  std::vector<std::vector<std::vector<int>>> pts(n);
  std::vector<std::vector<long long>> lift(n);
  size_t off = 0;
  for (int i = 0; i < n; ++i) {
    if (nterms[i] < 1) return mixed_fail(HC_ERR_INVALID_ARG, "hc_mixed_cells: empty support");
    pts[i].resize(nterms[i], std::vector<int>(n));
    lift[i].resize(nterms[i]);
    for (int k = 0; k < nterms[i]; ++k, ++off) {
      for (int j = 0; j < n; ++j) pts[i][k][j] = points[off * n + j];
      lift[i][k] = lifting[off];
    }
  }
  Search S;
  S.n = n;
  S.pts = &pts;
  S.lift = &lift;
  S.edges.resize(n);
  // 1. lower edges
  for (int i = 0; i < n; ++i) {
    const int m = (int)pts[i].size();
    std::vector<std::pair<int, int>> pairs;
    for (int p = 0; p < m; ++p)
      for (int q = p + 1; q < m; ++q) pairs.push_back({p, q});
    std::vector<Edge> cand(pairs.size());
    std::vector<char> keep(pairs.size(), 0);
    parallel_for((int)pairs.size(), [&](int t) {
      int p = pairs[t].first, q = pairs[t].second;
      Edge& e = cand[t];
      e.p = p;
      e.q = q;
      e.eq.resize(n);
      bool nz = false;
      for (int j = 0; j < n; ++j) {
        e.eq[j] = pts[i][p][j] - pts[i][q][j];
        nz = nz || e.eq[j] != 0;
      }
      if (!nz) return;
      e.eqb = (double)(lift[i][q] - lift[i][p]);
      for (int c = 0; c < m; ++c) {
        if (c == p || c == q) continue;
        for (int j = 0; j < n; ++j) e.ub.push_back(pts[i][p][j] - pts[i][c][j]);
        e.ubb.push_back((double)(lift[i][c] - lift[i][p]));
      }
      std::vector<double> be(1, e.eqb);
      keep[t] = S.classify(lp_margin(n, e.eq, be, e.ub, e.ubb));
    });
    for (size_t t = 0; t < cand.size(); ++t)
      if (keep[t]) S.edges[i].push_back(std::move(cand[t]));
  }
  S.order.resize(n);
  for (int i = 0; i < n; ++i) S.order[i] = i;
  std::stable_sort(S.order.begin(), S.order.end(),
                   [&](int a, int b) { return S.edges[a].size() < S.edges[b].size(); });
  // 2. relation table
  S.compat.assign(n, std::vector<std::vector<char>>(n));
  std::vector<std::pair<int, int>> tab;
  for (int a = 0; a < n; ++a)
    for (int b = a + 1; b < n; ++b) tab.push_back({a, b});
  for (auto& ab : tab) {
    const auto& Ea = S.edges[S.order[ab.first]];
    const auto& Eb = S.edges[S.order[ab.second]];
    S.compat[ab.first][ab.second].assign(Ea.size() * Eb.size(), 0);
  }
  std::vector<std::array<int, 3>> jobs;
  for (size_t t = 0; t < tab.size(); ++t)
    for (size_t x = 0; x < S.edges[S.order[tab[t].first]].size(); ++x) jobs.push_back({(int)t, (int)x, 0});
  parallel_for((int)jobs.size(), [&](int jj) {
    const auto& ab = tab[jobs[jj][0]];
    const int x = jobs[jj][1];
    const auto& Ea = S.edges[S.order[ab.first]];
    const auto& Eb = S.edges[S.order[ab.second]];
    const Edge& e = Ea[x];
    for (size_t y = 0; y < Eb.size(); ++y) {
      const Edge& f = Eb[y];
      std::vector<double> Aeq(e.eq), beq{e.eqb, f.eqb}, Aub(e.ub), bub(e.ubb);
      Aeq.insert(Aeq.end(), f.eq.begin(), f.eq.end());
      Aub.insert(Aub.end(), f.ub.begin(), f.ub.end());
      bub.insert(bub.end(), f.ubb.begin(), f.ubb.end());
      S.compat[ab.first][ab.second][(size_t)x * Eb.size() + y] = (char)S.classify(lp_margin(n, Aeq, beq, Aub, bub));
    }
  });
  // 3. search, in parallel over the edges of the first support
  if (n == 1) {
    for (int y = 0; y < (int)S.edges[0].size(); ++y) {
      std::vector<int> pick(1, y);
      S.leaf(pick, S.edges[0][y].eq, std::vector<double>{S.edges[0][y].eqb}, S.edges[0][y].ub, S.edges[0][y].ubb);
    }
  } else {
    parallel_for((int)S.edges[S.order[0]].size(), [&](int y) {
      const Edge& e = S.edges[S.order[0]][y];
      std::vector<int> pick(n, 0);
      pick[0] = y;
      std::vector<double> Aeq(e.eq), beq{e.eqb}, Aub(e.ub), bub(e.ubb);
      S.rec(1, pick, Aeq, beq, Aub, bub);
    });
  }
  if (S.degenerate) return mixed_fail(HC_ERR_INVALID_ARG, "hc_mixed_cells: the lifting is not generic");
  // deterministic order: by the cells' index tuples
  std::sort(S.cells.begin(), S.cells.end(), [](const Cell& a, const Cell& b) { return a.idx < b.idx; });
  *out_ncells = (int64_t)S.cells.size();
  if ((int64_t)S.cells.size() > max_cells)
    return mixed_fail(HC_ERR_TOO_LARGE, "hc_mixed_cells: more cells than max_cells (count in *out_ncells)");
  for (size_t c = 0; c < S.cells.size(); ++c) {
    const Cell& C = S.cells[c];
    if (out_indices)
      for (int j = 0; j < 2 * n; ++j) out_indices[c * 2 * n + j] = C.idx[j];
    if (out_normals)
      for (int j = 0; j < n; ++j) out_normals[c * n + j] = C.normal[j];
    if (out_beta)
      for (int j = 0; j < n; ++j) out_beta[c * n + j] = C.beta[j];
    if (out_volumes) out_volumes[c] = C.volume;
  }
  return HC_OK;
}

}  // extern "C"
