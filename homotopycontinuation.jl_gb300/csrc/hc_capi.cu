// hc_capi.cu — the extern "C" boundary of libhcgpu.so (declared in include/hcgpu.h):
// handle and option management, the host-side compilation of a homotopy into a monomial
// program with a static lane schedule, and the batched track calls.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <numeric>
#include <string>
#include <thread>
#include <vector>

#include "hc_dev.h"
#include "hc_slp.h"

namespace hcd {
cudaError_t launch_track(const Launch& la, int blocks, int warps_per_cta, cudaStream_t stream);
cudaError_t occupancy(int precision, int warps_per_cta, size_t smem, int* blocks_per_sm);
cudaError_t prepare_batch(int precision, size_t smem, int warps_per_cta, int* blocks_per_sm);
int certify_layout(const DevProg& P, int* bytes_out);
cudaError_t launch_certify(const DevProg& P, int64_t nitems, const int64_t* d_list, bool dw, const double* d_in,
                           hc_certificate* d_out, double* d_centers, double* d_enclosures, int real_coefficients,
                           int num_sms, cudaStream_t stream);
cudaError_t launch_batch(const BatchLaunch& bl, int blocks, int warps_per_cta, size_t smem, cudaStream_t stream);
}  // namespace hcd

using namespace hcd;

namespace {

std::mutex g_err_mu;
std::string g_err;

struct Term {
  int row;
  int mono;
  double re, im;
  int vterm;  // Jacobian terms: index of the value term supplying the coefficient
  int mult;   // Jacobian terms: exponent multiplier
  int orig;   // value terms: position in the caller's order
};

// Host copy of a compiled homotopy
struct HostProg {
  int n = 0, M = 0, nlev = 0, top = 0;
  std::vector<int2> mdef;
  std::vector<int> lev;
  struct Rows {
    int nrows = 0, nslots = 0;
    std::vector<int4> seg;
    std::vector<int> lane_seg, row_slot;
  } val, jac;
  std::vector<double2> vcoef64;
  std::vector<float2> vcoef32;
  std::vector<uint16_t> vmono;
  std::vector<uint32_t> jcode;
  std::vector<int> vorig;  // value storage index k holds the caller's term vorig[k] (F, then G)
  // operation census for the flop model
  long long val_terms = 0, jac_terms = 0;
};

// Monomial table closed under "parent" (drop one power of the first variable) and under
// the derivative monomials the Jacobian rows need; degree-ordered levels.
struct MonoTable {
  int n;
  std::map<std::vector<int>, int> idx;
  std::vector<std::vector<int>> list;
  explicit MonoTable(int nn) : n(nn) {}
  void insert(const std::vector<int>& e) {
    if (idx.count(e)) return;
    int deg = 0, v = -1;
    for (int j = 0; j < n; ++j) {
      deg += e[j];
      if (v < 0 && e[j] > 0) v = j;
    }
    if (deg > 0) {
      std::vector<int> p = e;
      p[v] -= 1;
      insert(p);
    }
    idx[e] = -1;
    list.push_back(e);
  }
};

// Lane schedule of a row table (terms sorted by row, then by multiplier), in two parts.
//  * Aligned groups: rows with identical (monomial, multiplier) sequences — every F row of a
//    dense system, and for each variable the n rows ∂F_i/∂x_j — are run g = group size lanes
//    side by side: lane set k (of s = ⌊32/g⌋ sets) takes piece k of every such row, so the g
//    lanes of a set read the same monomial at every step (one broadcast shared-memory load)
//    and the pieces are equal.
//  * The other rows are cut into segments of one multiplier and at most ~T/(32·per_lane) terms
//    and spread over the lanes, longest first to the least loaded lane.
// Slots are numbered row-major so a row's partials are contiguous and its total is a
// fixed-order sum; a lane runs its aligned pieces first, in the same order as its set.
// Storage: an aligned piece of the g rows is stored position-major (the g rows' terms at one
// position side by side), so the set's lanes read g consecutive coefficients; a segment is
// (stride, first storage index, end index, slot | multiplier << 24), and pos[k] receives the
// storage index of term k.
void build_segments(int nrows, const std::vector<Term>& terms, int per_lane, HostProg::Rows& R,
                    std::vector<int>& pos, bool align) {
  R.nrows = nrows;
  int T = (int)terms.size();
  std::vector<int> row_begin(nrows + 1, 0);
  for (int k = 0; k < T; ++k) row_begin[terms[k].row + 1] += 1;
  for (int r = 0; r < nrows; ++r) row_begin[r + 1] += row_begin[r];
  struct Chunk {
    int row, b, e, mult, start, stride;  // terms [b, e) stored from start with the stride
  };
  std::vector<Chunk> chunks;
  std::vector<std::vector<int>> lane_chunks(32);
  pos.assign(T, 0);
  int next = 0;  // next free storage index
  std::vector<long long> load(32, 0);
  // rows grouped by their (monomial, multiplier) sequence
  std::map<std::vector<std::pair<int, int>>, std::vector<int>> groups;
  for (int r = 0; r < nrows && align; ++r) {
    if (row_begin[r + 1] - row_begin[r] < 8) continue;
    std::vector<std::pair<int, int>> sig;
    for (int k = row_begin[r]; k < row_begin[r + 1]; ++k) sig.push_back({terms[k].mono, terms[k].mult});
    groups[sig].push_back(r);
  }
  // the group size carrying the most terms
  std::map<int, long long> by_size;
  for (auto& kv : groups)
    if (kv.second.size() >= 2) by_size[(int)kv.second.size()] += (long long)kv.first.size() * kv.second.size();
  int g = 0;
  long long best = 0;
  for (auto& kv : by_size)
    if (kv.first <= 32 && kv.second > best) {
      best = kv.second;
      g = kv.first;
    }
  std::vector<char> aligned(nrows, 0);
  if (g >= 2) {
    const int sets = 32 / g;
    for (auto& kv : groups) {
      if ((int)kv.second.size() != g) continue;
      const int Lr = (int)kv.first.size();
      for (int set = 0; set < sets; ++set) {
        const int pb = (int)((long long)Lr * set / sets), pe = (int)((long long)Lr * (set + 1) / sets);
        // the piece, cut where the multiplier changes (the same places in every row of the group)
        int k = pb;
        while (k < pe) {
          int k2 = k;
          while (k2 < pe && kv.first[k2].second == kv.first[k].second) ++k2;
          for (int m = 0; m < g; ++m) {
            const int r = kv.second[m], lane = set * g + m;
            lane_chunks[lane].push_back((int)chunks.size());
            chunks.push_back({r, row_begin[r] + k, row_begin[r] + k2, kv.first[k].second, next + m, g});
            for (int q = k; q < k2; ++q) pos[row_begin[r] + q] = next + (q - k) * g + m;
            load[lane] += k2 - k + 2;
          }
          next += (k2 - k) * g;
          k = k2;
        }
      }
      for (int r : kv.second) aligned[r] = 1;
    }
  }
  // the remaining rows
  int Trest = 0;
  for (int r = 0; r < nrows; ++r)
    if (!aligned[r]) Trest += row_begin[r + 1] - row_begin[r];
  const int L = std::max(8, (Trest + 32 * per_lane - 1) / (32 * per_lane));
  std::vector<int> rest;
  for (int r = 0; r < nrows; ++r) {
    if (aligned[r]) continue;
    int b = row_begin[r], e = row_begin[r + 1];
    int k = b;
    while (k < e) {  // runs of equal multiplier
      int k2 = k;
      while (k2 < e && terms[k2].mult == terms[k].mult) ++k2;
      int t = k2 - k;
      int nc = (t + L - 1) / L;
      for (int c = 0; c < nc; ++c) {
        int cb = k + (int)((long long)t * c / nc), ce = k + (int)((long long)t * (c + 1) / nc);
        rest.push_back((int)chunks.size());
        chunks.push_back({r, cb, ce, terms[k].mult, next, 1});
        for (int q = cb; q < ce; ++q) pos[q] = next + (q - cb);
        next += ce - cb;
      }
      k = k2;
    }
  }
  std::stable_sort(rest.begin(), rest.end(), [&](int a, int b) {
    return (chunks[a].e - chunks[a].b) > (chunks[b].e - chunks[b].b);
  });
  for (int ci : rest) {
    int bl = 0;
    for (int l = 1; l < 32; ++l)
      if (load[l] < load[bl]) bl = l;
    load[bl] += chunks[ci].e - chunks[ci].b + 2;
    lane_chunks[bl].push_back(ci);
  }
  for (int l = 0; l < 32; ++l) {  // aligned pieces first (in set order), then the rest by position
    auto it = std::stable_partition(lane_chunks[l].begin(), lane_chunks[l].end(),
                                    [&](int ci) { return aligned[chunks[ci].row] != 0; });
    std::sort(it, lane_chunks[l].end());
  }
  // slots in row-major order
  std::vector<int> order(chunks.size());
  std::iota(order.begin(), order.end(), 0);
  std::sort(order.begin(), order.end(), [&](int a, int b) {
    return chunks[a].row != chunks[b].row ? chunks[a].row < chunks[b].row : chunks[a].b < chunks[b].b;
  });
  std::vector<int> slot(chunks.size());
  R.row_slot.assign(nrows + 1, 0);
  for (size_t i = 0; i < order.size(); ++i) {
    slot[order[i]] = (int)i;
    R.row_slot[chunks[order[i]].row + 1] += 1;
  }
  for (int r = 0; r < nrows; ++r) R.row_slot[r + 1] += R.row_slot[r];
  R.nslots = (int)chunks.size();
  R.seg.clear();
  R.lane_seg.assign(33, 0);
  for (int l = 0; l < 32; ++l) {
    for (int ci : lane_chunks[l]) {
      const Chunk& c = chunks[ci];
      R.seg.push_back(make_int4(c.stride, c.start, c.start + (c.e - c.b) * c.stride, slot[ci] | (c.mult << 24)));
    }
    R.lane_seg[l + 1] = (int)R.seg.size();
  }
}

// full_series: every monomial keeps four Taylor orders (the toric homotopy's series rows read
// all of them), not only the two the straight-line rows need of the top degree
int build_program(int n, int nG, const int32_t* G_eq, const int32_t* G_exps, const double* G_coef, int nF,
                  const int32_t* F_eq, const int32_t* F_exps, const double* F_coef, HostProg& P,
                  std::string& err, bool full_series = false) {
  MonoTable mt(n);
  std::vector<int> zero(n, 0);
  mt.insert(zero);
  std::vector<int> e(n);
  int maxexp = 0;
  auto visit = [&](int cnt, const int32_t* eqs, const int32_t* exps) -> bool {
    for (int k = 0; k < cnt; ++k) {
      if (eqs[k] < 0 || eqs[k] >= n) return false;
      for (int j = 0; j < n; ++j) {
        e[j] = exps[(size_t)k * n + j];
        if (e[j] < 0) return false;
        maxexp = std::max(maxexp, e[j]);
      }
      mt.insert(e);
      for (int j = 0; j < n; ++j)
        if (e[j] > 0) {
          std::vector<int> d = e;
          d[j] -= 1;
          mt.insert(d);
        }
    }
    return true;
  };
  if (!visit(nG, G_eq, G_exps) || !visit(nF, F_eq, F_exps)) {
    err = "term table has an equation index outside [0,n) or a negative exponent";
    return HC_ERR_INVALID_ARG;
  }
  if (mt.list.size() > 65535 || (size_t)nG + nF > 65535) {
    err = "homotopy needs more than 65535 monomials or value terms";
    return HC_ERR_TOO_LARGE;
  }
  if (maxexp > 255) {
    err = "exponents above 255 are not supported";
    return HC_ERR_TOO_LARGE;
  }
  std::vector<std::vector<int>> mons = mt.list;
  std::stable_sort(mons.begin(), mons.end(), [](const std::vector<int>& a, const std::vector<int>& b) {
    int da = std::accumulate(a.begin(), a.end(), 0), db = std::accumulate(b.begin(), b.end(), 0);
    if (da != db) return da < db;
    return a > b;
  });
  std::map<std::vector<int>, int> index;
  for (size_t i = 0; i < mons.size(); ++i) index[mons[i]] = (int)i;
  P.n = n;
  P.M = (int)mons.size();
  P.mdef.assign(P.M, make_int2(0, 0));
  int maxdeg = 0;
  for (int m = 1; m < P.M; ++m) {
    const std::vector<int>& me = mons[m];
    int v = 0;
    while (me[v] == 0) ++v;
    std::vector<int> p = me;
    p[v] -= 1;
    P.mdef[m] = make_int2(index[p], v);
    maxdeg = std::max(maxdeg, std::accumulate(me.begin(), me.end(), 0));
  }
  P.lev.assign(maxdeg + 2, 0);
  {
    int cur = 0;
    for (int d = 0; d <= maxdeg; ++d) {
      P.lev[d] = cur;
      while (cur < P.M && std::accumulate(mons[cur].begin(), mons[cur].end(), 0) == d) ++cur;
    }
    P.lev[maxdeg + 1] = cur;
  }
  P.nlev = maxdeg + 1;
  P.top = full_series ? P.M : P.lev[maxdeg];
  // value terms (rows F_0..F_{n-1}, G_0..G_{n-1}) in caller order, then stably sorted by row
  std::vector<Term> vt;
  std::vector<std::vector<int>> vexp;
  auto addv = [&](int cnt, const int32_t* eqs, const int32_t* exps, const double* cf, int rowoff) {
    for (int k = 0; k < cnt; ++k) {
      for (int j = 0; j < n; ++j) e[j] = exps[(size_t)k * n + j];
      vt.push_back({rowoff + eqs[k], index[e], cf[2 * k], cf[2 * k + 1], 0, 1, (int)vt.size()});
      vexp.push_back(e);
    }
  };
  addv(nF, F_eq, F_exps, F_coef, 0);
  addv(nG, G_eq, G_exps, G_coef, n);
  std::stable_sort(vt.begin(), vt.end(), [](const Term& a, const Term& b) { return a.row < b.row; });
  // value terms at their storage indices (build_segments)
  std::vector<int> posv, posj;
  build_segments(2 * n, vt, 2, P.val, posv, true);
  P.vcoef64.resize(vt.size());
  P.vcoef32.resize(vt.size());
  P.vmono.resize(vt.size());
  P.vorig.resize(vt.size());
  for (size_t k = 0; k < vt.size(); ++k) {
    const int p = posv[k];
    P.vorig[p] = vt[k].orig;
    P.vcoef64[p] = make_double2(vt[k].re, vt[k].im);
    P.vcoef32[p] = make_float2((float)vt[k].re, (float)vt[k].im);
    P.vmono[p] = (uint16_t)vt[k].mono;
  }
  // Jacobian terms: ∂/∂x_j of value term k → (row, monomial e - e_j, storage index of value
  // term k, e_j)
  std::vector<Term> jt;
  for (size_t k = 0; k < vt.size(); ++k) {
    const std::vector<int>& ex = vexp[vt[k].orig];
    int eq = vt[k].row < n ? vt[k].row : vt[k].row - n;
    int off = vt[k].row < n ? 0 : n * n;
    for (int j = 0; j < n; ++j)
      if (ex[j] > 0) {
        std::vector<int> d = ex;
        d[j] -= 1;
        jt.push_back({off + j * n + eq, index[d], 0, 0, posv[k], ex[j], 0});
      }
  }
  std::stable_sort(jt.begin(), jt.end(), [](const Term& a, const Term& b) {
    return a.row != b.row ? a.row < b.row : a.mult < b.mult;
  });
  build_segments(2 * n * n, jt, 4, P.jac, posj, false);
  P.jcode.resize(jt.size());
  for (size_t k = 0; k < jt.size(); ++k) P.jcode[posj[k]] = (uint32_t)jt[k].mono | ((uint32_t)jt[k].vterm << 16);
  P.val_terms = (long long)vt.size();
  P.jac_terms = (long long)jt.size();
  return HC_OK;
}

inline int pad16(size_t b) { return (int)((b + 15) & ~(size_t)15); }

// vc64_global: the FP64 value coefficients stay in global memory (read through L1/L2) instead of
// being staged per CTA
TableLayout make_table_layout(const HostProg& P, int precision, bool vc64_global = false) {
  TableLayout T{};
  int off = 0;
  T.vc64_global = vc64_global ? 1 : 0;
  T.n64 = vc64_global ? 0 : pad16(P.vcoef64.size() * sizeof(double2));
  T.n32 = precision == HC_PREC_MIXED ? pad16(P.vcoef32.size() * sizeof(float2)) : 0;
  T.nmono = pad16(P.vmono.size() * sizeof(uint16_t));
  T.njcode = pad16(P.jcode.size() * sizeof(uint32_t));
  T.nmdef = pad16(P.mdef.size() * sizeof(int2));
  T.vcoef64 = off;
  off += T.n64;
  T.vcoef32 = off;
  off += T.n32;
  T.vmono = off;
  off += T.nmono;
  T.jcode = off;
  off += T.njcode;
  T.mdef = off;
  off += T.nmdef;
  T.bytes = off;
  return T;
}

// Per-warp shared layout. cold = true (mixed precision): shared memory holds what the FP32
// phases and the FP64 residual use every step — FP64 and FP32 monomials, FP32 Taylor series,
// FP64 value and FP32 Jacobian / Taylor partial sums — and the FP64 areas of the rare steps
// (double-double monomials and sums, FP64 series, FP64 Jacobian sums) go to a per-warp slice of
// global memory of L.cold bytes. This roughly halves the per-warp footprint and doubles the
// warps per SM.
WarpLayout make_warp_layout(const HostProg& P, int tor_n = 0, bool cold = false) {
  WarpLayout L{};
  int n = P.n;
  int vn = (n + 1) & ~1;
  size_t off = 0;
  auto take = [&](size_t bytes) {
    size_t o = off;
    off += (bytes + 15) & ~(size_t)15;
    return (int)o;
  };
  auto up16 = [](size_t b) { return (b + 15) & ~(size_t)15; };
  L.state = take(HC_STATE_BYTES);
  size_t series = (size_t)16 * (4 * (size_t)P.top + 2 * (size_t)(P.M - P.top));
  size_t mono_all = std::max({(size_t)P.M * 32, (size_t)P.M * 24, series});
  size_t part_all = std::max({(size_t)P.val.nslots * 32, (size_t)P.jac.nslots * 16, (size_t)16});
  if (cold) {
    L.jmono = (size_t)P.jac.nslots * 8 <= (size_t)P.M * 16 ? 1 : 0;
    L.mono = take(std::max({(size_t)P.M * 24, series / 2, (size_t)16}));
    L.part = take(std::max({(size_t)P.val.nslots * 24, L.jmono ? (size_t)0 : (size_t)P.jac.nslots * 8, (size_t)16}));
    L.cmono = 0;
    L.cpart = (int)up16(mono_all);
    L.cold = (int)(up16(mono_all) + up16(part_all));
  } else {
    L.mono = take(mono_all);
    L.part = take(part_all);
  }
  L.A = take((size_t)n * n * (cold ? 8 : 16));
  L.LU = take((size_t)n * n * (cold ? 8 : 16));
  L.xJ = cold ? 0 : take((size_t)vn * 16);
  L.dinv = take((size_t)vn * 16);
  L.ipiv = take(64);  // row permutation and its inverse, one byte per row
  L.vec = take((size_t)(cold ? HC_NCVEC - HC_NCVEC_COLD : HC_NCVEC) * vn * 16);
  L.rvec = take((size_t)(cold ? HC_NRVEC - HC_NRVEC_COLD : HC_NRVEC) * vn * 8);
  L.cvec = L.crvec = L.cxj = L.cA = L.cLU = -1;
  if (cold) {
    L.cA = L.cold;
    L.cold += (int)up16((size_t)n * n * 16);
    L.cLU = L.cold;
    L.cold += (int)up16((size_t)n * n * 16);
    L.cvec = L.cold;
    L.cold += (int)up16((size_t)HC_NCVEC_COLD * vn * 16);
    L.crvec = L.cold;
    L.cold += (int)up16((size_t)HC_NRVEC_COLD * vn * 8);
    L.cxj = L.cold;
    L.cold += (int)up16((size_t)vn * 16);
  }
  L.v32 = take((size_t)4 * vn * 8);
  L.tor = tor_n > 0 ? take((size_t)tor_n * (16 + 8 + 8)) : 0;
  L.tor_n = tor_n;
  L.vn = vn;
  L.bytes = (int)off;
  return L;
}

// Device copy of a compiled program: every array 16-byte aligned and padded to 16 bytes,
// appended to `blob`; bind_program turns the offsets into pointers once the blob is on the device.
struct ProgOffsets {
  size_t mdef, lev, c64, c32, mono, jcode, rows[2][3];
};

ProgOffsets pack_program(const HostProg& P, std::vector<char>& blob) {
  auto put = [&](const void* src, size_t bytes) {
    size_t o = (blob.size() + 15) & ~(size_t)15;
    blob.resize(o + ((bytes + 15) & ~(size_t)15), 0);
    if (bytes) memcpy(blob.data() + o, src, bytes);
    return o;
  };
  ProgOffsets o;
  o.mdef = put(P.mdef.data(), P.mdef.size() * sizeof(int2));
  o.lev = put(P.lev.data(), P.lev.size() * sizeof(int));
  o.c64 = put(P.vcoef64.data(), P.vcoef64.size() * sizeof(double2));
  o.c32 = put(P.vcoef32.data(), P.vcoef32.size() * sizeof(float2));
  o.mono = put(P.vmono.data(), P.vmono.size() * sizeof(uint16_t));
  o.jcode = put(P.jcode.data(), P.jcode.size() * sizeof(uint32_t));
  const HostProg::Rows* rows[2] = {&P.val, &P.jac};
  for (int q = 0; q < 2; ++q) {
    o.rows[q][0] = put(rows[q]->seg.data(), rows[q]->seg.size() * sizeof(int4));
    o.rows[q][1] = put(rows[q]->lane_seg.data(), rows[q]->lane_seg.size() * sizeof(int));
    o.rows[q][2] = put(rows[q]->row_slot.data(), rows[q]->row_slot.size() * sizeof(int));
  }
  return o;
}

DevProg bind_program(const HostProg& P, const ProgOffsets& o, const char* base, double gamma_re, double gamma_im) {
  DevProg D{};
  D.n = P.n;
  D.M = P.M;
  D.nlev = P.nlev;
  D.top = P.top;
  D.mdef = (const int2*)(base + o.mdef);
  D.lev = (const int*)(base + o.lev);
  D.vcoef64 = (const double2*)(base + o.c64);
  D.vcoef32 = (const float2*)(base + o.c32);
  D.vmono = (const uint16_t*)(base + o.mono);
  D.jcode = (const uint32_t*)(base + o.jcode);
  const HostProg::Rows* rows[2] = {&P.val, &P.jac};
  DevRows* drows[2] = {&D.val, &D.jac};
  for (int q = 0; q < 2; ++q) {
    DevRows& X = *drows[q];
    X.nrows = rows[q]->nrows;
    X.nterms = q == 0 ? (int)P.vcoef64.size() : (int)P.jcode.size();
    X.nslots = rows[q]->nslots;
    X.nseg = (int)rows[q]->seg.size();
    X.seg = (const int4*)(base + o.rows[q][0]);
    X.lane_seg = (const int*)(base + o.rows[q][1]);
    X.row_slot = (const int*)(base + o.rows[q][2]);
  }
  D.gamma_re = gamma_re;
  D.gamma_im = gamma_im;
  return D;
}

}  // namespace

struct hc_handle {
  hc_options opts;
  cudaStream_t stream = nullptr;
  int device = 0, num_sms = 0;
  std::string err;
  // program
  HostProg prog;
  bool has_prog = false;
  char* d_prog = nullptr;
  size_t d_prog_bytes = 0;
  DevProg dprog{};
  WarpLayout layout{};
  WarpLayout layout_cold{};  // mixed precision: rare FP64 areas in d_cold
  char* d_cold = nullptr;
  size_t cold_cap = 0;
  int last_warp_bytes = 0, last_table_bytes = 0;
  // buffers
  double2* d_starts = nullptr;
  hc_path_result* d_res = nullptr;
  double2* d_sol = nullptr;
  double* d_val = nullptr;
  double2* d_last = nullptr;
  int64_t cap_paths = 0, cap_vec = 0;
  unsigned long long* d_counter = nullptr;  // [queue head + HC_NSTATS counters]
  int* h_cancel = nullptr;                  // mapped host memory
  int* d_cancel = nullptr;
  double time_limit = 0;                    // seconds per host tracking call (0 = none)
  std::chrono::steady_clock::time_point deadline{};
  bool timed_out = false;
  double stats[HC_NSTATS + HC_NPHASE] = {0};
  StepModel* d_model = nullptr;  // learned step proposal (hc_set_step_model)
  // batch of homotopies (hc_set_batch): programs, instance tables per precision, work units
  bool has_batch = false;
  char* d_bprog = nullptr;
  size_t d_bprog_bytes = 0;
  BatchInstance* d_binst[2] = {nullptr, nullptr};  // [precision]
  BatchUnit* d_bunits = nullptr;
  int bninst = 0, bnunits = 0;
  int btbytes[2] = {0, 0}, bwstride[2] = {0, 0};
  size_t bunits_cap = 0;
  // launch plan by n (hc_set_batch_launch, hc_autotune_batch): paths per work unit (0: one per
  // warp of a CTA) and the staging of mixed-precision instances (0/2: FP64 value coefficients via
  // L1/L2 and the rare FP64 areas in d_bcold; 1: every table in shared memory)
  int32_t bunit_paths[33] = {0};
  int32_t bstaging[33] = {0};
  // host copies of every instance's tables for re-planning: [0] FP64, [1] mixed with everything
  // in shared memory, [2] mixed with global slices; estimated cost of one path
  std::vector<BatchInstance> bhost[3];
  std::vector<double> bcost;
  int bcold = 0;  // bytes per warp of the mixed batch's global slices (0: none)
  char* d_bcold = nullptr;
  size_t bcold_cap = 0;
  int64_t btotal_paths = 0, btotal_vec = 0;
  // CUDA graph of the batch launch, re-recorded when its key changes
  cudaGraphExec_t bgraph = nullptr;
  const void* bgraph_key[3] = {nullptr, nullptr, nullptr};
  int bgraph_endgame = -1, bgraph_blocks = 0, bgraph_wpc = 0;
  unsigned long long bgraph_gen = 0;
  unsigned long long generation = 1;  // bumped whenever options, model or batch change
  std::vector<int64_t> bpath_off, bvec_off, bnpaths;  // host copies of the batch's instance offsets
  std::vector<int> bn;
  // jump check of the host entry points (learned step control)
  int64_t* d_plist = nullptr;
  size_t plist_cap = 0;
  BatchUnit* d_runits = nullptr;
  size_t runits_cap = 0;
  double retracked = 0;     // paths re-tracked with plain step control by the last host call
  bool stats_on_host = false;  // the last call was a host entry point: its counters are final
  int last_blocks = 0, last_wpc = 0, last_lockstep = 0;
  cudaStream_t last_stream = nullptr;
  // toric homotopy (hc_set_toric): weight rows in program term order, per-path arguments
  bool toric = false;
  int tor_rows = 0;
  double* d_tor_w = nullptr;
  size_t tor_w_cap = 0;
  char* d_tor_path = nullptr;  // [4 × npaths doubles: t1, t0, ω, μ][npaths int32 rows]
  size_t tor_path_cap = 0;
  // straight-line program of F (hc_set_slp): generated source and its kernels per precision
  bool slp = false;
  std::string slp_src;
  SlpModule slp_mod[2];
  bool slp_built[2] = {false, false};
  // parameter homotopy of a straight-line program (hc_set_slp_parameter_homotopy): p then q
  int slp_np = 0;
  double2* d_slp_pq = nullptr;
  int slp_pq_cap = 0;
  // step log
  double* d_log = nullptr;
  unsigned long long* d_log_count = nullptr;
  long long log_cap = 0, log_lo = 0, log_hi = 0;
};

// Makes the handle's device current for the duration of an entry point and restores the
// caller's device afterwards, so that handles on several devices can be used from one thread.
struct DeviceGuard {
  int prev = -1;
  explicit DeviceGuard(const hc_handle* h) {
    int cur = -1;
    if (cudaGetDevice(&cur) == cudaSuccess && cur != h->device && cudaSetDevice(h->device) == cudaSuccess) prev = cur;
  }
  ~DeviceGuard() {
    if (prev >= 0) cudaSetDevice(prev);
  }
  DeviceGuard(const DeviceGuard&) = delete;
  DeviceGuard& operator=(const DeviceGuard&) = delete;
};

static int fail(hc_handle* h, int code, const std::string& msg) {
  if (h) h->err = msg;
  std::lock_guard<std::mutex> g(g_err_mu);
  g_err = msg;
  return code;
}
int hc_library_fail(int code, const char* msg) { return fail(nullptr, code, msg); }

// Run time limit of the host entry points (hc_set_time_limit). The clock starts when a call
// begins; waiting for the stream polls it, and at the deadline the handle's cancel flag is
// raised, so the kernel stops exactly as for hc_cancel: paths not yet finished report
// terminated_unknown, finished ones keep their results.
static void start_clock(hc_handle* h) {
  h->timed_out = false;
  *h->h_cancel = 0;
  if (h->time_limit > 0)
    h->deadline = std::chrono::steady_clock::now() +
                  std::chrono::duration_cast<std::chrono::steady_clock::duration>(
                      std::chrono::duration<double>(h->time_limit));
}
static cudaError_t wait_stream(hc_handle* h) {
  if (!(h->time_limit > 0)) return cudaStreamSynchronize(h->stream);
  while (true) {
    cudaError_t e = cudaStreamQuery(h->stream);
    if (e != cudaErrorNotReady) return e;
    if (!h->timed_out && std::chrono::steady_clock::now() >= h->deadline) {
      h->timed_out = true;
      __atomic_store_n(h->h_cancel, 1, __ATOMIC_SEQ_CST);
    }
    std::this_thread::sleep_for(std::chrono::microseconds(50));
  }
}
// status of a host call whose kernel was stopped by hc_cancel or by the time limit
static int stopped(hc_handle* h, const char* where) {
  if (h->timed_out) return fail(h, HC_ERR_TIMEOUT, std::string(where) + ": time limit reached");
  return fail(h, HC_ERR_CANCELLED, std::string(where) + ": cancelled");
}
static int cuda_fail(hc_handle* h, cudaError_t e, const char* where) {
  return fail(h, HC_ERR_CUDA, std::string(where) + ": " + cudaGetErrorString(e));
}
#define CK(call)                                         \
  do {                                                   \
    cudaError_t _e = (call);                             \
    if (_e != cudaSuccess) return cuda_fail(h, _e, #call); \
  } while (0)

extern "C" {

int hc_default_options(hc_options* o) {
  if (!o) return fail(nullptr, HC_ERR_INVALID_ARG, "hc_default_options: null pointer");
  memset(o, 0, sizeof(*o));
  o->max_steps = 10000;
  o->extended_precision = 1;
  o->max_step_size = INFINITY;
  o->max_initial_step_size = INFINITY;
  o->min_step_size = 1e-48;
  o->min_rel_step_size = 0.0;
  o->terminate_cond = 1e13;
  o->a = 0.125;
  o->beta_a = 1.0;
  o->beta_omega_p = 3.0;
  o->beta_tau = 0.4;
  o->strict_beta_tau = 0.3;
  o->min_newton_iters = 2;
  o->max_endgame_steps = 2000;
  o->max_endgame_extended_steps = 400;
  o->max_winding_number = 6;
  o->zero_is_at_infinity = 0;
  o->at_infinity_check = 1;
  o->only_nonsingular = 0;
  o->refine_steps = 3;
  o->endgame_start = 0.1;
  o->min_cond = 1e6;
  o->min_cond_growth = 1e4;
  o->min_coord_growth = 100.0;
  o->singular_min_accuracy = 1e-6;
  o->val_finite_tol = 0.05;
  o->val_at_infinity_tol = 0.01;
  o->sing_cond = 1e14;
  o->sing_accuracy = 1e-12;
  o->scaling_threshold = -30.0;
  o->precision = HC_PREC_FP64;
  o->step_control = HC_STEP_PLAIN;
  o->warps_per_cta = 0;
  o->ctas_per_sm = 0;
  o->lockstep = -1;
  o->reserved = 0;
  return HC_OK;
}

// the GPU-side knobs of hc_options (the tracker parameters are the caller's to choose)
static const char* invalid_knob(const hc_options* o) {
  if (o->warps_per_cta < 0 || o->warps_per_cta > HC_MAX_WARPS) return "warps_per_cta must lie in [0, 16]";
  if (o->ctas_per_sm < 0) return "ctas_per_sm must be >= 0";
  if (o->precision != HC_PREC_FP64 && o->precision != HC_PREC_MIXED) return "unknown precision";
  if (o->step_control != HC_STEP_PLAIN && o->step_control != HC_STEP_LEARNED && o->step_control != HC_STEP_EXPLORE)
    return "unknown step control";
  if (o->lockstep < -1 || o->lockstep > 3) return "lockstep must be -1, 0, 1, 2 or 3";
  return nullptr;
}

int hc_create(const hc_options* opts, hc_handle** out) {
  if (!out) return fail(nullptr, HC_ERR_INVALID_ARG, "hc_create: null output pointer");
  *out = nullptr;
  if (opts && invalid_knob(opts)) return fail(nullptr, HC_ERR_INVALID_ARG, std::string("hc_create: ") + invalid_knob(opts));
  hc_handle* h = new hc_handle();
  if (opts)
    h->opts = *opts;
  else
    hc_default_options(&h->opts);
  cudaError_t e = cudaGetDevice(&h->device);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&h->num_sms, cudaDevAttrMultiProcessorCount, h->device);
  if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking);
  if (e == cudaSuccess) e = cudaMalloc(&h->d_counter, (1 + HC_NSTATS + HC_NPHASE) * sizeof(unsigned long long));
  if (e == cudaSuccess) e = cudaHostAlloc(&h->h_cancel, sizeof(int), cudaHostAllocMapped);
  if (e == cudaSuccess) {
    *h->h_cancel = 0;
    e = cudaHostGetDevicePointer(&h->d_cancel, h->h_cancel, 0);
  }
  if (e != cudaSuccess) {
    int rc = cuda_fail(nullptr, e, "hc_create");
    hc_destroy(h);
    return rc;
  }
  *out = h;
  return HC_OK;
}

int hc_create_on_device(const hc_options* opts, int device, hc_handle** out) {
  int count = 0, cur = -1;
  cudaError_t e = cudaGetDeviceCount(&count);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "hc_create_on_device");
  if (device < 0 || device >= count) return fail(nullptr, HC_ERR_INVALID_ARG, "hc_create_on_device: no such device");
  e = cudaGetDevice(&cur);
  if (e == cudaSuccess) e = cudaSetDevice(device);
  if (e != cudaSuccess) return cuda_fail(nullptr, e, "hc_create_on_device");
  int rc = hc_create(opts, out);
  cudaSetDevice(cur);
  return rc;
}

void hc_destroy(hc_handle* h) {
  if (!h) return;
  DeviceGuard dg(h);
  if (h->stream) cudaStreamSynchronize(h->stream);
  cudaFree(h->d_prog);
  cudaFree(h->d_starts);
  cudaFree(h->d_res);
  cudaFree(h->d_sol);
  cudaFree(h->d_val);
  cudaFree(h->d_last);
  cudaFree(h->d_counter);
  cudaFree(h->d_cold);
  cudaFree(h->d_slp_pq);
  cudaFree(h->d_model);
  cudaFree(h->d_bprog);
  cudaFree(h->d_binst[0]);
  cudaFree(h->d_binst[1]);
  cudaFree(h->d_bunits);
  cudaFree(h->d_bcold);
  cudaFree(h->d_plist);
  cudaFree(h->d_runits);
  cudaFree(h->d_tor_w);
  cudaFree(h->d_tor_path);
  if (h->bgraph) cudaGraphExecDestroy(h->bgraph);
  cudaFree(h->d_log);
  cudaFree(h->d_log_count);
  if (h->h_cancel) cudaFreeHost(h->h_cancel);
  if (h->stream) cudaStreamDestroy(h->stream);
  delete h;
}

int hc_set_options(hc_handle* h, const hc_options* opts) {
  if (!h || !opts) return fail(h, HC_ERR_INVALID_ARG, "hc_set_options: null pointer");
  if (invalid_knob(opts)) return fail(h, HC_ERR_INVALID_ARG, std::string("hc_set_options: ") + invalid_knob(opts));
  h->opts = *opts;
  ++h->generation;
  return HC_OK;
}

int hc_set_homotopy(hc_handle* h, int n, int nG, const int32_t* G_eq, const int32_t* G_exps,
                    const double* G_coef, int nF, const int32_t* F_eq, const int32_t* F_exps,
                    const double* F_coef, double gamma_re, double gamma_im) {
  if (!h) return fail(h, HC_ERR_INVALID_ARG, "hc_set_homotopy: null handle");
  DeviceGuard dg(h);
  if (n < 1 || n > 32) return fail(h, HC_ERR_UNSUPPORTED, "hc_set_homotopy: need 1 <= n <= 32");
  if (nG < 0 || nF < 0 || (nG > 0 && (!G_eq || !G_exps || !G_coef)) || (nF > 0 && (!F_eq || !F_exps || !F_coef)))
    return fail(h, HC_ERR_INVALID_ARG, "hc_set_homotopy: bad term table");
  if (!std::isfinite(gamma_re) || !std::isfinite(gamma_im))
    return fail(h, HC_ERR_INVALID_ARG, "hc_set_homotopy: gamma must be finite");
  HostProg P;
  std::string err;
  int rc = build_program(n, nG, G_eq, G_exps, G_coef, nF, F_eq, F_exps, F_coef, P, err);
  if (rc != HC_OK) return fail(h, rc, "hc_set_homotopy: " + err);
  WarpLayout L = make_warp_layout(P);
  TableLayout T = make_table_layout(P, HC_PREC_MIXED);
  if ((size_t)T.bytes + L.bytes > 220 * 1024)
    return fail(h, HC_ERR_TOO_LARGE, "hc_set_homotopy: tables plus one path's working set exceed shared memory");
  std::vector<char> blob;
  ProgOffsets po = pack_program(P, blob);
  if (h->d_prog_bytes < blob.size()) {
    cudaFree(h->d_prog);
    h->d_prog = nullptr;
    h->d_prog_bytes = 0;
    CK(cudaMalloc(&h->d_prog, blob.size()));
    h->d_prog_bytes = blob.size();
  }
  CK(cudaMemcpyAsync(h->d_prog, blob.data(), blob.size(), cudaMemcpyHostToDevice, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  DevProg D = bind_program(P, po, h->d_prog, gamma_re, gamma_im);
  h->layout_cold = make_warp_layout(P, 0, true);
  h->prog = std::move(P);
  h->dprog = D;
  h->layout = L;
  h->has_prog = true;
  h->toric = false;
  h->slp = false;
  h->slp_np = 0;
  return HC_OK;
}

// the kernel of the handle's straight-line program for `precision`, compiled on first use
static int ensure_slp(hc_handle* h, int precision) {
  const int q = precision == HC_PREC_MIXED ? 1 : 0;
  if (h->slp_built[q]) return HC_OK;
  std::string err;
  int rc = slp_build(h->slp_src, q == 1, h->slp_mod[q], err);
  if (rc != HC_OK) return fail(h, rc, "hc_set_slp: " + err);
  h->slp_built[q] = true;
  return HC_OK;
}

int hc_set_slp(hc_handle* h, const hc_slp* F, const int32_t* degrees, const double* scaling, double gamma_re,
               double gamma_im) {
  if (!h) return fail(h, HC_ERR_INVALID_ARG, "hc_set_slp: null handle");
  DeviceGuard dg(h);
  if (!std::isfinite(gamma_re) || !std::isfinite(gamma_im))
    return fail(h, HC_ERR_INVALID_ARG, "hc_set_slp: gamma must be finite");
  SlpProgram S;
  std::string err;
  int rc = slp_validate(F, degrees, scaling, 0, 0, S, err);
  if (rc != HC_OK) return fail(h, rc, "hc_set_slp: " + err);
  const int n = S.n;
  // the start system's term table (s_i x_i^{D_i} - s_i) carries n, γ and the per-path layout;
  // F itself is evaluated by the generated code
  std::vector<int32_t> Geq, Gexp;
  std::vector<double> Gcf;
  for (int i = 0; i < n; ++i) {
    for (int q = 0; q < 2; ++q) {
      Geq.push_back(i);
      for (int j = 0; j < n; ++j) Gexp.push_back(q == 0 && j == i ? S.degrees[i] : 0);
      Gcf.push_back(q == 0 ? S.scaling[i] : -S.scaling[i]);
      Gcf.push_back(0.0);
    }
  }
  rc = hc_set_homotopy(h, n, (int)Geq.size(), Geq.data(), Gexp.data(), Gcf.data(), 0, nullptr, nullptr, nullptr,
                       gamma_re, gamma_im);
  if (rc != HC_OK) return rc;
  h->slp_src = slp_codegen(S);
  h->slp_built[0] = h->slp_built[1] = false;
  h->slp = true;
  rc = ensure_slp(h, h->opts.precision);
  if (rc != HC_OK) h->slp = false;
  return rc;
}

static void copy_source(const std::string& src, char* out, int64_t capacity, int64_t* length) {
  if (length) *length = (int64_t)src.size();
  if (out && capacity > 0) {
    size_t m = std::min<size_t>((size_t)capacity - 1, src.size());
    memcpy(out, src.data(), m);
    out[m] = 0;
  }
}

int hc_slp_source(const hc_slp* F, const int32_t* degrees, const double* scaling, char* out, int64_t capacity,
                  int64_t* length) {
  SlpProgram S;
  std::string err;
  int rc = slp_validate(F, degrees, scaling, 0, 0, S, err);
  if (rc != HC_OK) return fail(nullptr, rc, "hc_slp_source: " + err);
  copy_source(slp_codegen(S), out, capacity, length);
  return HC_OK;
}

int hc_slp_parameter_source(const hc_slp* F, int nparameters, int32_t parameters_offset, char* out,
                            int64_t capacity, int64_t* length) {
  if (nparameters < 1) return fail(nullptr, HC_ERR_INVALID_ARG, "hc_slp_parameter_source: need nparameters >= 1");
  SlpProgram S;
  std::string err;
  int rc = slp_validate(F, nullptr, nullptr, nparameters, parameters_offset, S, err);
  if (rc != HC_OK) return fail(nullptr, rc, "hc_slp_parameter_source: " + err);
  copy_source(slp_codegen(S), out, capacity, length);
  return HC_OK;
}

int hc_set_slp_parameters(hc_handle* h, const double* p, const double* q) {
  if (!h) return fail(h, HC_ERR_INVALID_ARG, "hc_set_slp_parameters: null handle");
  DeviceGuard dg(h);
  if (!h->slp || h->slp_np < 1)
    return fail(h, HC_ERR_NO_SYSTEM, "hc_set_slp_parameters: call hc_set_slp_parameter_homotopy first");
  if (!p || !q) return fail(h, HC_ERR_INVALID_ARG, "hc_set_slp_parameters: null parameters");
  const int m = h->slp_np;
  for (int k = 0; k < 2 * m; ++k)
    if (!std::isfinite(p[k]) || !std::isfinite(q[k]))
      return fail(h, HC_ERR_INVALID_ARG, "hc_set_slp_parameters: parameters must be finite");
  std::vector<double2> pq(2 * (size_t)m);
  for (int k = 0; k < m; ++k) {
    pq[k] = make_double2(p[2 * k], p[2 * k + 1]);
    pq[m + k] = make_double2(q[2 * k], q[2 * k + 1]);
  }
  CK(cudaStreamSynchronize(h->stream));  // a running launch reads the old values
  if (h->slp_pq_cap < 2 * m) {
    cudaFree(h->d_slp_pq);
    h->d_slp_pq = nullptr;
    h->slp_pq_cap = 0;
    CK(cudaMalloc(&h->d_slp_pq, pq.size() * sizeof(double2)));
    h->slp_pq_cap = 2 * m;
    ++h->generation;
  }
  CK(cudaMemcpyAsync(h->d_slp_pq, pq.data(), pq.size() * sizeof(double2), cudaMemcpyHostToDevice, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return HC_OK;
}

int hc_set_slp_parameter_homotopy(hc_handle* h, const hc_slp* F, int nparameters, int32_t parameters_offset,
                                  const double* p, const double* q) {
  if (!h) return fail(h, HC_ERR_INVALID_ARG, "hc_set_slp_parameter_homotopy: null handle");
  DeviceGuard dg(h);
  if (nparameters < 1) return fail(h, HC_ERR_INVALID_ARG, "hc_set_slp_parameter_homotopy: need nparameters >= 1");
  if (!p || !q) return fail(h, HC_ERR_INVALID_ARG, "hc_set_slp_parameter_homotopy: null parameters");
  SlpProgram S;
  std::string err;
  int rc = slp_validate(F, nullptr, nullptr, nparameters, parameters_offset, S, err);
  if (rc != HC_OK) return fail(h, rc, "hc_set_slp_parameter_homotopy: " + err);
  const int n = S.n;
  // a placeholder term table (x_i - 1) carries n and the per-path layout; H is evaluated by the
  // generated code alone
  std::vector<int32_t> Geq, Gexp;
  std::vector<double> Gcf;
  for (int i = 0; i < n; ++i)
    for (int k = 0; k < 2; ++k) {
      Geq.push_back(i);
      for (int j = 0; j < n; ++j) Gexp.push_back(k == 0 && j == i ? 1 : 0);
      Gcf.push_back(k == 0 ? 1.0 : -1.0);
      Gcf.push_back(0.0);
    }
  rc = hc_set_homotopy(h, n, (int)Geq.size(), Geq.data(), Gexp.data(), Gcf.data(), 0, nullptr, nullptr, nullptr,
                       1.0, 0.0);
  if (rc != HC_OK) return rc;
  h->slp_src = slp_codegen(S);
  h->slp_built[0] = h->slp_built[1] = false;
  h->slp = true;
  h->slp_np = nparameters;
  rc = hc_set_slp_parameters(h, p, q);
  if (rc == HC_OK) rc = ensure_slp(h, h->opts.precision);
  if (rc != HC_OK) {
    h->slp = false;
    h->slp_np = 0;
  }
  return rc;
}

// handle-owned device buffers for `npaths` results and `nvec` complex vector elements
static int ensure_capacity_v(hc_handle* h, int64_t npaths, int64_t nvec) {
  if (npaths <= h->cap_paths && nvec <= h->cap_vec) return HC_OK;
  cudaFree(h->d_starts);
  cudaFree(h->d_res);
  cudaFree(h->d_sol);
  cudaFree(h->d_val);
  cudaFree(h->d_last);
  h->d_starts = nullptr;
  h->d_res = nullptr;
  h->d_sol = nullptr;
  h->d_val = nullptr;
  h->d_last = nullptr;
  npaths = std::max(npaths, h->cap_paths);
  nvec = std::max(nvec, h->cap_vec);
  h->cap_paths = h->cap_vec = 0;
  size_t nv = (size_t)nvec;
  CK(cudaMalloc(&h->d_starts, nv * sizeof(double2)));
  CK(cudaMalloc(&h->d_res, (size_t)npaths * sizeof(hc_path_result)));
  CK(cudaMalloc(&h->d_sol, nv * sizeof(double2)));
  CK(cudaMalloc(&h->d_val, nv * sizeof(double)));
  CK(cudaMalloc(&h->d_last, nv * sizeof(double2)));
  h->cap_paths = npaths;
  h->cap_vec = nvec;
  return HC_OK;
}
static int ensure_capacity(hc_handle* h, int64_t npaths, int n) { return ensure_capacity_v(h, npaths, npaths * n); }

// per-path overrides and the toric weights of a plain-tracker launch (all optional)
struct PathArgs {
  const double *t1 = nullptr, *t0 = nullptr, *omega = nullptr, *mu = nullptr;
  const double* tor_w = nullptr;
  const int32_t* tor_row = nullptr;
};
static int track_device_impl(hc_handle* h, int64_t npaths, const double* d_starts, int endgame, double t1_re,
                             double t1_im, double t0_re, double t0_im, hc_path_result* d_results,
                             double* d_solutions, double* d_valuation, double* d_last, cudaStream_t s,
                             const hc_options& O, const int64_t* d_path_list, const PathArgs& pa = PathArgs());

// Warps per CTA when the options leave it open: as many as fit, except that mixed-precision
// launches use 4 rather than 5..7 (one CTA per SM; with 5..7 warps some of the SM's four
// schedulers run two warps and the others one, and the FP32-phase-heavy mixed tracker lost
// 5% at 5 warps against 4 on 10 dense cubics, while the FP64 tracker gained 10%).
// Lockstep scheduling of a CTA's warps. Measured on one GB300 (paths/s; per-warp, then lockstep
// of the CTA (1), of the warps of a sub-partition (2), of two sub-partitions (3)):
//   10 dense cubics, mixed + learned, 8 warps   34.5k | 44.0k  44.5k  47.5k
//   10 dense cubics, mixed + plain, 8 warps     21.2k | 25.6k  27.6k  28.7k
//   11 dense cubics, mixed + learned, 6 warps   25.9k | 24.4k  27.8k  26.2k
//   8 sparse quartics, FP64 + learned, 8 warps  16.1k | 23.2k  19.5k  22.2k
//   7 dense cubics, FP64 + plain, 8 warps       22.8k | 28.4k
//   2,000 uneven instances (batch), mixed + learned, 8 warps  61.6k | 89.2k  73.9k  85.6k
// The warps share the instruction cache when they run the same code; with 4 or 5 warps the
// waits cost more than that gains.
// With up to 16 warps per CTA (CTA-wide lockstep; 8 warps → the most that fit): 6 dense cubics,
// mixed + plain, 100k → 115k (16 warps); 7 dense cubics 72k → 90k (16); 8 dense cubics 58.8k →
// 68.6k (13); 8 sparse quartics, mixed + learned, 20.4k → 22.2k (12), FP64 + learned 23.2k →
// 23.6k (11). On those smaller programs the CTA-wide barrier beats the groups of four (8 dense
// cubics at 8 warps 58.8k vs 54.7k, 6 dense cubics 100k vs 74k); the groups win on the 10 dense
// cubics (2,880 value terms).
static int lockstep_for(const hc_options& O, int wpc, bool batch = false, long long value_terms = 0) {
  if (O.lockstep >= 0) return O.lockstep;
  if (batch) return wpc >= 8 ? 1 : 0;
  if (wpc >= 8) return O.precision == HC_PREC_MIXED && value_terms >= 2000 ? 3 : 1;
  return O.precision == HC_PREC_MIXED && wpc >= 6 ? 2 : 0;
}

// Mixed precision: 5 warps per CTA (two sub-partitions with two warps, two with one) measured
// 5% below 4 on 10 dense cubics; 6 warps measured 16% above 4 on 11 dense cubics.
static int balanced_warps(int wpc, int precision) {
  if (precision == HC_PREC_MIXED && wpc == 5) return 4;
  return wpc;
}

int hc_track_device(hc_handle* h, int64_t npaths, const double* d_starts, int endgame, double t1_re,
                    double t1_im, double t0_re, double t0_im, hc_path_result* d_results, double* d_solutions,
                    double* d_valuation, double* d_last, void* stream) {
  if (!h) return fail(h, HC_ERR_INVALID_ARG, "hc_track_device: null handle");
  DeviceGuard dg(h);
  if (!h->has_prog) return fail(h, HC_ERR_NO_SYSTEM, "hc_track_device: call hc_set_homotopy first");
  if (h->toric) return fail(h, HC_ERR_INVALID_ARG, "hc_track_device: the handle holds a toric homotopy (hc_track_toric)");
  if (npaths < 0) return fail(h, HC_ERR_INVALID_ARG, "hc_track_device: npaths < 0");
  if (npaths == 0) return HC_OK;
  if (!d_starts || !d_results || !d_solutions) return fail(h, HC_ERR_INVALID_ARG, "hc_track_device: null buffer");
  if (h->opts.step_control == HC_STEP_LEARNED && !h->d_model)
    return fail(h, HC_ERR_INVALID_ARG, "hc_track_device: learned step control needs hc_set_step_model");
  cudaStream_t s = stream ? (cudaStream_t)stream : h->stream;
  h->stats_on_host = false;
  return track_device_impl(h, npaths, d_starts, endgame, t1_re, t1_im, t0_re, t0_im, d_results, d_solutions,
                           d_valuation, d_last, s, h->opts, nullptr);
}

// one launch of the tracking kernel with options O; with d_path_list, queue item i tracks path
// d_path_list[i] in place (results and endpoints at that path's own index)
static int track_device_impl(hc_handle* h, int64_t npaths, const double* d_starts, int endgame, double t1_re,
                             double t1_im, double t0_re, double t0_im, hc_path_result* d_results,
                             double* d_solutions, double* d_valuation, double* d_last, cudaStream_t s,
                             const hc_options& O, const int64_t* d_path_list, const PathArgs& pa) {
  Launch la{};
  la.P = h->dprog;
  la.O = O;
  // mixed precision on a straight-line homotopy: FP64 value coefficients read from global
  // memory and the rare FP64 areas in the handle's cold buffer, so twice the warps fit per SM
  const bool cold = O.precision == HC_PREC_MIXED && !h->toric;
  la.L = cold ? h->layout_cold : h->layout;
  la.T = make_table_layout(h->prog, O.precision, cold);
  la.npaths = npaths;
  la.starts = (const double2*)d_starts;
  la.res = d_results;
  la.sol = (double2*)d_solutions;
  la.val = d_valuation;
  la.last = (double2*)d_last;
  la.mode = endgame ? 1 : 0;
  la.t1_re = t1_re;
  la.t1_im = t1_im;
  la.t0_re = t0_re;
  la.t0_im = t0_im;
  la.counter = h->d_counter;
  la.cancel = h->d_cancel;
  la.stats = h->d_counter + 1;
  la.log = h->log_cap > 0 ? h->d_log : nullptr;
  la.log_count = h->d_log_count;
  la.log_cap = h->log_cap;
  la.log_lo = h->log_lo;
  la.log_hi = h->log_hi;
  la.model = O.step_control == HC_STEP_LEARNED ? h->d_model : nullptr;
  la.slp_pq = h->slp && h->slp_np > 0 ? h->d_slp_pq : nullptr;
  la.phase = h->d_counter + 1 + HC_NSTATS;
  la.path_list = d_path_list;
  la.path_t1 = pa.t1;
  la.path_t0 = pa.t0;
  la.path_omega = pa.omega;
  la.path_mu = pa.mu;
  la.tor_w = pa.tor_w;
  la.tor_row = pa.tor_row;
  if (la.log) CK(cudaMemsetAsync(h->d_log_count, 0, sizeof(unsigned long long), s));
  // warps per CTA: as many as fit next to one copy of the tables (capped at HC_MAX_WARPS)
  const size_t smem_cap = 227 * 1024;
  int wpc = O.warps_per_cta;
  if (wpc <= 0) {
    wpc = (int)std::min<size_t>(HC_MAX_WARPS, (smem_cap - la.T.bytes) / la.L.bytes);
    wpc = std::max(wpc, 1);
    wpc = balanced_warps(wpc, O.precision);
  }
  size_t smem = (size_t)la.T.bytes + (size_t)wpc * la.L.bytes;
  while (wpc > 1 && smem > smem_cap) {
    --wpc;
    smem = (size_t)la.T.bytes + (size_t)wpc * la.L.bytes;
  }
  la.lockstep = lockstep_for(O, wpc, false, h->prog.val_terms);
  h->last_lockstep = la.lockstep;
  int bps = 0;
  cudaKernel_t jit = nullptr;  // the NVRTC kernel of a straight-line program
  if (h->slp) {
    int rc = ensure_slp(h, O.precision);
    if (rc != HC_OK) return rc;
    jit = h->slp_mod[O.precision == HC_PREC_MIXED ? 1 : 0].kernel;
    CK(cudaFuncSetAttribute((const void*)jit, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, (const void*)jit, 32 * wpc, smem));
  } else {
    CK(occupancy(O.precision, wpc, smem, &bps));
  }
  if (bps < 1) return fail(h, HC_ERR_TOO_LARGE, "hc_track_device: kernel does not fit on an SM");
  if (O.ctas_per_sm > 0) bps = std::min(bps, O.ctas_per_sm);
  int64_t want = ((int64_t)npaths + wpc - 1) / wpc;
  int blocks = (int)std::min<int64_t>((int64_t)bps * h->num_sms, want);
  if (cold) {
    // one slice per warp of the launch; grown only, allocated when a launch first needs more
    size_t need = (size_t)blocks * wpc * (size_t)la.L.cold;
    if (h->cold_cap < need) {
      CK(cudaStreamSynchronize(s));
      cudaFree(h->d_cold);
      h->d_cold = nullptr;
      h->cold_cap = 0;
      size_t cap = (size_t)bps * h->num_sms * wpc * (size_t)la.L.cold;  // the largest launch of this shape
      CK(cudaMalloc(&h->d_cold, std::max(cap, need)));
      h->cold_cap = std::max(cap, need);
    }
    la.cold = h->d_cold;
  }
  h->last_warp_bytes = la.L.bytes;
  h->last_table_bytes = la.T.bytes;
  // a cold layout keeps part of every warp's vectors, A and LU in the global slices: never
  // launch it without them
  if (la.L.cold > 0 && !la.cold) return fail(h, HC_ERR_CUDA, "track: cold layout without its global slices");
  CK(cudaMemsetAsync(h->d_counter, 0, (1 + HC_NSTATS + HC_NPHASE) * sizeof(unsigned long long), s));
  if (jit) {
    void* args[] = {(void*)&la};
    CK(cudaLaunchKernel((const void*)jit, dim3(blocks), dim3(32 * wpc), args, smem, s));
  } else {
    CK(launch_track(la, blocks, wpc, s));
  }
  h->last_blocks = blocks;
  h->last_wpc = wpc;
  h->last_stream = s;
  return HC_OK;
}

// Jump check of the host entry points with learned step control. A path that jumps onto
// another path ends at that path's solution: two nonsingular endpoints coincide. Returns the
// paths (indices into res/sol) whose nonsingular endpoints coincide with another's within
// rtol·max(‖x‖∞, 1). The candidates are swept in order of a fixed projection p(x) = Σ w·x
// (weights of absolute sum at most 1, all distinct) scaled by max(‖x‖∞, 1): coincident
// endpoints' keys differ by at most 2·rtol, and unlike a single coordinate the projection
// does not put every endpoint whose largest entry is that coordinate on the same key.
static std::vector<int64_t> coincident_paths(const hc_path_result* res, const double2* sol, int64_t npaths, int n,
                                             double rtol = 1e-8) {
  struct C {
    double key, norm;
    int64_t k;
  };
  std::vector<double> wt(2 * (size_t)n);
  for (int i = 0; i < 2 * n; ++i) {  // (0.5 .. 1) / (2n), signs alternating
    const double f = 0.6180339887498949 * (i + 1);
    wt[i] = (i & 1 ? -1.0 : 1.0) * (0.5 + 0.5 * (f - std::floor(f))) / (2.0 * n);
  }
  std::vector<C> c;
  c.reserve((size_t)npaths);
  for (int64_t k = 0; k < npaths; ++k) {
    if (res[k].return_code != 1 || res[k].singular) continue;  // EndgameTrackerCode success
    const double2* x = sol + k * n;
    double m = 0, p = 0;
    for (int i = 0; i < n; ++i) {
      m = std::max(m, std::max(std::fabs(x[i].x), std::fabs(x[i].y)));
      p += wt[2 * i] * x[i].x + wt[2 * i + 1] * x[i].y;
    }
    if (!std::isfinite(m)) continue;
    c.push_back({p / std::max(m, 1.0), m, k});
  }
  std::sort(c.begin(), c.end(), [](const C& a, const C& b) { return a.key < b.key; });
  std::vector<char> mark(npaths, 0);
  for (size_t a = 0; a < c.size(); ++a)
    for (size_t b = a + 1; b < c.size() && c[b].key - c[a].key <= 4 * rtol; ++b) {
      const double2* xa = sol + c[a].k * n;
      const double2* xb = sol + c[b].k * n;
      double tol = rtol * std::max(std::max(c[a].norm, c[b].norm), 1.0), d = 0;
      for (int i = 0; i < n && d <= tol; ++i) d = std::max(d, std::max(std::fabs(xa[i].x - xb[i].x), std::fabs(xa[i].y - xb[i].y)));
      if (d <= tol) mark[c[a].k] = mark[c[b].k] = 1;
    }
  std::vector<int64_t> out;
  for (int64_t k = 0; k < npaths; ++k)
    if (mark[k]) out.push_back(k);
  return out;
}

int hc_track(hc_handle* h, int64_t npaths, const double* starts, int endgame, double t1_re, double t1_im,
             double t0_re, double t0_im, hc_path_result* out_results, double* out_solutions, double* out_valuation,
             double* out_last) {
  if (!h) return fail(h, HC_ERR_INVALID_ARG, "hc_track: null handle");
  DeviceGuard dg(h);
  if (!h->has_prog) return fail(h, HC_ERR_NO_SYSTEM, "hc_track: call hc_set_homotopy first");
  if (h->toric) return fail(h, HC_ERR_INVALID_ARG, "hc_track: the handle holds a toric homotopy (hc_track_toric)");
  if (npaths < 0) return fail(h, HC_ERR_INVALID_ARG, "hc_track: npaths < 0");
  if (npaths == 0) return HC_OK;
  if (!starts || !out_results || !out_solutions) return fail(h, HC_ERR_INVALID_ARG, "hc_track: null buffer");
  int n = h->prog.n;
  int rc = ensure_capacity(h, npaths, n);
  if (rc != HC_OK) return rc;
  size_t nv = (size_t)npaths * n;
  start_clock(h);
  CK(cudaMemcpyAsync(h->d_starts, starts, nv * sizeof(double2), cudaMemcpyHostToDevice, h->stream));
  rc = hc_track_device(h, npaths, (const double*)h->d_starts, endgame, t1_re, t1_im, t0_re, t0_im, h->d_res,
                       (double*)h->d_sol, h->d_val, (double*)h->d_last, nullptr);
  if (rc != HC_OK) return rc;
  // copies into pageable host memory block the host until the kernel ends: poll the time
  // limit before them
  if (h->time_limit > 0) CK(wait_stream(h));
  CK(cudaMemcpyAsync(out_results, h->d_res, (size_t)npaths * sizeof(hc_path_result), cudaMemcpyDeviceToHost,
                     h->stream));
  CK(cudaMemcpyAsync(out_solutions, h->d_sol, nv * sizeof(double2), cudaMemcpyDeviceToHost, h->stream));
  if (out_valuation)
    CK(cudaMemcpyAsync(out_valuation, h->d_val, nv * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
  if (out_last) CK(cudaMemcpyAsync(out_last, h->d_last, nv * sizeof(double2), cudaMemcpyDeviceToHost, h->stream));
  unsigned long long st[HC_NSTATS + HC_NPHASE];
  CK(cudaMemcpyAsync(st, h->d_counter + 1, sizeof(st), cudaMemcpyDeviceToHost, h->stream));
  CK(wait_stream(h));
  for (int i = 0; i < HC_NSTATS + HC_NPHASE; ++i) h->stats[i] = (double)st[i];
  h->retracked = 0;
  h->stats_on_host = true;
  if (*h->h_cancel) return stopped(h, "hc_track");
  if (h->opts.step_control == HC_STEP_LEARNED && endgame) {
    // re-track the paths whose endpoints coincide with plain step control, in place
    std::vector<int64_t> idx = coincident_paths(out_results, (const double2*)out_solutions, npaths, n);
    if (!idx.empty()) {
      if (h->plist_cap < idx.size()) {
        cudaFree(h->d_plist);
        h->d_plist = nullptr;
        h->plist_cap = 0;
        CK(cudaMalloc(&h->d_plist, idx.size() * sizeof(int64_t)));
        h->plist_cap = idx.size();
      }
      CK(cudaMemcpyAsync(h->d_plist, idx.data(), idx.size() * sizeof(int64_t), cudaMemcpyHostToDevice, h->stream));
      hc_options O = h->opts;
      O.step_control = HC_STEP_PLAIN;
      rc = track_device_impl(h, (int64_t)idx.size(), (const double*)h->d_starts, endgame, t1_re, t1_im, t0_re,
                             t0_im, h->d_res, (double*)h->d_sol, h->d_val, (double*)h->d_last, h->stream, O,
                             h->d_plist);
      if (rc != HC_OK) return rc;
      if (h->time_limit > 0) CK(wait_stream(h));
      for (int64_t k : idx) {
        CK(cudaMemcpyAsync(out_results + k, h->d_res + k, sizeof(hc_path_result), cudaMemcpyDeviceToHost,
                           h->stream));
        CK(cudaMemcpyAsync(out_solutions + 2 * k * n, h->d_sol + k * n, n * sizeof(double2),
                           cudaMemcpyDeviceToHost, h->stream));
        if (out_valuation)
          CK(cudaMemcpyAsync(out_valuation + k * n, h->d_val + k * n, n * sizeof(double), cudaMemcpyDeviceToHost,
                             h->stream));
        if (out_last)
          CK(cudaMemcpyAsync(out_last + 2 * k * n, h->d_last + k * n, n * sizeof(double2), cudaMemcpyDeviceToHost,
                             h->stream));
      }
      CK(cudaMemcpyAsync(st, h->d_counter + 1, sizeof(st), cudaMemcpyDeviceToHost, h->stream));
      CK(wait_stream(h));
      for (int i = 0; i < HC_NSTATS + HC_NPHASE; ++i) h->stats[i] += (double)st[i];
      h->stats[0] -= (double)idx.size();  // paths: counted once
      h->retracked = (double)idx.size();
      if (*h->h_cancel) return stopped(h, "hc_track");
    }
  }
  return HC_OK;
}

int hc_set_step_log(hc_handle* h, int64_t capacity, int64_t path_lo, int64_t path_hi) {
  if (!h || capacity < 0 || path_lo < 0 || path_hi < path_lo)
    return fail(h, HC_ERR_INVALID_ARG, "hc_set_step_log: bad argument");
  DeviceGuard dg(h);
  if (capacity != h->log_cap) {
    cudaFree(h->d_log);
    h->d_log = nullptr;
    h->log_cap = 0;
    if (capacity > 0) CK(cudaMalloc(&h->d_log, (size_t)capacity * HC_LOG_FIELDS * sizeof(double)));
    if (!h->d_log_count) CK(cudaMalloc(&h->d_log_count, sizeof(unsigned long long)));
    h->log_cap = capacity;
  }
  h->log_lo = path_lo;
  h->log_hi = path_hi;
  return HC_OK;
}

int hc_get_step_log(hc_handle* h, double* out, int64_t max_records, int64_t* n_records) {
  if (!h || !n_records || max_records < 0 || (max_records > 0 && !out))
    return fail(h, HC_ERR_INVALID_ARG, "hc_get_step_log: bad argument");
  DeviceGuard dg(h);
  *n_records = 0;
  if (h->log_cap == 0) return HC_OK;
  unsigned long long cnt = 0;
  CK(cudaMemcpyAsync(&cnt, h->d_log_count, sizeof(cnt), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  int64_t m = std::min<int64_t>((int64_t)std::min<unsigned long long>(cnt, (unsigned long long)h->log_cap), max_records);
  if (m > 0) {
    CK(cudaMemcpyAsync(out, h->d_log, (size_t)m * HC_LOG_FIELDS * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
  }
  *n_records = (int64_t)cnt;
  return HC_OK;
}

static uint16_t to_bf16(float f) {  // round to nearest even; NaN stays NaN
  uint32_t u;
  std::memcpy(&u, &f, 4);
  if ((u & 0x7fffffffu) > 0x7f800000u) return (uint16_t)((u >> 16) | 0x40);
  u += 0x7fffu + ((u >> 16) & 1u);
  return (uint16_t)(u >> 16);
}

int hc_set_toric(hc_handle* h, int n, int nF, const int32_t* F_eq, const int32_t* F_exps, const double* F_coef,
                 int nrows, const double* weights) {
  if (!h) return fail(h, HC_ERR_INVALID_ARG, "hc_set_toric: null handle");
  DeviceGuard dg(h);
  if (n < 1 || n > 32) return fail(h, HC_ERR_UNSUPPORTED, "hc_set_toric: need 1 <= n <= 32");
  if (nF < 1 || !F_eq || !F_exps || !F_coef) return fail(h, HC_ERR_INVALID_ARG, "hc_set_toric: bad term table");
  if (nrows < 1 || !weights) return fail(h, HC_ERR_INVALID_ARG, "hc_set_toric: need at least one weight row");
  for (size_t k = 0; k < (size_t)nrows * nF; ++k)
    if (!(weights[k] >= 0.0) || !std::isfinite(weights[k]))
      return fail(h, HC_ERR_INVALID_ARG, "hc_set_toric: weights must be finite and non-negative");
  HostProg P;
  std::string err;
  int rc = build_program(n, 0, nullptr, nullptr, nullptr, nF, F_eq, F_exps, F_coef, P, err, true);
  if (rc != HC_OK) return fail(h, rc, "hc_set_toric: " + err);
  const int T = (int)P.vcoef64.size();
  WarpLayout L = make_warp_layout(P, T);
  TableLayout TL = make_table_layout(P, HC_PREC_FP64);
  if ((size_t)TL.bytes + L.bytes > 220 * 1024)
    return fail(h, HC_ERR_TOO_LARGE, "hc_set_toric: tables plus one path's working set exceed shared memory");
  // weight rows in program term order
  std::vector<double> w((size_t)nrows * T);
  for (int r = 0; r < nrows; ++r)
    for (int k = 0; k < T; ++k) w[(size_t)r * T + k] = weights[(size_t)r * nF + P.vorig[k]];
  std::vector<char> blob;
  ProgOffsets po = pack_program(P, blob);
  if (h->d_prog_bytes < blob.size()) {
    cudaFree(h->d_prog);
    h->d_prog = nullptr;
    h->d_prog_bytes = 0;
    CK(cudaMalloc(&h->d_prog, blob.size()));
    h->d_prog_bytes = blob.size();
  }
  if (h->tor_w_cap < w.size()) {
    cudaFree(h->d_tor_w);
    h->d_tor_w = nullptr;
    h->tor_w_cap = 0;
    CK(cudaMalloc(&h->d_tor_w, w.size() * sizeof(double)));
    h->tor_w_cap = w.size();
  }
  CK(cudaMemcpyAsync(h->d_prog, blob.data(), blob.size(), cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemcpyAsync(h->d_tor_w, w.data(), w.size() * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  DevProg D = bind_program(P, po, h->d_prog, 1.0, 0.0);
  h->prog = std::move(P);
  h->dprog = D;
  h->layout = L;
  h->has_prog = true;
  h->toric = true;
  h->slp = false;
  h->slp_np = 0;
  h->tor_rows = nrows;
  return HC_OK;
}

int hc_track_toric(hc_handle* h, int64_t npaths, const double* starts, const int32_t* rows, const double* t1,
                   const double* t0, const double* omega, const double* mu, hc_path_result* out_results,
                   double* out_solutions) {
  if (!h) return fail(h, HC_ERR_INVALID_ARG, "hc_track_toric: null handle");
  DeviceGuard dg(h);
  if (!h->has_prog || !h->toric) return fail(h, HC_ERR_NO_SYSTEM, "hc_track_toric: call hc_set_toric first");
  if (npaths < 0) return fail(h, HC_ERR_INVALID_ARG, "hc_track_toric: npaths < 0");
  if (npaths == 0) return HC_OK;
  if (!starts || !rows || !t1 || !t0 || !out_results || !out_solutions)
    return fail(h, HC_ERR_INVALID_ARG, "hc_track_toric: null buffer");
  for (int64_t k = 0; k < npaths; ++k) {
    if (rows[k] < 0 || rows[k] >= h->tor_rows)
      return fail(h, HC_ERR_INVALID_ARG, "hc_track_toric: weight row out of range");
    if (!std::isfinite(t1[k]) || !std::isfinite(t0[k]) || t1[k] < 0.0 || t0[k] < 0.0)
      return fail(h, HC_ERR_INVALID_ARG, "hc_track_toric: times must be finite and non-negative");
  }
  const int n = h->prog.n;
  int rc = ensure_capacity(h, npaths, n);
  if (rc != HC_OK) return rc;
  const size_t nv = (size_t)npaths * n;
  const size_t pbytes = (size_t)npaths * (4 * sizeof(double) + sizeof(int32_t));
  if (h->tor_path_cap < pbytes) {
    cudaFree(h->d_tor_path);
    h->d_tor_path = nullptr;
    h->tor_path_cap = 0;
    CK(cudaMalloc(&h->d_tor_path, pbytes));
    h->tor_path_cap = pbytes;
  }
  double* dp = (double*)h->d_tor_path;
  int32_t* drow = (int32_t*)(dp + 4 * npaths);
  PathArgs pa;
  pa.t1 = dp;
  pa.t0 = dp + npaths;
  pa.omega = omega ? dp + 2 * npaths : nullptr;
  pa.mu = mu ? dp + 3 * npaths : nullptr;
  pa.tor_w = h->d_tor_w;
  pa.tor_row = drow;
  start_clock(h);
  CK(cudaMemcpyAsync(h->d_starts, starts, nv * sizeof(double2), cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemcpyAsync(dp, t1, npaths * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemcpyAsync(dp + npaths, t0, npaths * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  if (omega) CK(cudaMemcpyAsync(dp + 2 * npaths, omega, npaths * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  if (mu) CK(cudaMemcpyAsync(dp + 3 * npaths, mu, npaths * sizeof(double), cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemcpyAsync(drow, rows, npaths * sizeof(int32_t), cudaMemcpyHostToDevice, h->stream));
  // the toric tracker runs in FP64 with the plain step rule
  hc_options O = h->opts;
  O.precision = HC_PREC_FP64;
  O.step_control = HC_STEP_PLAIN;
  rc = track_device_impl(h, npaths, (const double*)h->d_starts, 0, 0.0, 0.0, 1.0, 0.0, h->d_res, (double*)h->d_sol,
                         nullptr, nullptr, h->stream, O, nullptr, pa);
  if (rc != HC_OK) return rc;
  if (h->time_limit > 0) CK(wait_stream(h));  // before the blocking copies to pageable memory
  CK(cudaMemcpyAsync(out_results, h->d_res, (size_t)npaths * sizeof(hc_path_result), cudaMemcpyDeviceToHost,
                     h->stream));
  CK(cudaMemcpyAsync(out_solutions, h->d_sol, nv * sizeof(double2), cudaMemcpyDeviceToHost, h->stream));
  unsigned long long st[HC_NSTATS + HC_NPHASE];
  CK(cudaMemcpyAsync(st, h->d_counter + 1, sizeof(st), cudaMemcpyDeviceToHost, h->stream));
  CK(wait_stream(h));
  for (int i = 0; i < HC_NSTATS + HC_NPHASE; ++i) h->stats[i] = (double)st[i];
  h->retracked = 0;
  h->stats_on_host = true;
  if (*h->h_cancel) return stopped(h, "hc_track_toric");
  return HC_OK;
}

int hc_set_step_model(hc_handle* h, const float* params, const float* mean, const float* std, double confidence,
                      double max_factor) {
  if (!h || !params || !mean || !std) return fail(h, HC_ERR_INVALID_ARG, "hc_set_step_model: null pointer");
  DeviceGuard dg(h);
  if (!(confidence > 0.0 && confidence < 1.0) || !(max_factor >= 1.0 && max_factor <= 1e3))
    return fail(h, HC_ERR_INVALID_ARG, "hc_set_step_model: need 0 < confidence < 1 and 1 <= max_factor <= 1000");
  const int np = hc_mlp_num_params();
  for (int i = 0; i < np; ++i)
    if (!std::isfinite(params[i])) return fail(h, HC_ERR_INVALID_ARG, "hc_set_step_model: non-finite parameter");
  StepModel M;
  std::memset(&M, 0, sizeof(M));
  for (int i = 0; i < HC_NFEAT; ++i) {
    if (!std::isfinite(mean[i]) || !(std[i] > 0.f) || !std::isfinite(std[i]))
      return fail(h, HC_ERR_INVALID_ARG, "hc_set_step_model: bad feature normalisation");
    M.mean[i] = mean[i];
    M.stdinv[i] = 1.0f / std[i];
  }
  M.c = (float)std::log(confidence / (1.0 - confidence));
  M.logmax = (float)std::log(max_factor);
  // parameter layout of hc_mlp.cu: W1[64][12] b1[64] W2[64][64] b2[64] W3[2][64] b3[2]
  const float* p = params;
  for (int u = 0; u < 64; ++u)
    for (int i = 0; i < HC_NFEAT; ++i) M.W1T[i * 64 + u] = to_bf16(*p++);
  for (int i = 0; i < 64; ++i) M.b1[i] = *p++;
  for (int u = 0; u < 64; ++u)
    for (int v = 0; v < 64; ++v) M.W2T[v * 64 + u] = to_bf16(*p++);
  for (int i = 0; i < 64; ++i) M.b2[i] = *p++;
  for (int i = 0; i < 2 * 64; ++i) M.W3[i] = to_bf16(*p++);
  for (int i = 0; i < 2; ++i) M.b3[i] = *p++;
  if (p - params != np) return fail(h, HC_ERR_INVALID_ARG, "hc_set_step_model: parameter layout mismatch");
  if (!h->d_model) CK(cudaMalloc(&h->d_model, sizeof(StepModel)));
  CK(cudaMemcpyAsync(h->d_model, &M, sizeof(StepModel), cudaMemcpyHostToDevice, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  ++h->generation;
  return HC_OK;
}

// ---------------------------------------------------------------------------- batches
}  // extern "C"

// Mixed-precision instance tables with the staging `staging[n]` per n. Instances with global
// slices share one slice stride (the largest), so the warps of CTAs on different instances
// never overlap.
static void mixed_instances(const hc_handle* h, const int32_t* staging, std::vector<BatchInstance>& I, int* tb,
                            int* ws, int* cold) {
  I.resize(h->bninst);
  *tb = *ws = *cold = 0;
  for (int i = 0; i < h->bninst; ++i) {
    I[i] = h->bhost[staging[h->bn[i]] == 1 ? 1 : 2][i];
    *tb = std::max(*tb, I[i].T.bytes);
    *ws = std::max(*ws, I[i].L.bytes);
    *cold = std::max(*cold, I[i].L.cold);
  }
  for (auto& B : I)
    if (B.L.cold > 0) B.L.cold = *cold;
}

// Work units of the instances in `which` (every instance when null): at most unit_paths[n]
// paths of one instance (0: `wpc`, one path per warp of a CTA — measured fastest on 2,000
// uneven instances, since small units leave little idle time at the end of a unit, when a
// CTA's warps wait for its slowest path before the tables are re-staged), largest estimated
// cost first.
static std::vector<BatchUnit> batch_units(const hc_handle* h, const int32_t* unit_paths, int wpc,
                                          const std::vector<int>* which) {
  struct U {
    BatchUnit u;
    double cost;
  };
  std::vector<U> units;
  auto add = [&](int i) {
    int64_t up = unit_paths[h->bn[i]] > 0 ? unit_paths[h->bn[i]] : wpc;
    for (int64_t lo = 0; lo < h->bnpaths[i]; lo += up) {
      int64_t hi = std::min<int64_t>(h->bnpaths[i], lo + up);
      units.push_back({BatchUnit{i, (int)lo, (int)hi, 0}, h->bcost[i] * (double)(hi - lo)});
    }
  };
  if (which)
    for (int i : *which) add(i);
  else
    for (int i = 0; i < h->bninst; ++i) add(i);
  std::stable_sort(units.begin(), units.end(), [](const U& a, const U& b) { return a.cost > b.cost; });
  std::vector<BatchUnit> out(units.size());
  for (size_t k = 0; k < units.size(); ++k) out[k] = units[k].u;
  return out;
}

// warps per CTA the default unit size assumes (shared-memory fit of the mixed tables, at most
// HC_MAX_BATCH_WARPS)
static int batch_wpc_estimate(int tb, int ws) {
  return (int)std::max<int64_t>(
      1, std::min<int64_t>(HC_MAX_BATCH_WARPS, (227 * 1024 - HC_LAUNCH_SMEM - tb) / std::max(ws, 1)));
}

// upload `units` into a device array of the handle (grown on demand)
static int upload_units(hc_handle* h, BatchUnit** d, size_t* cap, const std::vector<BatchUnit>& units) {
  if (*cap < units.size() || !*d) {
    CK(cudaStreamSynchronize(h->stream));
    cudaFree(*d);
    *d = nullptr;
    *cap = 0;
    size_t c = std::max<size_t>(1, units.size());
    CK(cudaMalloc(d, c * sizeof(BatchUnit)));
    *cap = c;
  }
  if (!units.empty())
    CK(cudaMemcpyAsync(*d, units.data(), units.size() * sizeof(BatchUnit), cudaMemcpyHostToDevice, h->stream));
  return HC_OK;
}

// Make (unit_paths, staging) the batch's launch plan: mixed instance tables, queue of units.
static int apply_batch_plan(hc_handle* h, const int32_t* unit_paths, const int32_t* staging) {
  std::vector<BatchInstance> I1;
  int tb = 0, ws = 0, cold = 0;
  mixed_instances(h, staging, I1, &tb, &ws, &cold);
  std::vector<BatchUnit> units = batch_units(h, unit_paths, batch_wpc_estimate(tb, ws), nullptr);
  CK(cudaStreamSynchronize(h->stream));
  CK(cudaMemcpyAsync(h->d_binst[1], I1.data(), I1.size() * sizeof(BatchInstance), cudaMemcpyHostToDevice,
                     h->stream));
  int rc = upload_units(h, &h->d_bunits, &h->bunits_cap, units);
  if (rc != HC_OK) return rc;
  CK(cudaStreamSynchronize(h->stream));
  h->bnunits = (int)units.size();
  h->btbytes[1] = tb;
  h->bwstride[1] = ws;
  h->bcold = cold;
  std::memcpy(h->bunit_paths, unit_paths, sizeof(h->bunit_paths));
  std::memcpy(h->bstaging, staging, sizeof(h->bstaging));
  ++h->generation;
  return HC_OK;
}

extern "C" {

int hc_set_batch(hc_handle* h, int ninstances, const hc_instance_desc* inst, const int32_t* unit_paths,
                 int64_t* total_paths, int64_t* total_elements) {
  if (!h) return fail(h, HC_ERR_INVALID_ARG, "hc_set_batch: null handle");
  DeviceGuard dg(h);
  if (ninstances < 1 || !inst) return fail(h, HC_ERR_INVALID_ARG, "hc_set_batch: need at least one instance");
  for (int i = 0; i < ninstances; ++i) {
    const hc_instance_desc& d = inst[i];
    std::string at = "hc_set_batch: instance " + std::to_string(i) + ": ";
    if (d.n < 1 || d.n > 32) return fail(h, HC_ERR_UNSUPPORTED, at + "need 1 <= n <= 32");
    if (d.nG < 0 || d.nF < 0 || (d.nG > 0 && (!d.G_eq || !d.G_exps || !d.G_coef)) ||
        (d.nF > 0 && (!d.F_eq || !d.F_exps || !d.F_coef)))
      return fail(h, HC_ERR_INVALID_ARG, at + "bad term table");
    if (!std::isfinite(d.gamma_re) || !std::isfinite(d.gamma_im))
      return fail(h, HC_ERR_INVALID_ARG, at + "gamma must be finite");
    if (d.npaths < 0 || d.npaths > (int64_t)1 << 30) return fail(h, HC_ERR_INVALID_ARG, at + "bad npaths");
  }
  if (unit_paths)
    for (int n = 0; n <= 32; ++n)
      if (unit_paths[n] < 0) return fail(h, HC_ERR_INVALID_ARG, "hc_set_batch: negative unit_paths entry");
  // compile the programs on all host cores
  std::vector<HostProg> P(ninstances);
  std::vector<int> rcs(ninstances, HC_OK);
  std::vector<std::string> errs(ninstances);
  {
    int nt = (int)std::max(1u, std::min(32u, std::thread::hardware_concurrency()));
    nt = std::min(nt, ninstances);
    std::vector<std::thread> th;
    for (int t = 0; t < nt; ++t)
      th.emplace_back([&, t] {
        for (int i = t; i < ninstances; i += nt) {
          const hc_instance_desc& d = inst[i];
          rcs[i] = build_program(d.n, d.nG, d.G_eq, d.G_exps, d.G_coef, d.nF, d.F_eq, d.F_exps, d.F_coef, P[i],
                                 errs[i]);
        }
      });
    for (auto& x : th) x.join();
  }
  for (int i = 0; i < ninstances; ++i)
    if (rcs[i] != HC_OK) return fail(h, rcs[i], "hc_set_batch: instance " + std::to_string(i) + ": " + errs[i]);
  std::vector<char> blob;
  std::vector<ProgOffsets> off(ninstances);
  std::vector<BatchInstance> I[3];
  for (auto& v : I) v.resize(ninstances);
  std::vector<double> cost(ninstances);
  int tb0 = 0, ws0 = 0;
  int64_t tp = 0, tv = 0;
  for (int i = 0; i < ninstances; ++i) {
    WarpLayout L = make_warp_layout(P[i]);
    TableLayout T32 = make_table_layout(P[i], HC_PREC_MIXED);
    if ((size_t)HC_LAUNCH_SMEM + T32.bytes + L.bytes > 220 * 1024)
      return fail(h, HC_ERR_TOO_LARGE,
                  "hc_set_batch: instance " + std::to_string(i) + ": tables plus one path exceed shared memory");
    off[i] = pack_program(P[i], blob);
    for (int v = 0; v < 3; ++v) {
      BatchInstance& B = I[v][i];
      B.T = v == 0 ? make_table_layout(P[i], HC_PREC_FP64) : make_table_layout(P[i], HC_PREC_MIXED, v == 2);
      B.L = v == 0 ? L : make_warp_layout(P[i], 0, v == 2);
      B.npaths = inst[i].npaths;
      B.path_off = tp;
      B.vec_off = tv;
    }
    tb0 = std::max(tb0, I[0][i].T.bytes);
    ws0 = std::max(ws0, I[0][i].L.bytes);
    // monomial evaluations, Jacobian terms and the LU of one path
    cost[i] = (double)P[i].M * inst[i].n + (double)inst[i].n * inst[i].n * inst[i].n + (double)P[i].jcode.size();
    tp += inst[i].npaths;
    tv += inst[i].npaths * inst[i].n;
  }
  // upload: programs and instance tables; the launch plan (mixed tables by staging, units) follows
  h->has_batch = false;
  if (h->d_bprog_bytes < blob.size()) {
    cudaFree(h->d_bprog);
    h->d_bprog = nullptr;
    h->d_bprog_bytes = 0;
    CK(cudaMalloc(&h->d_bprog, blob.size()));
    h->d_bprog_bytes = blob.size();
  }
  for (int i = 0; i < ninstances; ++i) {
    DevProg D = bind_program(P[i], off[i], h->d_bprog, inst[i].gamma_re, inst[i].gamma_im);
    for (int v = 0; v < 3; ++v) I[v][i].P = D;
  }
  for (int q = 0; q < 2; ++q) {
    cudaFree(h->d_binst[q]);
    h->d_binst[q] = nullptr;
    CK(cudaMalloc(&h->d_binst[q], (size_t)ninstances * sizeof(BatchInstance)));
  }
  CK(cudaMemcpyAsync(h->d_bprog, blob.data(), blob.size(), cudaMemcpyHostToDevice, h->stream));
  CK(cudaMemcpyAsync(h->d_binst[0], I[0].data(), (size_t)ninstances * sizeof(BatchInstance),
                     cudaMemcpyHostToDevice, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  h->bninst = ninstances;
  h->btbytes[0] = tb0;
  h->bwstride[0] = ws0;
  h->btotal_paths = tp;
  h->btotal_vec = tv;
  h->bpath_off.resize(ninstances);
  h->bvec_off.resize(ninstances);
  h->bnpaths.resize(ninstances);
  h->bn.resize(ninstances);
  for (int i = 0; i < ninstances; ++i) {
    h->bpath_off[i] = I[0][i].path_off;
    h->bvec_off[i] = I[0][i].vec_off;
    h->bnpaths[i] = inst[i].npaths;
    h->bn[i] = inst[i].n;
  }
  for (int v = 0; v < 3; ++v) h->bhost[v] = std::move(I[v]);
  h->bcost = std::move(cost);
  int32_t up[33] = {0};
  if (unit_paths) std::memcpy(up, unit_paths, sizeof(up));
  int rc = apply_batch_plan(h, up, h->bstaging);
  if (rc != HC_OK) return rc;
  h->has_batch = true;
  if (total_paths) *total_paths = tp;
  if (total_elements) *total_elements = tv;
  return HC_OK;
}

int hc_set_batch_launch(hc_handle* h, const int32_t* unit_paths, const int32_t* staging) {
  if (!h) return fail(h, HC_ERR_INVALID_ARG, "hc_set_batch_launch: null handle");
  DeviceGuard dg(h);
  if (!h->has_batch) return fail(h, HC_ERR_NO_SYSTEM, "hc_set_batch_launch: call hc_set_batch first");
  int32_t up[33] = {0}, st[33] = {0};
  for (int n = 0; n <= 32; ++n) {
    up[n] = unit_paths ? unit_paths[n] : 0;
    st[n] = staging ? staging[n] : 0;
    if (up[n] < 0) return fail(h, HC_ERR_INVALID_ARG, "hc_set_batch_launch: negative unit_paths entry");
    if (st[n] < 0 || st[n] > 2) return fail(h, HC_ERR_INVALID_ARG, "hc_set_batch_launch: staging entries must be 0, 1 or 2");
  }
  return apply_batch_plan(h, up, st);
}

// shared memory, warps per CTA and CTAs of a batch launch with options O
static int batch_geometry(hc_handle* h, const hc_options& O, int nunits, size_t* smem_out, int* wpc_out,
                          int* blocks_out) {
  const int q = O.precision == HC_PREC_MIXED ? 1 : 0;
  const size_t smem_cap = 227 * 1024;
  const size_t fixed = (size_t)HC_LAUNCH_SMEM + h->btbytes[q];
  int wpc = std::min(O.warps_per_cta, HC_MAX_BATCH_WARPS);
  if (wpc <= 0)
    wpc = balanced_warps(
        (int)std::max<size_t>(1, std::min<size_t>(HC_MAX_BATCH_WARPS, (smem_cap - fixed) / h->bwstride[q])),
        O.precision);
  size_t smem = fixed + (size_t)wpc * h->bwstride[q];
  while (wpc > 1 && smem > smem_cap) {
    --wpc;
    smem = fixed + (size_t)wpc * h->bwstride[q];
  }
  if (smem > smem_cap) return fail(h, HC_ERR_TOO_LARGE, "batch: working set exceeds shared memory");
  int bps = 0;
  CK(prepare_batch(O.precision, smem, wpc, &bps));
  if (bps < 1) return fail(h, HC_ERR_TOO_LARGE, "batch: kernel does not fit on an SM");
  if (O.ctas_per_sm > 0) bps = std::min(bps, O.ctas_per_sm);
  *smem_out = smem;
  *wpc_out = wpc;
  *blocks_out = (int)std::min<int64_t>((int64_t)bps * h->num_sms, nunits);
  return HC_OK;
}

static BatchLaunch batch_launch(hc_handle* h, const hc_options& O, const double* d_starts, int endgame,
                                hc_path_result* d_results, double* d_solutions, const BatchUnit* units,
                                int nunits, int wpc) {
  const int q = O.precision == HC_PREC_MIXED ? 1 : 0;
  BatchLaunch bl{};
  Launch& la = bl.base;
  la.O = O;
  la.npaths = h->btotal_paths;
  la.starts = (const double2*)d_starts;
  la.res = d_results;
  la.sol = (double2*)d_solutions;
  la.mode = endgame ? 1 : 0;
  la.t1_re = 1.0;
  la.t0_re = 0.0;
  la.counter = h->d_counter;
  la.cancel = h->d_cancel;
  la.stats = h->d_counter + 1;
  la.model = O.step_control == HC_STEP_LEARNED ? h->d_model : nullptr;
  la.phase = h->d_counter + 1 + HC_NSTATS;
  bl.inst = h->d_binst[q];
  bl.units = units;
  bl.nunits = nunits;
  bl.tbytes = h->btbytes[q];
  bl.wstride = h->bwstride[q];
  la.cold = q == 1 ? h->d_bcold : nullptr;
  la.lockstep = lockstep_for(O, wpc, true);
  return bl;
}

// the mixed batch's per-warp global slices for a launch of `blocks` CTAs of `wpc` warps
static int ensure_bcold(hc_handle* h, const hc_options& O, int blocks, int wpc) {
  if (O.precision != HC_PREC_MIXED || h->bcold <= 0) return HC_OK;
  size_t need = (size_t)blocks * wpc * (size_t)h->bcold;
  if (h->bcold_cap >= need) return HC_OK;
  CK(cudaStreamSynchronize(h->stream));
  cudaFree(h->d_bcold);
  h->d_bcold = nullptr;
  h->bcold_cap = 0;
  CK(cudaMalloc(&h->d_bcold, need));
  h->bcold_cap = need;
  ++h->generation;  // a recorded graph holds the old address
  return HC_OK;
}

int hc_track_batch_device(hc_handle* h, const double* d_starts, int endgame, hc_path_result* d_results,
                          double* d_solutions, void* stream) {
  if (!h) return fail(h, HC_ERR_INVALID_ARG, "hc_track_batch_device: null handle");
  DeviceGuard dg(h);
  if (!h->has_batch) return fail(h, HC_ERR_NO_SYSTEM, "hc_track_batch_device: call hc_set_batch first");
  if (h->btotal_paths == 0) return HC_OK;
  if (!d_starts || !d_results || !d_solutions)
    return fail(h, HC_ERR_INVALID_ARG, "hc_track_batch_device: null buffer");
  if (h->opts.step_control == HC_STEP_LEARNED && !h->d_model)
    return fail(h, HC_ERR_INVALID_ARG, "hc_track_batch_device: learned step control needs hc_set_step_model");
  size_t smem = 0;
  int wpc = 0, blocks = 0;
  int rc = batch_geometry(h, h->opts, h->bnunits, &smem, &wpc, &blocks);
  if (rc != HC_OK) return rc;
  rc = ensure_bcold(h, h->opts, blocks, wpc);
  if (rc != HC_OK) return rc;
  h->stats_on_host = false;
  cudaStream_t s = stream ? (cudaStream_t)stream : h->stream;
  const bool same = h->bgraph && h->bgraph_key[0] == d_starts && h->bgraph_key[1] == d_results &&
                    h->bgraph_key[2] == d_solutions && h->bgraph_endgame == (endgame ? 1 : 0) &&
                    h->bgraph_blocks == blocks && h->bgraph_wpc == wpc && h->bgraph_gen == h->generation;
  if (!same) {
    if (h->bgraph) cudaGraphExecDestroy(h->bgraph);
    h->bgraph = nullptr;
    BatchLaunch bl =
        batch_launch(h, h->opts, d_starts, endgame, d_results, d_solutions, h->d_bunits, h->bnunits, wpc);
    // record: clear the queue head and counters, then the kernel
    cudaGraph_t g = nullptr;
    CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
    cudaError_t e =
        cudaMemsetAsync(h->d_counter, 0, (1 + HC_NSTATS + HC_NPHASE) * sizeof(unsigned long long), h->stream);
    if (e == cudaSuccess) e = launch_batch(bl, blocks, wpc, smem, h->stream);
    cudaError_t e2 = cudaStreamEndCapture(h->stream, &g);
    if (e == cudaSuccess) e = e2;
    if (e == cudaSuccess) e = cudaGraphInstantiate(&h->bgraph, g, 0);
    if (g) cudaGraphDestroy(g);
    if (e != cudaSuccess) {
      h->bgraph = nullptr;
      return cuda_fail(h, e, "hc_track_batch_device: recording the launch");
    }
    h->bgraph_key[0] = d_starts;
    h->bgraph_key[1] = d_results;
    h->bgraph_key[2] = d_solutions;
    h->bgraph_endgame = endgame ? 1 : 0;
    h->bgraph_blocks = blocks;
    h->bgraph_wpc = wpc;
    h->bgraph_gen = h->generation;
  }
  CK(cudaGraphLaunch(h->bgraph, s));
  h->last_blocks = blocks;
  h->last_wpc = wpc;
  h->last_lockstep = lockstep_for(h->opts, wpc, true);
  h->last_stream = s;
  return HC_OK;
}

int hc_track_batch(hc_handle* h, const double* starts, int endgame, hc_path_result* out_results,
                   double* out_solutions) {
  if (!h) return fail(h, HC_ERR_INVALID_ARG, "hc_track_batch: null handle");
  DeviceGuard dg(h);
  if (!h->has_batch) return fail(h, HC_ERR_NO_SYSTEM, "hc_track_batch: call hc_set_batch first");
  if (h->btotal_paths == 0) return HC_OK;
  if (!starts || !out_results || !out_solutions) return fail(h, HC_ERR_INVALID_ARG, "hc_track_batch: null buffer");
  int rc = ensure_capacity_v(h, h->btotal_paths, h->btotal_vec);
  if (rc != HC_OK) return rc;
  size_t nv = (size_t)h->btotal_vec;
  start_clock(h);
  CK(cudaMemcpyAsync(h->d_starts, starts, nv * sizeof(double2), cudaMemcpyHostToDevice, h->stream));
  rc = hc_track_batch_device(h, (const double*)h->d_starts, endgame, h->d_res, (double*)h->d_sol, nullptr);
  if (rc != HC_OK) return rc;
  if (h->time_limit > 0) CK(wait_stream(h));  // before the blocking copies to pageable memory
  CK(cudaMemcpyAsync(out_results, h->d_res, (size_t)h->btotal_paths * sizeof(hc_path_result),
                     cudaMemcpyDeviceToHost, h->stream));
  CK(cudaMemcpyAsync(out_solutions, h->d_sol, nv * sizeof(double2), cudaMemcpyDeviceToHost, h->stream));
  unsigned long long st[HC_NSTATS + HC_NPHASE];
  CK(cudaMemcpyAsync(st, h->d_counter + 1, sizeof(st), cudaMemcpyDeviceToHost, h->stream));
  CK(wait_stream(h));
  for (int i = 0; i < HC_NSTATS + HC_NPHASE; ++i) h->stats[i] = (double)st[i];
  h->retracked = 0;
  h->stats_on_host = true;
  if (*h->h_cancel) return stopped(h, "hc_track_batch");
  if (h->opts.step_control == HC_STEP_LEARNED && endgame) {
    // per instance: re-track the paths whose endpoints coincide with plain step control, in place
    std::vector<BatchUnit> units;
    for (int i = 0; i < h->bninst; ++i) {
      std::vector<int64_t> idx = coincident_paths(out_results + h->bpath_off[i],
                                                  (const double2*)out_solutions + h->bvec_off[i], h->bnpaths[i],
                                                  h->bn[i]);
      for (int64_t k : idx) units.push_back(BatchUnit{i, (int)k, (int)k + 1, 0});
    }
    if (!units.empty()) {
      if (h->runits_cap < units.size()) {
        cudaFree(h->d_runits);
        h->d_runits = nullptr;
        h->runits_cap = 0;
        CK(cudaMalloc(&h->d_runits, units.size() * sizeof(BatchUnit)));
        h->runits_cap = units.size();
      }
      CK(cudaMemcpyAsync(h->d_runits, units.data(), units.size() * sizeof(BatchUnit), cudaMemcpyHostToDevice,
                         h->stream));
      hc_options O = h->opts;
      O.step_control = HC_STEP_PLAIN;
      size_t smem = 0;
      int wpc = 0, blocks = 0;
      rc = batch_geometry(h, O, (int)units.size(), &smem, &wpc, &blocks);
      if (rc != HC_OK) return rc;
      rc = ensure_bcold(h, O, blocks, wpc);
      if (rc != HC_OK) return rc;
      BatchLaunch bl = batch_launch(h, O, (const double*)h->d_starts, endgame, h->d_res, (double*)h->d_sol,
                                    h->d_runits, (int)units.size(), wpc);
      CK(cudaMemsetAsync(h->d_counter, 0, (1 + HC_NSTATS + HC_NPHASE) * sizeof(unsigned long long), h->stream));
      CK(launch_batch(bl, blocks, wpc, smem, h->stream));
      if (h->time_limit > 0) CK(wait_stream(h));
      for (const BatchUnit& u : units) {
        int64_t r = h->bpath_off[u.inst] + u.lo, e = h->bvec_off[u.inst] + (int64_t)u.lo * h->bn[u.inst];
        CK(cudaMemcpyAsync(out_results + r, h->d_res + r, sizeof(hc_path_result), cudaMemcpyDeviceToHost,
                           h->stream));
        CK(cudaMemcpyAsync(out_solutions + 2 * e, h->d_sol + e, h->bn[u.inst] * sizeof(double2),
                           cudaMemcpyDeviceToHost, h->stream));
      }
      CK(cudaMemcpyAsync(st, h->d_counter + 1, sizeof(st), cudaMemcpyDeviceToHost, h->stream));
      CK(wait_stream(h));
      for (int i = 0; i < HC_NSTATS + HC_NPHASE; ++i) h->stats[i] += (double)st[i];
      h->stats[0] -= (double)units.size();
      h->retracked = (double)units.size();
      if (*h->h_cancel) return stopped(h, "hc_track_batch");
    }
  }
  return HC_OK;
}

int hc_autotune_batch(hc_handle* h, const double* starts, int sample, const int32_t* candidates, int ncandidates,
                      int repeats, int32_t* unit_paths_out, int32_t* staging_out, double* ms_out) {
  if (!h) return fail(h, HC_ERR_INVALID_ARG, "hc_autotune_batch: null handle");
  DeviceGuard dg(h);
  if (!h->has_batch) return fail(h, HC_ERR_NO_SYSTEM, "hc_autotune_batch: call hc_set_batch first");
  if (!starts || !candidates || ncandidates < 1 || ncandidates > 16 || repeats < 1)
    return fail(h, HC_ERR_INVALID_ARG, "hc_autotune_batch: need starts, 1..16 candidates and repeats >= 1");
  for (int c = 0; c < ncandidates; ++c)
    if (candidates[c] < 1) return fail(h, HC_ERR_INVALID_ARG, "hc_autotune_batch: candidates must be positive");
  if (h->btotal_paths == 0) return HC_OK;
  int rc = ensure_capacity_v(h, h->btotal_paths, h->btotal_vec);
  if (rc != HC_OK) return rc;
  start_clock(h);
  CK(cudaMemcpyAsync(h->d_starts, starts, (size_t)h->btotal_vec * sizeof(double2), cudaMemcpyHostToDevice,
                     h->stream));
  const hc_options O = h->opts;
  const bool mixed = O.precision == HC_PREC_MIXED;
  const int nst = mixed ? 2 : 1;
  const int32_t stval[2] = {2, 1};  // global slices, all shared
  std::vector<int> byn[33];
  for (int i = 0; i < h->bninst; ++i)
    if (h->bnpaths[i] > 0 && (sample <= 0 || (int)byn[h->bn[i]].size() < sample)) byn[h->bn[i]].push_back(i);
  int32_t up[33], st[33];
  std::memcpy(up, h->bunit_paths, sizeof(up));
  std::memcpy(st, h->bstaging, sizeof(st));
  if (ms_out)
    for (int k = 0; k < 33 * 2 * ncandidates; ++k) ms_out[k] = std::nan("");
  cudaEvent_t ev[2];
  CK(cudaEventCreate(&ev[0]));
  CK(cudaEventCreate(&ev[1]));
  auto run = [&](int n) -> int {
    double best = INFINITY;
    int32_t bu = up[n], bs = st[n];
    for (int si = 0; si < nst; ++si) {
      st[n] = mixed ? stval[si] : st[n];
      std::vector<BatchInstance> I1;
      int tb = 0, ws = 0, cold = 0;
      mixed_instances(h, st, I1, &tb, &ws, &cold);
      if (mixed) {
        CK(cudaStreamSynchronize(h->stream));
        CK(cudaMemcpyAsync(h->d_binst[1], I1.data(), I1.size() * sizeof(BatchInstance), cudaMemcpyHostToDevice,
                           h->stream));
        h->btbytes[1] = tb;
        h->bwstride[1] = ws;
        h->bcold = cold;
      }
      for (int c = 0; c < ncandidates; ++c) {
        up[n] = candidates[c];
        std::vector<BatchUnit> units = batch_units(h, up, 0, &byn[n]);
        int r = upload_units(h, &h->d_runits, &h->runits_cap, units);
        if (r != HC_OK) return r;
        size_t smem = 0;
        int wpc = 0, blocks = 0;
        r = batch_geometry(h, O, (int)units.size(), &smem, &wpc, &blocks);
        if (r != HC_OK) return r;
        r = ensure_bcold(h, O, blocks, wpc);
        if (r != HC_OK) return r;
        BatchLaunch bl = batch_launch(h, O, (const double*)h->d_starts, 1, h->d_res, (double*)h->d_sol,
                                      h->d_runits, (int)units.size(), wpc);
        for (int k = 0; k <= repeats; ++k) {  // k = 0: warm-up
          if (k == 1) CK(cudaEventRecord(ev[0], h->stream));
          CK(cudaMemsetAsync(h->d_counter, 0, (1 + HC_NSTATS + HC_NPHASE) * sizeof(unsigned long long),
                             h->stream));
          CK(launch_batch(bl, blocks, wpc, smem, h->stream));
        }
        CK(cudaEventRecord(ev[1], h->stream));
        CK(wait_stream(h));
        if (*h->h_cancel) return stopped(h, "hc_autotune_batch");
        float ms = 0;
        CK(cudaEventElapsedTime(&ms, ev[0], ev[1]));
        const double t = (double)ms / repeats;
        if (ms_out) ms_out[(n * 2 + si) * ncandidates + c] = t;
        if (t < best) {
          best = t;
          bu = up[n];
          bs = st[n];
        }
      }
    }
    up[n] = bu;
    st[n] = bs;
    return HC_OK;
  };
  for (int n = 1; n <= 32 && rc == HC_OK; ++n)
    if (!byn[n].empty()) rc = run(n);
  cudaEventDestroy(ev[0]);
  cudaEventDestroy(ev[1]);
  if (rc == HC_OK) rc = apply_batch_plan(h, up, st);
  else {  // restore the previous plan's tables (keeping the first error)
    int32_t pu[33], ps[33];
    std::memcpy(pu, h->bunit_paths, sizeof(pu));
    std::memcpy(ps, h->bstaging, sizeof(ps));
    apply_batch_plan(h, pu, ps);
  }
  if (rc != HC_OK) return rc;
  if (unit_paths_out) std::memcpy(unit_paths_out, up, sizeof(up));
  if (staging_out) std::memcpy(staging_out, st, sizeof(st));
  return HC_OK;
}

int hc_certify(hc_handle* h, int64_t ncand, const double* cand, int real_coefficients, hc_certificate* out,
               double* out_centers, double* out_enclosures) {
  if (!h) return fail(h, HC_ERR_INVALID_ARG, "hc_certify: null handle");
  DeviceGuard dg(h);
  if (!h->has_prog) return fail(h, HC_ERR_NO_SYSTEM, "hc_certify: call hc_set_homotopy first");
  if (h->slp) return fail(h, HC_ERR_UNSUPPORTED, "hc_certify: not available for a straight-line program");
  if (ncand < 0) return fail(h, HC_ERR_INVALID_ARG, "hc_certify: ncandidates < 0");
  if (ncand == 0) return HC_OK;
  if (!cand || !out || !out_centers || !out_enclosures) return fail(h, HC_ERR_INVALID_ARG, "hc_certify: null buffer");
  int bytes = 0;
  if (certify_layout(h->dprog, &bytes) != 0)
    return fail(h, HC_ERR_TOO_LARGE, "hc_certify: the system's certification working set exceeds shared memory");
  int n = h->prog.n;
  int rc = ensure_capacity(h, ncand, n);
  if (rc != HC_OK) return rc;
  size_t nv = (size_t)ncand * n;
  static_assert(sizeof(hc_certificate) <= sizeof(hc_path_result), "certificates reuse the result buffer");
  hc_certificate* d_cert = (hc_certificate*)h->d_res;
  CK(cudaMemcpyAsync(h->d_starts, cand, nv * sizeof(double2), cudaMemcpyHostToDevice, h->stream));
  CK(launch_certify(h->dprog, ncand, nullptr, false, (const double*)h->d_starts, d_cert, (double*)h->d_sol,
                    (double*)h->d_last, real_coefficients ? 1 : 0, h->num_sms, h->stream));
  CK(cudaMemcpyAsync(out, d_cert, (size_t)ncand * sizeof(hc_certificate), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  // the candidates FP64 balls did not certify, again with double-word centres
  std::vector<int64_t> again;
  for (int64_t k = 0; k < ncand; ++k)
    if (!out[k].certified) again.push_back(k);
  if (!again.empty()) {
    if (h->plist_cap < again.size()) {
      cudaFree(h->d_plist);
      h->d_plist = nullptr;
      h->plist_cap = 0;
      CK(cudaMalloc(&h->d_plist, again.size() * sizeof(int64_t)));
      h->plist_cap = again.size();
    }
    CK(cudaMemcpyAsync(h->d_plist, again.data(), again.size() * sizeof(int64_t), cudaMemcpyHostToDevice, h->stream));
    CK(launch_certify(h->dprog, (int64_t)again.size(), h->d_plist, true, (const double*)h->d_starts, d_cert,
                      (double*)h->d_sol, (double*)h->d_last, real_coefficients ? 1 : 0, h->num_sms, h->stream));
    CK(cudaMemcpyAsync(out, d_cert, (size_t)ncand * sizeof(hc_certificate), cudaMemcpyDeviceToHost, h->stream));
  }
  CK(cudaMemcpyAsync(out_centers, h->d_sol, nv * sizeof(double2), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaMemcpyAsync(out_enclosures, h->d_last, nv * sizeof(double2), cudaMemcpyDeviceToHost, h->stream));
  CK(cudaStreamSynchronize(h->stream));
  return HC_OK;
}

int hc_cancel(hc_handle* h) {
  if (!h) return fail(h, HC_ERR_INVALID_ARG, "hc_cancel: null handle");
  __atomic_store_n(h->h_cancel, 1, __ATOMIC_SEQ_CST);
  return HC_OK;
}

int hc_set_time_limit(hc_handle* h, double seconds) {
  if (!h || !(seconds >= 0) || std::isinf(seconds))
    return fail(h, HC_ERR_INVALID_ARG, "hc_set_time_limit: need a handle and a finite limit >= 0");
  h->time_limit = seconds;
  return HC_OK;
}

const char* hc_last_error(hc_handle* h) {
  if (h) return h->err.c_str();
  std::lock_guard<std::mutex> g(g_err_mu);
  return g_err.c_str();
}

int hc_last_stats(hc_handle* h, double* out, int nout) {
  if (!h || !out || nout < 0) return fail(h, HC_ERR_INVALID_ARG, "hc_last_stats: bad argument");
  DeviceGuard dg(h);
  if (h->last_blocks > 0 && !h->stats_on_host) {  // counters of the last device-entry-point call
    unsigned long long st[HC_NSTATS + HC_NPHASE];
    CK(cudaMemcpyAsync(st, h->d_counter + 1, sizeof(st), cudaMemcpyDeviceToHost, h->last_stream));
    CK(cudaStreamSynchronize(h->last_stream));
    for (int i = 0; i < HC_NSTATS + HC_NPHASE; ++i) h->stats[i] = (double)st[i];
  }
  // [0] paths, [1] evaluations with Jacobian, [2] residual-only evaluations, [3] double-double
  // residuals, [4] Taylor orders (Σ K), [5] LU factorizations, [6] triangular solve pairs,
  // [7] FP32 Taylor evaluations redone in FP64, [8] paths moved to FP64 (mixed precision);
  // derived: [9] monomials M, [10] value terms, [11] Jacobian terms, [12] blocks, [13] warps
  // per block, [14] shared bytes per warp, [15] shared bytes of the CTA tables, [16] top-degree
  // monomial offset; [17] learned step proposals made, [18] of them rejected by Newton;
  // [19 ..] cycle counters of the tracker phases (HcPhase order; profiling builds only);
  // [19 + HC_NPHASE] paths re-tracked with plain step control by the jump check;
  // [20 + HC_NPHASE] lockstep mode of the last launch (0 per warp, 1 CTA, 2 sub-partition, 3 two
  // sub-partitions)
  double all[21 + HC_NPHASE];
  for (int i = 0; i < 9; ++i) all[i] = h->stats[i];
  all[9] = h->prog.M;
  all[10] = (double)h->prog.val_terms;
  all[11] = (double)h->prog.jac_terms;
  all[12] = h->last_blocks;
  all[13] = h->last_wpc;
  all[14] = h->last_warp_bytes ? h->last_warp_bytes : h->layout.bytes;
  all[15] = h->last_warp_bytes ? h->last_table_bytes : make_table_layout(h->prog, h->opts.precision).bytes;
  all[16] = h->prog.top;
  all[17] = h->stats[9];
  all[18] = h->stats[10];
  for (int k = 0; k < HC_NPHASE; ++k) all[19 + k] = h->stats[HC_NSTATS + k];
  all[19 + HC_NPHASE] = h->retracked;
  all[20 + HC_NPHASE] = h->last_lockstep;
  for (int i = 0; i < nout && i < 21 + HC_NPHASE; ++i) out[i] = all[i];
  return HC_OK;
}

}  // extern "C"

// =========================================================================================
// hc_track_noalloc: a tracking call that performs no device memory allocation.
//
// Some callers cannot call cudaMalloc: code running under an allocator that owns all device
// memory (a framework's caching pool, a memory-capped sandbox, an embedded runtime) or code
// that must not allocate on its hot path. For them this entry point keeps the scratch memory
// of the tracking kernel — the work-queue head, the counters, the cancel flag and the
// compiled homotopy tables — in the file-scope array below instead of in handle-owned
// allocations. The caller still passes the device buffers for start solutions, results and
// endpoints.
//
// Limits and sharing rules:
//   * the array holds HC_NOALLOC_SCRATCH_BYTES (1 MiB) on every GPU that loads this library,
//     for the life of the process; homotopies whose compiled tables exceed
//     HC_NOALLOC_MAX_PROGRAM_BYTES are rejected with HC_ERR_TOO_LARGE;
//   * every call on a device uses the same array and leaves its contents behind; the queue
//     head and counters are cleared at the start of each call, the tables are overwritten;
//     calls whose kernels overlap on the GPU race on the array and must be serialised by the
//     caller (for instance by issuing them on one stream);
//   * the first call on a device looks up the array's device address (cudaGetSymbolAddress)
//     once for that device; make that first call outside any stream capture.
// =========================================================================================
namespace {

constexpr size_t HC_NOALLOC_SCRATCH_BYTES = 1u << 20;
constexpr size_t HC_NOALLOC_HEADER_BYTES = 256;  // queue head, HC_NSTATS counters, cancel flag at +128
static_assert((1 + HC_NSTATS) * sizeof(unsigned long long) <= 128, "counters overlap the cancel flag");
constexpr size_t HC_NOALLOC_MAX_PROGRAM_BYTES = HC_NOALLOC_SCRATCH_BYTES - HC_NOALLOC_HEADER_BYTES;

static __device__ __align__(256) unsigned char g_noalloc_scratch[HC_NOALLOC_SCRATCH_BYTES];

constexpr int HC_NOALLOC_MAX_DEVICES = 64;
std::mutex g_noalloc_mu;
unsigned char* g_noalloc_ptr[HC_NOALLOC_MAX_DEVICES] = {nullptr};

// device address of g_noalloc_scratch on the current device (looked up once per device)
cudaError_t noalloc_scratch(unsigned char** out) {
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= HC_NOALLOC_MAX_DEVICES) return cudaErrorInvalidDevice;
  std::lock_guard<std::mutex> g(g_noalloc_mu);
  if (!g_noalloc_ptr[dev]) {
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess) return e;
    g_noalloc_ptr[dev] = (unsigned char*)p;
  }
  *out = g_noalloc_ptr[dev];
  return cudaSuccess;
}

}  // namespace

extern "C" int hc_track_noalloc(const hc_options* opts, int n, int nG, const int32_t* G_eq, const int32_t* G_exps,
                                const double* G_coef, int nF, const int32_t* F_eq, const int32_t* F_exps,
                                const double* F_coef, double gamma_re, double gamma_im, int64_t npaths,
                                const double* d_starts, int endgame, double t1_re, double t1_im, double t0_re,
                                double t0_im, hc_path_result* d_results, double* d_solutions, void* stream) {
  hc_handle* h = nullptr;  // errors go to the library-wide message
  if (!opts) return fail(h, HC_ERR_INVALID_ARG, "hc_track_noalloc: null options");
  if (opts->step_control == HC_STEP_LEARNED)
    return fail(h, HC_ERR_UNSUPPORTED, "hc_track_noalloc: learned step control needs a handle (hc_set_step_model)");
  if (opts->step_control != HC_STEP_PLAIN && opts->step_control != HC_STEP_EXPLORE)
    return fail(h, HC_ERR_INVALID_ARG, "hc_track_noalloc: unknown step control");
  if (invalid_knob(opts)) return fail(h, HC_ERR_INVALID_ARG, std::string("hc_track_noalloc: ") + invalid_knob(opts));
  {
    // The compiled tables are copied from a host buffer that lives only for this call; a
    // copy recorded into a graph would read it after it is freed. Checked before any other
    // CUDA call so that a refused call leaves the capture intact.
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    cudaError_t ce = cudaStreamIsCapturing((cudaStream_t)stream, &cs);
    if (ce != cudaSuccess) return cuda_fail(h, ce, "hc_track_noalloc: stream query");
    if (cs != cudaStreamCaptureStatusNone)
      return fail(h, HC_ERR_UNSUPPORTED,
                  "hc_track_noalloc: the stream is being captured; the tables are copied from a temporary host "
                  "buffer, so calls cannot be recorded into a graph");
  }
  if (n < 1 || n > 32) return fail(h, HC_ERR_UNSUPPORTED, "hc_track_noalloc: need 1 <= n <= 32");
  if (nG < 0 || nF < 0 || (nG > 0 && (!G_eq || !G_exps || !G_coef)) || (nF > 0 && (!F_eq || !F_exps || !F_coef)))
    return fail(h, HC_ERR_INVALID_ARG, "hc_track_noalloc: bad term table");
  if (!std::isfinite(gamma_re) || !std::isfinite(gamma_im))
    return fail(h, HC_ERR_INVALID_ARG, "hc_track_noalloc: gamma must be finite");
  if (npaths < 0) return fail(h, HC_ERR_INVALID_ARG, "hc_track_noalloc: npaths < 0");
  if (npaths == 0) return HC_OK;
  if (!d_starts || !d_results || !d_solutions) return fail(h, HC_ERR_INVALID_ARG, "hc_track_noalloc: null buffer");
  if (opts->precision != HC_PREC_FP64 && opts->precision != HC_PREC_MIXED)
    return fail(h, HC_ERR_INVALID_ARG, "hc_track_noalloc: unknown precision");
  HostProg P;
  std::string err;
  int rc = build_program(n, nG, G_eq, G_exps, G_coef, nF, F_eq, F_exps, F_coef, P, err);
  if (rc != HC_OK) return fail(h, rc, "hc_track_noalloc: " + err);
  WarpLayout L = make_warp_layout(P);
  TableLayout T = make_table_layout(P, opts->precision);
  // compiled tables: packed exactly as hc_set_homotopy packs them
  std::vector<char> blob;
  ProgOffsets po = pack_program(P, blob);
  if (blob.size() > HC_NOALLOC_MAX_PROGRAM_BYTES)
    return fail(h, HC_ERR_TOO_LARGE,
                "hc_track_noalloc: compiled homotopy needs " + std::to_string(blob.size()) +
                    " bytes, the static scratch holds " + std::to_string(HC_NOALLOC_MAX_PROGRAM_BYTES));
  unsigned char* scratch = nullptr;
  cudaError_t e = noalloc_scratch(&scratch);
  if (e != cudaSuccess) return cuda_fail(h, e, "hc_track_noalloc: cudaGetSymbolAddress");
  int dev = 0, sms = 0;
  e = cudaGetDevice(&dev);
  if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (e != cudaSuccess) return cuda_fail(h, e, "hc_track_noalloc: device query");
  cudaStream_t s = (cudaStream_t)stream;
  unsigned char* prog = scratch + HC_NOALLOC_HEADER_BYTES;
  e = cudaMemsetAsync(scratch, 0, HC_NOALLOC_HEADER_BYTES, s);
  if (e == cudaSuccess) e = cudaMemcpyAsync(prog, blob.data(), blob.size(), cudaMemcpyHostToDevice, s);
  if (e != cudaSuccess) return cuda_fail(h, e, "hc_track_noalloc: staging the tables");
  DevProg D = bind_program(P, po, (const char*)prog, gamma_re, gamma_im);
  Launch la{};
  la.P = D;
  la.O = *opts;
  la.L = L;
  la.T = T;
  la.npaths = npaths;
  la.starts = (const double2*)d_starts;
  la.res = d_results;
  la.sol = (double2*)d_solutions;
  la.val = nullptr;
  la.last = nullptr;
  la.mode = endgame ? 1 : 0;
  la.t1_re = t1_re;
  la.t1_im = t1_im;
  la.t0_re = t0_re;
  la.t0_im = t0_im;
  la.counter = (unsigned long long*)scratch;
  la.stats = (unsigned long long*)scratch + 1;
  la.cancel = (volatile int*)(scratch + 128);
  la.log = nullptr;
  la.log_count = nullptr;
  la.log_cap = 0;
  la.model = nullptr;
  la.phase = nullptr;
  const size_t smem_cap = 227 * 1024;
  int wpc = opts->warps_per_cta;
  if (wpc <= 0) {
    wpc = std::max(1, (int)std::min<size_t>(8, (smem_cap - T.bytes) / L.bytes));
    wpc = balanced_warps(wpc, opts->precision);
  }
  size_t smem = (size_t)T.bytes + (size_t)wpc * L.bytes;
  while (wpc > 1 && smem > smem_cap) {
    --wpc;
    smem = (size_t)T.bytes + (size_t)wpc * L.bytes;
  }
  if (smem > smem_cap) return fail(h, HC_ERR_TOO_LARGE, "hc_track_noalloc: working set exceeds shared memory");
  la.lockstep = lockstep_for(*opts, wpc, false, P.val_terms);
  int bps = 0;
  e = occupancy(opts->precision, wpc, smem, &bps);
  if (e != cudaSuccess) return cuda_fail(h, e, "hc_track_noalloc: occupancy");
  if (bps < 1) return fail(h, HC_ERR_TOO_LARGE, "hc_track_noalloc: kernel does not fit on an SM");
  if (opts->ctas_per_sm > 0) bps = std::min(bps, opts->ctas_per_sm);
  int64_t want = ((int64_t)npaths + wpc - 1) / wpc;
  int blocks = (int)std::min<int64_t>((int64_t)bps * sms, want);
  e = launch_track(la, blocks, wpc, s);
  if (e != cudaSuccess) return cuda_fail(h, e, "hc_track_noalloc: launch");
  return HC_OK;
}
