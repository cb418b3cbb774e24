// hc_track.cuh — one warp tracks one path of a straight-line homotopy.
//
// Every LANE of the warp executes the same control flow; scalar state is replicated in all
// lanes (all reductions are xor-butterflies, so every LANE gets bit-identical values) and
// vector element i lives with LANE i (n ≤ 32). Matrices, monomial values, Taylor series and
// the per-path vectors sit in this warp's slice of shared memory.
//
// The algorithm restates, routine by routine, the reference's
//   Tracker           src/tracker.jl:517-968
//   Predictor         src/predictor.jl:124-371
//   Newton corrector  src/newton_corrector.jl:55-286
//   MatrixWorkspace   src/linear_algebra.jl:88-885 (square case)
//   WeightedNorm      src/norm.jl:101-234
//   SegmentStepper    src/utils.jl:300-394
//   Valuation         src/valuation.jl:38-228
//   EndgameTracker    src/endgame_tracker.jl:260-721, 847-888
// with the same decisions, thresholds and state machine (factorized / scaled flags of the
// Jacobian workspace included). In HC_PREC_MIXED the corrector Jacobian, its LU and the
// predictor's Taylor coefficients are complex FP32; residuals, updates, condition numbers and
// all decisions stay FP64.
#pragma once
#include "hc_rtc.h"

// heavy routines are real calls: keeps the kernel compact (compile time and I-cache)
#define HC_NI __noinline__
#define LANE ((int)(threadIdx.x & 31))

#include "hc_dev.h"
#include "hc_types.cuh"

namespace hcd {

enum { PADE21 = 0, HERMITE = 1 };
enum { NEWT_CONVERGED = 0, NEWT_TERMINATED, NEWT_MAX_ITERS, NEWT_SINGULARITY };
enum {
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
enum {
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
  EC_terminated_unknown
};
__device__ __forceinline__ int ec_from_tc(int c) {  // src/endgame_tracker.jl:119-139
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

struct NewtonResult {
  int code;
  double accuracy;
  int iters;
  double omega, theta, mu_low, norm_dx0;
};

// SegmentStepper (src/utils.jl:300-394)
struct Stepper {
  c64 start, target;
  double absD, s, sp;
  bool forward;
  __device__ void init(c64 st, c64 tg) {
    start = st;
    target = tg;
    absD = cabs(tg - st);
    forward = cabs(st) < cabs(tg);
    s = sp = forward ? 0.0 : absD;
  }
  __device__ bool is_done() const { return forward ? s == absD : s == 0.0; }
  __device__ void step_success() { s = sp; }
  __device__ void propose(double ds) { sp = forward ? jmin(s + ds, absD) : jmax(s - ds, 0.0); }
  __device__ double dist_to_target() const { return forward ? absD - s : s; }
  __device__ double Ds() const { return forward ? sp - s : s - sp; }
  __device__ c64 t_at(double ss) const {
    if (forward) {
      if (ss == 0.0) return start;
      if (ss == absD) return target;
      return start + (ss / absD) * (target - start);
    } else {
      if (ss == absD) return start;
      if (ss == 0.0) return target;
      return target + (ss / absD) * (start - target);
    }
  }
  __device__ c64 t() const { return t_at(s); }
  __device__ c64 tp() const { return t_at(sp); }
  __device__ c64 Dt() const {
    return forward ? ((sp - s) / absD) * (target - start) : ((s - sp) / absD) * (target - start);
  }
};

static __device__ __noinline__ double h_fn(double a) { return 2 * a * (sqrt(4 * a * a + 1) - 2 * a); }

static __device__ __noinline__ c64 t_to_s_plane(c64 t, int m) {  // src/predictor.jl:338-351
  double r = fast_abs(t);
  if (t.im == 0.0 && t.re > 0) return C64(nthroot(r, m));
  double th = hc_atan2(t.im, t.re);
  th = fmod(th, 2 * M_PI);
  if (th < 0) th += 2 * M_PI;
  return nthroot(r, m) * cis(th / m);
}
__device__ __forceinline__ c64 cpow_int(c64 a, int k) {
  c64 r = C64(1.0);
  for (int i = 0; i < k; ++i) r = r * a;
  return r;
}

// ------------------------------------------------------------------------------------------
#ifdef HC_PHASE_CLOCKS
// profiling builds: adds the cycles of the enclosing scope to one phase counter (lane 0)
struct PhaseClock {
  unsigned long long* acc;
  long long t0;
#ifdef __CUDA_ARCH__
  __device__ explicit PhaseClock(unsigned long long* a) : acc(a), t0(clock64()) {}
  __device__ ~PhaseClock() {
    if ((threadIdx.x & 31) == 0) *acc += (unsigned long long)(clock64() - t0);
  }
#else
  __device__ explicit PhaseClock(unsigned long long* a) : acc(a), t0(0) {}
#endif
};
#define HC_PHASE(k) PhaseClock hc_phase_clock_(&ph[k])
#else
#define HC_PHASE(k)
#endif

template <bool MIXED>
struct PathTracker {
  using JT = typename std::conditional<MIXED, c32, c64>::type;

  const Launch* a;
  const DevProg* P;
  const hc_options* O;
  int n;
  // shared-memory regions of this warp
  // per-term tables staged in this CTA's shared memory
  const c64* vcoef64;
  const c32* vcoef32;
  const uint16_t* vmono;
  const uint32_t* jcode;
  const int2* mdef;
  c64* mono64;
  char* part;
  // areas of the FP64 working set that mixed precision rarely touches (double-double monomials
  // and partial sums, FP64 Taylor series, FP64 Jacobian partial sums): a global-memory slice
  // with the cold layout, else the same shared areas as mono64 / part
  char* mono_c;
  char* part_c;
  char* Ab;   // A and LU of the current Jacobian's arithmetic (Aprec): Ab64/LUb64 or Ab32/LUb32
  char* LUb;
  char *Ab64, *LUb64, *Ab32, *LUb32;
  c64* xJ;
  c64* dinv;  // reciprocals of U's diagonal, stored in the LU's arithmetic (c64 or c32)
  c32* v32;   // FP32 staging vectors (4 × vn)
  int* ipiv;
  // complex vectors
  c64 *x, *xh, *xb, *r, *s1, *tx0, *tx1, *tx2, *tx3, *ptx0, *ptx1, *u;
  c64 *sol, *lastp, *pred, *ppred, *smp;
  // real vectors
  double *w, *winv, *rs, *egrs, *egcs, *ais, *ait, *aia, *aic, *vx, *vtx, *dvx, *dvtx, *nu2, *nu1, *lx2, *lx1,
      *lxd2, *lxd1;

  // ---- MatrixWorkspace state (src/linear_algebra.jl:7-22)
  bool factorized, scaled;
  int Aprec;  // 64 or 32: arithmetic of the current A / LU
  bool j64;   // mixed precision only: this path fell back to an FP64 Jacobian
  bool omega_reseed;  // mixed precision: take ω from the first FP64 correction after the switch
  double pred_delta;  // relative correction of the last ẋ refinement step (≈ FP32 solve error)
  c64 tJ;     // t of the last Jacobian evaluation (its x is xJ)

  // ---- ToricHomotopy (src/homotopies/toric_homotopy.jl:9-35): the current path's weights w
  // and its coefficients u·t^w, cached for the t of the last evaluation (tc_t)
  bool toric;
  c64* tcoef;
  double *tpow, *tw;
  double tc_t;
  const c64* vc;  // value-term coefficients the rows read: vcoef64, or tcoef

  // ---- Predictor state (src/predictor.jl:72-103)
  int pmethod, porder, wnum;
  double trust_region, local_error, cond_H_xd;
  c64 pt, pprev_t, ps, pprev_s;
  double tx_norm[4];

  // ---- Corrector (src/newton_corrector.jl:35-53) and constant expressions of the step
  // control, evaluated once instead of once per step by every lane
  double ca, ch_a;
  double k_sq12ha;     // sqrt(1 - 2 h(a))                      newton!
  double k_a7;         // a^7                                   init_newton!
  double k_c1;         // sqrt(1 + 2 h(β_a a)) - 1              initial_step_size / update_stepsize!
  double k_c1half;     // sqrt(1 + 2 h(β_a a / 2)) - 1
  double k_hahalf;     // h(β_a a / 2)
  double k_tolacc;     // a^(2^min_newton_iters - 1) h(a)       check_terminated!
  double k_a7h, k_a5h; // a^7 h(a), a^5 h(a)                    update_precision!

  // ---- Tracker state (src/tracker.jl:307-338)
  Stepper ss;
  double Ds_prev, accuracy, omega, omega_prev, mu, tau, norm_dx0;
  bool extended_prec, used_extended_prec, refined_extended_prec, keep_extended_prec, use_strict_beta_tau;
  int tcode;
  long long accepted_steps, rejected_steps, last_steps_failed, ext_accepted_steps, ext_rejected_steps;

  // ---- EndgameTracker state (src/endgame_tracker.jl:177-215)
  int ecode;
  bool singular_endgame, jtz0, jtz1, eg_singular;
  int eg_wnum;  // 0 == nothing
  double eg_accuracy, eg_cond, last_t, singular_start;
  long long steps_eg, ext_steps_eg_start, singular_steps;
  double sample_times[3], sample_conds[3];
  int sidx[3];  // sample slot permutation
  double logt2, logt1;

  long long cur_path;

  // ---- learned / exploratory step proposals (options.step_control)
  float phi[HC_NFEAT];   // features that decided the current step's size
  bool phi_valid;
  float step_logf;       // log multiplier applied to the current step (0: plain rule)
  double ds_plain_cur;   // plain proposal of the current step
  unsigned acc_hist;     // 1 = accepted, newest in bit 0
  int cooldown;          // accepted steps to wait after a rejected learned proposal

  // ---- counters
  unsigned long long c_evalj, c_eval, c_evaldd, c_taylor, c_lu, c_solve, c_taylor64, c_switch64, c_learned,
      c_learned_rej;
#ifdef HC_PHASE_CLOCKS
  mutable unsigned long long ph[HC_NPHASE];
#endif

  // all 32 lanes call init with the same arguments (the object is one per warp, in shared memory)
  __device__ void init(const Launch* la, char* base, char* tbase) {
    a = la;
    P = &la->P;
    O = &la->O;
    n = P->n;
    const WarpLayout& L = la->L;
    const TableLayout& TL = la->T;
    vcoef64 = TL.vc64_global ? (const c64*)la->P.vcoef64 : (const c64*)(tbase + TL.vcoef64);
    vcoef32 = (const c32*)(tbase + TL.vcoef32);
    vmono = (const uint16_t*)(tbase + TL.vmono);
    jcode = (const uint32_t*)(tbase + TL.jcode);
    mdef = (const int2*)(tbase + TL.mdef);
    mono64 = (c64*)(base + L.mono);
    part = base + L.part;
    // the vectors a cold layout keeps in the warp's global slice: complex from sol on
    // (HC_NCVEC_COLD), real from egrs on (HC_NRVEC_COLD), and xJ
    c64* cv_end = nullptr;
    double* rv_end = nullptr;
    xJ = nullptr;
    Ab64 = LUb64 = nullptr;
    if (L.cold > 0 && la->cold) {
      char* cb = la->cold + (size_t)(blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5)) * (size_t)L.cold;
      mono_c = cb + L.cmono;
      part_c = cb + L.cpart;
      if (L.cvec >= 0) cv_end = (c64*)(cb + L.cvec);
      if (L.crvec >= 0) rv_end = (double*)(cb + L.crvec);
      if (L.cxj >= 0) xJ = (c64*)(cb + L.cxj);
      if (L.cA >= 0) Ab64 = cb + L.cA;
      if (L.cLU >= 0) LUb64 = cb + L.cLU;
    } else {
      mono_c = (char*)mono64;
      part_c = part;
    }
    Ab32 = base + L.A;
    LUb32 = base + L.LU;
    if (!Ab64) Ab64 = Ab32;
    if (!LUb64) LUb64 = LUb32;
    Ab = Ab64;
    LUb = LUb64;
    if (!xJ) xJ = (c64*)(base + L.xJ);
    ipiv = (int*)(base + L.ipiv);
    c64* cv = (c64*)(base + L.vec);
    const int vn = L.vn;
    x = cv + 0 * vn;
    xh = cv + 1 * vn;
    xb = cv + 2 * vn;
    r = cv + 3 * vn;
    s1 = cv + 4 * vn;
    tx0 = cv + 5 * vn;
    tx1 = cv + 6 * vn;
    tx2 = cv + 7 * vn;
    tx3 = cv + 8 * vn;
    ptx0 = cv + 9 * vn;
    ptx1 = cv + 10 * vn;
    u = cv + 11 * vn;
    static_assert(HC_NCVEC - HC_NCVEC_COLD == 12, "sol .. smp are the vectors a cold layout moves");
    if (!cv_end) cv_end = cv + 12 * vn;
    sol = cv_end + 0 * vn;
    lastp = cv_end + 1 * vn;
    pred = cv_end + 2 * vn;
    ppred = cv_end + 3 * vn;
    smp = cv_end + 4 * vn;  // 6 vectors
    double* rv = (double*)(base + L.rvec);
    w = rv + 0 * vn;
    rs = rv + 1 * vn;
    winv = rv + 2 * vn;
    static_assert(HC_NRVEC - HC_NRVEC_COLD == 3, "egrs .. lxd1 are the vectors a cold layout moves");
    if (!rv_end) rv_end = rv + 3 * vn;
    egrs = rv_end + 0 * vn;
    egcs = rv_end + 1 * vn;
    ais = rv_end + 2 * vn;
    ait = rv_end + 3 * vn;
    aia = rv_end + 4 * vn;
    aic = rv_end + 5 * vn;
    vx = rv_end + 6 * vn;
    vtx = rv_end + 7 * vn;
    dvx = rv_end + 8 * vn;
    dvtx = rv_end + 9 * vn;
    nu2 = rv_end + 10 * vn;
    nu1 = rv_end + 11 * vn;
    lx2 = rv_end + 12 * vn;
    lx1 = rv_end + 13 * vn;
    lxd2 = rv_end + 14 * vn;
    lxd1 = rv_end + 15 * vn;
    dinv = (c64*)(base + L.dinv);
    v32 = (c32*)(base + L.v32);
    toric = !MIXED && la->tor_w != nullptr && L.tor_n > 0;
    tcoef = (c64*)(base + L.tor);
    tpow = (double*)(tcoef + L.tor_n);
    tw = tpow + L.tor_n;
    tc_t = dNaN();
    vc = toric ? (const c64*)tcoef : vcoef64;
    factorized = scaled = false;
    Aprec = 64;
    j64 = false;
    ca = O->a;
    ch_a = h_fn(ca);
    k_sq12ha = sqrt(1 - 2 * ch_a);
    k_a7 = hc_pow(ca, 7.0);
    double ab = O->beta_a * O->a;
    k_c1 = sqrt(1 + 2 * h_fn(ab)) - 1;
    k_hahalf = h_fn(0.5 * ab);
    k_c1half = sqrt(1 + 2 * k_hahalf) - 1;
    k_tolacc = hc_pow(ca, (double)((1 << O->min_newton_iters) - 1)) * ch_a;
    k_a7h = hc_pow(ca, 7.0) * ch_a;
    k_a5h = hc_pow(ca, 5.0) * ch_a;
  }

  __device__ void reset_counters() {
    c_evalj = c_eval = c_evaldd = c_taylor = c_lu = c_solve = c_taylor64 = c_switch64 = 0;
    c_learned = c_learned_rej = 0;
#ifdef HC_PHASE_CLOCKS
    for (int k = 0; k < HC_NPHASE; ++k) ph[k] = 0;
#endif
  }

  // host cancel flag, read by lane 0 and broadcast so the warp stays converged
  __device__ __forceinline__ bool cancelled() const { return __shfl_sync(FULL, *a->cancel, 0) != 0; }

  // ---------------------------------------------------------------- small vector helpers
  __device__ __forceinline__ c64 ld(const c64* v) const { return LANE < n ? v[LANE] : C64(0.0); }
  __device__ __forceinline__ void st(c64* v, c64 val) const {
    if (LANE < n) v[LANE] = val;
  }
  __device__ __forceinline__ double ldr(const double* v) const { return LANE < n ? v[LANE] : 0.0; }
  __device__ __forceinline__ void str(double* v, double val) const {
    if (LANE < n) v[LANE] = val;
  }
  __device__ __forceinline__ c64 gamma() const { return C64(P->gamma_re, P->gamma_im); }

  // ---------------------------------------------------------------- norms (src/norm.jl)
  // ‖x‖ with weights w (w == nullptr: InfNorm), x given per LANE
  // (the weights are applied as reciprocals, kept in winv next to w)
  __device__ HC_NI double vnorm(c64 xi, const double* wv) const {
    HC_PHASE(PH_NORM);
    double d = 0.0;
    c64 q = xi;
    if (LANE < n && wv) q = xi * winv[LANE];
    if (LANE < n) d = abs2(q);
    double dmax = wseq_max_fast(d, LANE, n);
    double r = sqrt(dmax);
    if (isinf(r)) return wjmax(LANE < n ? cabs(q) : 0.0, LANE, n);
    return r;
  }
  // InfNorm distance (src/norm.jl:150-169) with its overflow branch (abs for the first
  // entry, abs2 for the others)
  __device__ HC_NI double inf_dist(c64 xi, c64 yi) const {
    c64 q = xi - yi;
    double d = LANE < n ? abs2(q) : 0.0;
    double dmax = wseq_max_fast(d, LANE, n);
    double r = sqrt(dmax);
    if (isinf(r)) return wjmax(LANE == 0 ? cabs(q) : (LANE < n ? abs2(q) : 0.0), LANE, n);
    return r;
  }
  __device__ HC_NI void norm_init(c64 xi) {  // src/norm.jl:101-113
    double point_norm = vnorm(xi, nullptr);
    if (LANE < n) {
      double wi = fast_abs(xi);
      if (wi < 1e-4 * point_norm)
        wi = 1e-4 * point_norm;
      else if (wi > 0x1p511 * point_norm)
        wi = 0x1p511 * point_norm;
      w[LANE] = jmax(wi, 1e-6);
      winv[LANE] = 1.0 / w[LANE];
    }
  }
  __device__ HC_NI void norm_update(c64 xi) {  // src/norm.jl:122-136
    double norm_x = vnorm(xi, w);
    if (LANE < n) {
      double wi = (fast_abs(xi) + w[LANE]) / 2;
      if (wi < 1e-4 * norm_x)
        wi = 1e-4 * norm_x;
      else if (wi > 0x1p511 * norm_x)
        wi = 0x1p511 * norm_x;
      if (isfinite(wi)) {
        w[LANE] = jmax(wi, 1e-6);
        winv[LANE] = 1.0 / w[LANE];
      }
    }
  }

  // ---------------------------------------------------------------- evaluation
  // monomial values (level by level; m = mono[parent] * x[var])
  __device__ HC_NI void eval_mono64(const c64* xv) {
    HC_PHASE(PH_MONO);
    __syncwarp();
    if (LANE == 0) mono64[0] = C64(1.0);
    for (int L = 1; L < P->nlev; ++L) {
      int b = __ldg(P->lev + L), e = __ldg(P->lev + L + 1);
      for (int m = b + LANE; m < e; m += 32) {
        int2 d = mdef[m];
        mono64[m] = mono64[d.x] * xv[d.y];
      }
      __syncwarp();
    }
  }
  // FP32 monomials for FP32 Jacobians: the chain of eval_mono64 in FP32 from x rounded once
  // (n conversions instead of one per monomial: FP64 conversions run on the FP64 pipe)
  __device__ HC_NI void eval_mono32(const c64* xv) {
    c32* m32 = (c32*)(mono64 + P->M);
    if (LANE < n) v32[LANE] = to32(xv[LANE]);
    if (LANE == 0) m32[0] = C32(1.f);
    __syncwarp();
    for (int L = 1; L < P->nlev; ++L) {
      int b = __ldg(P->lev + L), e = __ldg(P->lev + L + 1);
      for (int m = b + LANE; m < e; m += 32) {
        int2 d = mdef[m];
        m32[m] = m32[d.x] * v32[d.y];
      }
      __syncwarp();
    }
  }
  // sum of the partial slots of row r
  template <class T>
  __device__ __forceinline__ T row_sum(const DevRows& R, const T* pp, int rr) const {
    T acc;
    acc.re = acc.im = 0;
    int k1 = __ldg(R.row_slot + rr + 1);
    for (int k = __ldg(R.row_slot + rr); k < k1; ++k) acc = acc + pp[k];
    return acc;
  }
  // value rows on FP64 monomials: lane i < n returns F_i, G_i
  __device__ HC_NI void val_rows64(c64& Fi, c64& Gi) {
    HC_PHASE(PH_VALROWS);
    const DevRows& R = P->val;
    c64* pp = (c64*)part;
    int s0 = __ldg(R.lane_seg + LANE), s1e = __ldg(R.lane_seg + LANE + 1);
    for (int s = s0; s < s1e; ++s) {
      int4 g = __ldg(R.seg + s);
      c64 a0 = C64(0.0), a1 = a0, a2 = a0, a3 = a0;
      const int D = g.x;  // the segment's stride between consecutive terms
      int t = g.y;
      for (; t + 3 * D < g.z; t += 4 * D) {
        int m0 = vmono[t], m1 = vmono[t + D], m2 = vmono[t + 2 * D], m3 = vmono[t + 3 * D];
        c64 c0 = vc[t], c1 = vc[t + D], c2 = vc[t + 2 * D], c3 = vc[t + 3 * D];
        a0 = cfma(c0, mono64[m0], a0);
        a1 = cfma(c1, mono64[m1], a1);
        a2 = cfma(c2, mono64[m2], a2);
        a3 = cfma(c3, mono64[m3], a3);
      }
      for (; t < g.z; t += D) a0 = cfma(vc[t], mono64[vmono[t]], a0);
      pp[g.w & 0xffffff] = (a0 + a1) + (a2 + a3);
    }
    __syncwarp();
    Fi = Gi = C64(0.0);
    if (LANE < n) {
      Fi = row_sum(R, pp, LANE);
      Gi = row_sum(R, pp, n + LANE);
    }
    __syncwarp();
  }
  // Jacobian rows in arithmetic T → A = ts * J_G + tt * J_F. A Jacobian term's coefficient
  // is (segment multiplier) × (value-term coefficient).
  template <class T>
  __device__ HC_NI void jac_rows(c64 ts64, c64 tt64) {
    HC_PHASE(PH_JACROWS);
    const DevRows& R = P->jac;
    // FP32 partial sums: in the FP64 monomial area when the layout says so (val_rows64 has
    // consumed the FP64 monomials; the FP32 ones this reads lie above them)
    T* pp = std::is_same<T, c32>::value ? (a->L.jmono ? (T*)mono64 : (T*)part) : (T*)part_c;
    const T* mv;
    const T* cf;
    if constexpr (std::is_same<T, c64>::value) {
      mv = mono64;
      cf = vc;
    } else {
      mv = (const c32*)(mono64 + P->M);
      cf = vcoef32;
    }
    int s0 = __ldg(R.lane_seg + LANE), s1e = __ldg(R.lane_seg + LANE + 1);
    for (int s = s0; s < s1e; ++s) {
      int4 g = __ldg(R.seg + s);
      T a0, a1, a2, a3;
      a0.re = a0.im = 0;
      a1 = a2 = a3 = a0;
      const int D = g.x;
      int t = g.y;
      for (; t + 3 * D < g.z; t += 4 * D) {
        uint32_t k0 = jcode[t], k1 = jcode[t + D], k2 = jcode[t + 2 * D], k3 = jcode[t + 3 * D];
        a0 = cfma(cf[k0 >> 16], mv[k0 & 0xffff], a0);
        a1 = cfma(cf[k1 >> 16], mv[k1 & 0xffff], a1);
        a2 = cfma(cf[k2 >> 16], mv[k2 & 0xffff], a2);
        a3 = cfma(cf[k3 >> 16], mv[k3 & 0xffff], a3);
      }
      for (; t < g.z; t += D) {
        uint32_t k0 = jcode[t];
        a0 = cfma(cf[k0 >> 16], mv[k0 & 0xffff], a0);
      }
      T sum = (a0 + a1) + (a2 + a3);
      int mult = (g.w >> 24) & 0xff;
      if (mult != 1) sum = sum * (decltype(sum.re))mult;
      pp[g.w & 0xffffff] = sum;
    }
    __syncwarp();
    T* A = (T*)Ab;
    T ts = conv<T>(ts64), tt = conv<T>(tt64);
    int nn = n * n;
    if (toric) {
      for (int e = LANE; e < nn; e += 32) A[e] = row_sum(R, pp, e);
    } else {
      for (int e = LANE; e < nn; e += 32) {
        T f = row_sum(R, pp, e), gg = row_sum(R, pp, nn + e);
        A[e] = ts * gg + tt * f;
      }
    }
    __syncwarp();
  }

#ifdef HC_SLP
  // ---- a system given as a straight-line program: evaluators generated for it (hc_slp.cu)
  // G_i = s_i (x_i^{D_i} - 1) of the total-degree start system and dG_i/dx_i, lane i < n
  __device__ __forceinline__ void slp_start(c64 xi, c64& G, c64& dG) const {
    const int i = LANE < n ? LANE : 0;
    const int D = hcslp::slp_degree[i];
    const double s = hcslp::slp_scaling[i];
    const c64 p = hcslp::spow(xi, D - 1);
    G = s * (p * xi - C64(1.0));
    dG = (s * (double)D) * p;
  }
  // parameters of a parameter homotopy (p then q), unused otherwise
  __device__ __forceinline__ const c64* slp_pq() const { return (const c64*)a->slp_pq; }
  __device__ HC_NI void slp_H_eval(const c64* xv, c64 t, c64* out) {
    __syncwarp();
    c64 F;
    hcslp::eval_v<c64>(xv, slp_pq(), t, LANE, F);
    if (LANE < n) {
      if constexpr (hcslp::NP > 0) {
        out[LANE] = F;  // H(x, t) = F(x; t p + (1 - t) q)
      } else {
        c64 G, dG;
        slp_start(xv[LANE], G, dG);
        out[LANE] = (gamma() * t) * G + (C64(1.0) - t) * F;
      }
    }
    __syncwarp();
  }
  // residual r = H(x, t) in FP64 and the Jacobian in arithmetic T: lane j writes column j
  // (A is column-major, A[j n + i] = ∂H_i/∂x_j) from its forward-mode tangents
  template <class T>
  __device__ HC_NI void slp_H_eval_jac(const c64* xv, c64 t) {
    __syncwarp();
    const c64 ts = gamma() * t, tt = C64(1.0) - t;
    T Fi, col[hcslp::NV];
    hcslp::eval_vt<T>(xv, slp_pq(), t, LANE, Fi, col);
    c64 F64;
    if constexpr (std::is_same<T, c64>::value)
      F64 = Fi;
    else
      hcslp::eval_v<c64>(xv, slp_pq(), t, LANE, F64);
    T* A = (T*)Ab;
    if (LANE < n) {
      if constexpr (hcslp::NP > 0) {
        r[LANE] = F64;
#pragma unroll
        for (int i = 0; i < hcslp::NV; ++i) A[LANE * n + i] = col[i];
      } else {
        c64 G, dG;
        slp_start(xv[LANE], G, dG);
        r[LANE] = ts * G + tt * F64;
        const T tsT = conv<T>(ts), ttT = conv<T>(tt), dGT = conv<T>(dG);
#pragma unroll
        for (int i = 0; i < hcslp::NV; ++i) {
          T e = ttT * col[i];
          if (i == LANE) e = e + tsT * dGT;
          A[LANE * n + i] = e;
        }
      }
    }
    __syncwarp();
  }
  __device__ HC_NI void slp_H_eval_dd(const c64* xv, c64 t, c64* out) {
    __syncwarp();
    cdd F;
    hcslp::eval_v<cdd>(xv, slp_pq(), t, LANE, F);
    if (LANE < n) {
      if constexpr (hcslp::NP > 0) {
        out[LANE] = round_c(F);
      } else {
        const cdd s = cdd_of(C64(hcslp::slp_scaling[LANE]));
        const cdd G = s * hcslp::spow(cdd_of(xv[LANE]), hcslp::slp_degree[LANE]) - s;
        const cdd ts = cdd_of(gamma() * t), tt = cdd_of(C64(1.0) - t);
        out[LANE] = round_c(ts * G + tt * F);
      }
    }
    __syncwarp();
  }
  // taylor!: order K of H(x(s), t + s) with x(s) = Σ_{k<K} tx_k s^k (K = 1: ∂H/∂t, for the
  // straight-line homotopy γ G(x) - F(x))
  __device__ HC_NI void slp_H_taylor(int K, c64 t, c64* out) {
    __syncwarp();
    c64 Flo, Fhi;
    if (K == 1)
      hcslp::series1(tx0, tx1, tx2, slp_pq(), t, LANE, Flo, Fhi);
    else if (K == 2)
      hcslp::series2(tx0, tx1, tx2, slp_pq(), t, LANE, Flo, Fhi);
    else
      hcslp::series3(tx0, tx1, tx2, slp_pq(), t, LANE, Flo, Fhi);
    if constexpr (hcslp::NP > 0) {
      if (LANE < n) out[LANE] = Fhi;  // taylor!(u, v, F, tx, tp!(H, t)) (parameter_homotopy.jl:98-101)
      __syncwarp();
      return;
    }
    if (LANE < n) {
      // G_i along x_i(s): s_i (x_i(s)^D - 1), four orders by repeated truncated products
      const c64 z = C64(0.0);
      const c64 x0 = tx0[LANE], x1 = K > 1 ? tx1[LANE] : z, x2 = K > 2 ? tx2[LANE] : z;
      c64 p0 = C64(1.0), p1 = z, p2 = z, p3 = z;
      for (int d = 0; d < hcslp::slp_degree[LANE]; ++d) {
        const c64 q3 = p0 * z + p1 * x2 + p2 * x1 + p3 * x0;
        const c64 q2 = p0 * x2 + p1 * x1 + p2 * x0;
        const c64 q1 = p0 * x1 + p1 * x0;
        p0 = p0 * x0;
        p1 = q1;
        p2 = q2;
        p3 = q3;
      }
      const double sc = hcslp::slp_scaling[LANE];
      const c64 pw[4] = {p0 - C64(1.0), p1, p2, p3};
      const int lo = K == 1 ? 0 : K - 1, hi = K == 1 ? 0 : K;
      const c64 glo = sc * pw[lo], ghi = sc * pw[hi];
      if (K == 1)
        out[LANE] = gamma() * glo - Flo;
      else
        out[LANE] = gamma() * (glo + t * ghi) + ((C64(1.0) - t) * Fhi - Flo);
    }
    __syncwarp();
  }
#endif

  // H(x,t) (src/homotopies/straight_line_homotopy.jl:96-104) → out (vector)
  __device__ HC_NI void H_eval(const c64* xv, c64 t, c64* out) {
    HC_PHASE(PH_EVAL);
#ifdef HC_SLP
    slp_H_eval(xv, t, out);
    ++c_eval;
    return;
#endif
    if (toric) toric_coeffs(t.re);
    eval_mono64(xv);
    c64 F, G;
    val_rows64(F, G);
    if (toric) {
      st(out, F);  // toric: H(x, t) = F(x; u·t^w)
    } else {
      c64 ts = gamma() * t, tt = C64(1.0) - t;
      st(out, ts * G + tt * F);
    }
    ++c_eval;
  }
  // H and its Jacobian (:106-124) in arithmetic T for the Jacobian
  template <class T>
  __device__ HC_NI void H_eval_jac(const c64* xv, c64 t) {
    HC_PHASE(PH_EVALJ);
    // the A and LU of this arithmetic (the cold layout keeps the FP64 ones in global memory)
    Ab = std::is_same<T, c32>::value ? Ab32 : Ab64;
    LUb = std::is_same<T, c32>::value ? LUb32 : LUb64;
#ifdef HC_SLP
    slp_H_eval_jac<T>(xv, t);
#else
    if (toric) toric_coeffs(t.re);
    eval_mono64(xv);
    if constexpr (std::is_same<T, c32>::value) eval_mono32(xv);
    c64 F, G;
    val_rows64(F, G);
    c64 ts = gamma() * t, tt = C64(1.0) - t;
    if (toric)
      st(r, F);
    else
      st(r, ts * G + tt * F);
    jac_rows<T>(ts, tt);
#endif
    Aprec = std::is_same<T, c32>::value ? 32 : 64;
    st(xJ, ld(xv));
    tJ = t;
    ++c_evalj;
  }
  // double-double residual (:81-94), rounded to FP64 on store
  __device__ HC_NI void H_eval_dd(const c64* xv, c64 t, c64* out) {
    HC_PHASE(PH_DD);
#ifdef HC_SLP
    slp_H_eval_dd(xv, t, out);
    ++c_evaldd;
    return;
#endif
    if (toric) toric_coeffs(t.re);
    __syncwarp();
    cdd* md = (cdd*)mono_c;
    if (LANE == 0) md[0] = cdd_of(C64(1.0));
    for (int L = 1; L < P->nlev; ++L) {
      int b = __ldg(P->lev + L), e = __ldg(P->lev + L + 1);
      for (int m = b + LANE; m < e; m += 32) {
        int2 d = mdef[m];
        md[m] = md[d.x] * cdd_of(xv[d.y]);
      }
      __syncwarp();
    }
    const DevRows& R = P->val;
    cdd* pp = (cdd*)part_c;
    int s0 = __ldg(R.lane_seg + LANE), s1e = __ldg(R.lane_seg + LANE + 1);
    for (int s = s0; s < s1e; ++s) {
      int4 g = __ldg(R.seg + s);
      cdd acc = cdd_of(C64(0.0));
      for (int tt = g.y; tt < g.z; tt += g.x) acc = acc + cdd_of(vc[tt]) * md[vmono[tt]];
      pp[g.w & 0xffffff] = acc;
    }
    __syncwarp();
    if (LANE < n) {
      cdd F = cdd_of(C64(0.0)), G = cdd_of(C64(0.0));
      for (int k = __ldg(R.row_slot + LANE); k < __ldg(R.row_slot + LANE + 1); ++k) F = F + pp[k];
      for (int k = __ldg(R.row_slot + n + LANE); k < __ldg(R.row_slot + n + LANE + 1); ++k) G = G + pp[k];
      if (toric) {
        out[LANE] = round_c(F);
      } else {
        cdd ts = cdd_of(gamma() * t), tt = cdd_of(C64(1.0) - t);
        out[LANE] = round_c(ts * G + tt * F);
      }
    }
    __syncwarp();
    ++c_evaldd;
  }

  // coeffs! (src/homotopies/toric_homotopy.jl:147-180) for real t ≥ 0: c = u·t^w, t^w = exp(w log t)
  __device__ HC_NI void toric_coeffs(double t) {
    if (t == tc_t) return;
    __syncwarp();
    const int T = a->L.tor_n;
    const double lt = hc_log(t);
    for (int k = LANE; k < T; k += 32) {
      const double w = tw[k];
      const double p = (t == 0.0) ? (w == 0.0 ? 1.0 : 0.0) : hc_exp(w * lt);
      tpow[k] = p;
      tcoef[k] = vcoef64[k] * p;
    }
    tc_t = t;
    __syncwarp();
  }
  // taylor! of the toric homotopy (src/homotopies/toric_homotopy.jl:181-278): the K-th Taylor
  // coefficient of F(x(t+ε); c(t+ε)), u_i = Σ_k Σ_{j=0..K} c_k^(j) m_k^(K−j), with the
  // coefficient series c^(j) = u·binom(w, j)·t^(w−j) (K = 1: c' = w·c/t; t = 0: the limits the
  // reference takes) and the monomial series of orders 0..K (a toric program keeps all four
  // orders of every monomial)
  __device__ HC_NI void taylor_rows_toric(int K, double t, c64* out) {
    toric_coeffs(t);
    const c64* S = mono64;
    const DevRows& R = P->val;
    c64* pp = (c64*)part;
    const bool at0 = (t == 0.0);
    const double ti = 1.0 / t;
    int s0 = __ldg(R.lane_seg + LANE), s1e = __ldg(R.lane_seg + LANE + 1);
    for (int s = s0; s < s1e; ++s) {
      int4 g = __ldg(R.seg + s);
      c64 acc = C64(0.0);
      for (int k = g.y; k < g.z; k += g.x) {
        const c64* Sm = S + (int)vmono[k] * 4;
        const double w = tw[k];
        const c64 u0 = vcoef64[k];
        if (K == 1) {
          const c64 d = at0 ? (w == 1.0 ? u0 : C64(0.0)) : (w * tcoef[k]) * ti;
          acc = cfma(d, Sm[0], acc);
        } else {
          double pw[4];
          if (at0) {
            pw[0] = w < 1e-12 ? 1.0 : 0.0;
            pw[1] = (pw[0] == 0.0 && fabs(w - 1.0) <= 0x1p-26 * fmax(fabs(w), 1.0)) ? 1.0 : 0.0;
            pw[2] = pw[3] = 0.0;
          } else {
            pw[0] = tpow[k];
            pw[1] = w * pw[0] * ti;
            pw[2] = 0.5 * (w - 1) * pw[1] * ti;
            pw[3] = (w - 2) * pw[2] * ti / 3;
          }
#pragma unroll
          for (int j = 0; j < 4; ++j)
            if (j <= K) acc = cfma(u0 * pw[j], Sm[K - j], acc);
        }
      }
      pp[g.w & 0xffffff] = acc;
    }
    __syncwarp();
    if (LANE < n) out[LANE] = row_sum(R, pp, LANE);
    __syncwarp();
  }

  // Taylor series of the homotopy in arithmetic T.
  //   K == 1: u = γ G(x) − F(x)                                 (:130-137)
  //   K ≥ 2: u = γ(G_{K−1} + t G_K) + (1−t) F_K − F_{K−1}, x(ε) = Σ_{k<K} tx_k ε^k  (:138-154)
  // Series storage: monomials below the top degree keep orders 0..3 (stride 4); top-degree
  // monomials, which are nobody's parent, keep only the two orders the rows need.
  // Returns false when T is FP32 and the a-priori rounding bound of the rows
  // (2^-21 · Σ|terms|) exceeds 1e-3 · |u_i| for some i: the caller then recomputes in FP64.
  template <class T>
  __device__ HC_NI bool H_taylor(int K, c64 t, c64* out) {
    HC_PHASE(PH_TAYLOR);
#ifdef HC_SLP
    slp_H_taylor(K, t, out);  // FP64 series in both precisions
    c_taylor += K;
    return true;
#endif
    constexpr bool F32 = std::is_same<T, c32>::value;
    __syncwarp();
    T* S = F32 ? (T*)mono64 : (T*)mono_c;
    const int top = P->top;
    T* ST = S + 4 * top;
    const int lo = (K == 1) ? 0 : K - 1, hi = (K == 1) ? 0 : K;
    const c64* txv[3] = {tx0, tx1, tx2};
    const int vn = a->L.vn;
    if constexpr (F32) {
      // the series inputs rounded to FP32 once (not once per monomial)
      if (LANE < n)
        for (int k = 0; k < K && k < 3; ++k) v32[k * vn + LANE] = to32(txv[k][LANE]);
    }
    if (LANE == 0) {
      for (int k = 0; k < 4; ++k) {
        S[k].re = (k == 0) ? 1 : 0;
        S[k].im = 0;
      }
    }
    for (int L = 1; L < P->nlev; ++L) {
      int b = __ldg(P->lev + L), e = __ldg(P->lev + L + 1);
      for (int m = b + LANE; m < e; m += 32) {
        int2 d = mdef[m];
        T X[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          if (k < K) {
            if constexpr (F32)
              X[k] = v32[k * vn + d.y];
            else
              X[k] = txv[k][d.y];
          } else {
            X[k].re = X[k].im = 0;
          }
        }
        const T* Sp = S + d.x * 4;
        // a parent's orders up to hi feed its children; a top-degree monomial needs lo and hi only
        const bool parent = m < top;
        T c[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
          T acc;
          acc.re = acc.im = 0;
          if (parent ? k <= hi : (k == lo || k == hi)) {
#pragma unroll
            for (int j = 0; j <= k; ++j) acc = cfma(Sp[j], X[k - j], acc);
          }
          c[k] = acc;
        }
        if (parent) {
#pragma unroll
          for (int k = 0; k < 4; ++k) S[m * 4 + k] = c[k];
        } else {
          ST[(m - top) * 2] = c[lo];
          ST[(m - top) * 2 + 1] = c[hi];
        }
      }
      __syncwarp();
    }
    if constexpr (!F32) {
      if (toric) {
        taylor_rows_toric(K, t.re, out);
        c_taylor += K;
        return true;
      }
    }
    const DevRows& R = P->val;
    T* pp = F32 ? (T*)part : (T*)part_c;
    const T* cf;
    if constexpr (std::is_same<T, c64>::value)
      cf = vcoef64;
    else
      cf = vcoef32;
    int s0 = __ldg(R.lane_seg + LANE), s1e = __ldg(R.lane_seg + LANE + 1);
    for (int s = s0; s < s1e; ++s) {
      int4 g = __ldg(R.seg + s);
      T a0, a1, b0, b1;
      a0.re = a0.im = 0;
      a1 = b0 = b1 = a0;
      float e0 = 0.f, e1 = 0.f;
      const int D = g.x;
      int tt = g.y;
      for (; tt + D < g.z; tt += 2 * D) {
        int m0 = vmono[tt], m1 = vmono[tt + D];
        T c0 = cf[tt], c1 = cf[tt + D];
        const T* q0 = (m0 < top) ? S + m0 * 4 + lo : ST + (m0 - top) * 2;
        const T* q1 = (m1 < top) ? S + m1 * 4 + lo : ST + (m1 - top) * 2;
        int d0 = (m0 < top) ? hi - lo : 1, d1 = (m1 < top) ? hi - lo : 1;
        T v00 = q0[0], v01 = q0[d0], v10 = q1[0], v11 = q1[d1];
        a0 = cfma(c0, v00, a0);
        a1 = cfma(c0, v01, a1);
        b0 = cfma(c1, v10, b0);
        b1 = cfma(c1, v11, b1);
        if constexpr (F32) {
          float ac0 = fabsf(c0.re) + fabsf(c0.im), ac1 = fabsf(c1.re) + fabsf(c1.im);
          e0 += ac0 * (fabsf(v00.re) + fabsf(v00.im)) + ac1 * (fabsf(v10.re) + fabsf(v10.im));
          e1 += ac0 * (fabsf(v01.re) + fabsf(v01.im)) + ac1 * (fabsf(v11.re) + fabsf(v11.im));
        }
      }
      for (; tt < g.z; tt += D) {
        int m0 = vmono[tt];
        T c0 = cf[tt];
        const T* q0 = (m0 < top) ? S + m0 * 4 + lo : ST + (m0 - top) * 2;
        int d0 = (m0 < top) ? hi - lo : 1;
        T v00 = q0[0], v01 = q0[d0];
        a0 = cfma(c0, v00, a0);
        a1 = cfma(c0, v01, a1);
        if constexpr (F32) {
          float ac0 = fabsf(c0.re) + fabsf(c0.im);
          e0 += ac0 * (fabsf(v00.re) + fabsf(v00.im));
          e1 += ac0 * (fabsf(v01.re) + fabsf(v01.im));
        }
      }
      int slot = g.w & 0xffffff;
      pp[slot] = a0 + b0;
      pp[R.nslots + slot] = a1 + b1;
      if constexpr (F32) {
        float* pe = (float*)(pp + 2 * R.nslots);
        pe[slot] = e0;
        pe[R.nslots + slot] = e1;
      }
    }
    __syncwarp();
    double ratio = 0.0;
    if (LANE < n) {
      T F0 = row_sum(R, pp, LANE), F1 = row_sum(R, pp + R.nslots, LANE);
      T G0 = row_sum(R, pp, n + LANE), G1 = row_sum(R, pp + R.nslots, n + LANE);
      c64 g0 = to64(G0), g1 = to64(G1), f0 = to64(F0), f1 = to64(F1);
      c64 uu;
      if (K == 1)
        uu = gamma() * g0 - f0;
      else
        uu = gamma() * (g0 + t * g1) + ((C64(1.0) - t) * f1 - f0);
      out[LANE] = uu;
      if constexpr (F32) {
        const float* pe = (const float*)(pp + 2 * R.nslots);
        // the bound in FP32 (a magnitude estimate; FP64 adds would run on the FP64 pipe)
        auto asum = [&](const float* e, int rr) {
          float acc = 0.f;
          for (int k = __ldg(R.row_slot + rr); k < __ldg(R.row_slot + rr + 1); ++k) acc += e[k];
          return acc;
        };
        float AF0 = asum(pe, LANE), AF1 = asum(pe + R.nslots, LANE);
        float AG0 = asum(pe, n + LANE), AG1 = asum(pe + R.nslots, n + LANE);
        float gab = sqrtf((float)abs2(gamma()));
        float bound;
        if (K == 1) {
          bound = gab * AG0 + AF0;
        } else {
          float at = sqrtf((float)abs2(t)), a1t = sqrtf((float)abs2(C64(1.0) - t));
          bound = gab * (AG0 + at * AG1) + a1t * AF1 + AF0;
        }
        bound *= 0x1p-21f;
        float au = sqrtf((float)abs2(uu));
        float rf = (au > 0.f) ? bound / au : (bound > 0.f ? __int_as_float(0x7f800000) : 0.f);
        ratio = isnan(rf) ? dINF() : (double)rf;
      }
    }
    __syncwarp();
    c_taylor += K;
    if constexpr (F32) return wmax_plain(ratio) <= 1e-3;
    return true;
  }

  // ---------------------------------------------------------------- linear algebra
  __device__ HC_NI void updated() {  // src/linear_algebra.jl:88-98
    __syncwarp();
    int nn = n * n;
    if (Aprec == 64) {
      const c64* A = (const c64*)Ab;
      c64* LU = (c64*)LUb;
      for (int e = LANE; e < nn; e += 32) LU[e] = A[e];
    } else {
      const c32* A = (const c32*)Ab;
      c32* LU = (c32*)LUb;
      for (int e = LANE; e < nn; e += 32) LU[e] = A[e];
    }
    factorized = false;
    scaled = false;
    __syncwarp();
  }
  template <class T>
  __device__ HC_NI void lu_factor_T() {  // src/linear_algebra.jl:130-184
    T* A = (T*)LUb;
    __syncwarp();
    // pivot search in T's own precision: comparisons of FP32 magnitudes are exact, so the
    // pivots are those of an FP64 search on the same values, without FP64 instructions
    using R = decltype(T{}.re);
    T* dv = (T*)dinv;  // reciprocal pivots in T
    // the row interchanges composed into one permutation: lane i ends with the source row of
    // row i (stored with its inverse, so that each solve permutes with one shuffle)
    int perm = LANE;
    for (int k = 0; k < n; ++k) {
      R v = -1;
      if (LANE >= k && LANE < n) v = abs2(A[k * n + LANE]);
      R vk = __shfl_sync(FULL, v, k);
      int kp = k;
      R amax = vk;
      if (!isnan(vk)) {
        if constexpr (std::is_same<R, float>::value) {
          // non-negative FP32 magnitudes order like their bit patterns: one warp max-reduction
          // and the lowest candidate lane holding it (the same maximum and tie rule as below)
          const bool cand = LANE >= k && LANE < n && (LANE == k || !isnan(v));
          const unsigned key = cand ? __float_as_uint(v) : 0u;
          const unsigned mx = __reduce_max_sync(FULL, key);
          kp = __ffs(__ballot_sync(FULL, cand && key == mx)) - 1;
          amax = __uint_as_float(mx);
        } else {
          R bv = (LANE > k && LANE < n && !isnan(v)) ? v : (R)-1;
          if (LANE == k) bv = vk;
          int bi = (LANE >= k && LANE < n) ? LANE : 1 << 30;
#pragma unroll
          for (int o = 16; o; o >>= 1) {
            R ov = __shfl_xor_sync(FULL, bv, o);
            int oi = __shfl_xor_sync(FULL, bi, o);
            if (ov > bv || (ov == bv && oi < bi)) {
              bv = ov;
              bi = oi;
            }
          }
          kp = bi;
          amax = bv;
        }
      }
      if (kp != k) {
        const int pk = __shfl_sync(FULL, perm, k), pp = __shfl_sync(FULL, perm, kp);
        if (LANE == k) perm = pp;
        if (LANE == kp) perm = pk;
      }
      if (amax != (R)0) {
        if (kp != k) {
          if (LANE < n) {
            T tmp = A[LANE * n + k];
            A[LANE * n + k] = A[LANE * n + kp];
            A[LANE * n + kp] = tmp;
          }
          __syncwarp();
        }
        T Akk = A[k * n + k];
        auto d = Akk.re * Akk.re + Akk.im * Akk.im;
        auto id = (decltype(d))1 / d;
        T rec;
        rec.re = Akk.re * id;
        rec.im = -Akk.im * id;
        if (LANE > k && LANE < n) A[k * n + LANE] = A[k * n + LANE] * rec;
        if (LANE == 0) dv[k] = rec;
        __syncwarp();
      } else {
        // zero pivot column: U_kk = 0 and the solves divide by zero, as in the reference
        if (LANE == 0) {
          T one;
          one.re = 1;
          one.im = 0;
          dv[k] = div_fast(one, A[k * n + k]);
        }
        __syncwarp();
      }
      // trailing update, lane i over the rows below the pivot (column after column)
      if (LANE > k && LANE < n) {
        const T l = A[k * n + LANE];
        for (int j = k + 1; j < n; ++j) A[j * n + LANE] = cfms(l, A[j * n + k], A[j * n + LANE]);
      }
      __syncwarp();
    }
    unsigned char* pv = (unsigned char*)ipiv;
    if (LANE < n) {
      pv[LANE] = (unsigned char)perm;
      pv[32 + perm] = (unsigned char)LANE;
    }
    __syncwarp();
  }
  __device__ HC_NI void factorize() {
    HC_PHASE(PH_LU);
    if (Aprec == 64)
      lu_factor_T<c64>();
    else
      lu_factor_T<c32>();
    factorized = true;
    ++c_lu;
  }
  // pivot, unit lower, upper (src/linear_algebra.jl:268-316); b per LANE → x per LANE
  template <class T>
  __device__ HC_NI c64 lu_solve_T(c64 b64) {
    const T* A = (const T*)LUb;
    T b = shfl(conv<T>(b64), LANE < n ? (int)((const unsigned char*)ipiv)[LANE] : LANE);
    const T* dv = (const T*)dinv;
    for (int j = 0; j < n; ++j) {
      T xj = shfl(b, j);
      if (LANE > j && LANE < n) b = cfms(A[j * n + LANE], xj, b);
    }
    for (int j = n - 1; j >= 0; --j) {
      if (LANE == j) b = b * dv[j];
      T xj = shfl(b, j);
      if (LANE < j) b = cfms(A[j * n + LANE], xj, b);
    }
    ++c_solve;
    return LANE < n ? to64(b) : C64(0.0);
  }
  // adjoint solve (src/linear_algebra.jl:318-354)
  template <class T>
  __device__ HC_NI c64 lu_solve_adj_T(c64 b64) {
    const T* A = (const T*)LUb;
    T b = conv<T>(b64);
    const T* dv = (const T*)dinv;
    for (int j = 0; j < n; ++j) {  // ldiv_adj_upper!
      if (LANE == j) b = b * conj(dv[j]);
      T xj = shfl(b, j);
      if (LANE > j && LANE < n) b = b - conj(A[LANE * n + j]) * xj;
    }
    for (int i = n - 1; i >= 0; --i) {  // ldiv_adj_unit_lower!
      T xi = shfl(b, i);
      if (LANE < i) b = b - conj(A[LANE * n + i]) * xi;
    }
    b = shfl(b, LANE < n ? (int)((const unsigned char*)ipiv)[32 + LANE] : LANE);  // _inverse_ipiv!
    ++c_solve;
    return LANE < n ? to64(b) : C64(0.0);
  }
  __device__ c64 lu_solve(c64 b) { return Aprec == 64 ? lu_solve_T<c64>(b) : lu_solve_T<c32>(b); }
  __device__ c64 lu_solve_adj(c64 b) { return Aprec == 64 ? lu_solve_adj_T<c64>(b) : lu_solve_adj_T<c32>(b); }
  __device__ c64 A_at(int i, int j) const {
    return Aprec == 64 ? ((const c64*)Ab)[j * n + i] : to64(((const c32*)Ab)[j * n + i]);
  }

  // LA.ldiv!(x, WS, b) (src/linear_algebra.jl:389-408)
  __device__ HC_NI c64 ws_ldiv(c64 b) {
    if (n == 1) return LANE == 0 ? cdiv(b, A_at(0, 0)) : C64(0.0);
    if (!factorized) factorize();
    if (scaled) b = ldr(rs) * b;
    return lu_solve(b);
  }
  // skeel_row_scaling! (:432-459) of the current A with column weights c
  __device__ HC_NI void skeel_row_scaling(double* d, const double* c, double thr) {
    __syncwarp();
    // 2^-e as a bit pattern (exact; exp2 would run on the FP64 pipe)
    auto pow2neg = [](int e) -> double {
      int b = 1023 - e;
      return (b >= 1 && b <= 2046) ? __longlong_as_double((long long)b << 52) : exp2((double)-e);
    };
    // FP32 Jacobians with weights in FP32 range: the row sums in FP32 (only their binary
    // exponents are used); otherwise in FP64
    const double cl = LANE < n ? c[LANE] : 1.0;
    if (Aprec == 32 && __all_sync(FULL, cl > 1e-30 && cl < 1e30)) {
      const c32* A32 = (const c32*)Ab;
      const float cf = (float)cl;
      float di = 0.f;
      for (int j = 0; j < n; ++j) {
        float cj = __shfl_sync(FULL, cf, j);
        if (LANE < n) {
          c32 a = A32[j * n + LANE];
          di = fmaf(hypotf(a.re, a.im), cj, di);
        }
      }
      float m = wjmaxf(di, LANE, n);
      float sth = (float)thr + m;
      if (LANE < n) {
        int e = 0;
        frexpf(di, &e);
        if (!isfinite(di)) e = 0;
        d[LANE] = ((float)e < sth) ? 1.0 : pow2neg(e);
      }
      __syncwarp();
      return;
    }
    double di = 0.0;
    if (LANE < n)
      for (int j = 0; j < n; ++j) {
        double a2 = abs2(A_at(LANE, j));
        double av = (a2 > 1e-36 && a2 < 1e36) ? (double)sqrtf((float)a2) : sqrt(a2);
        di += av * c[j];
      }
    double m = wjmax(di, LANE, n);
    double s = thr + m;
    if (LANE < n) {
      int e = 0;
      frexp(di, &e);
      if (!isfinite(di)) e = 0;
      d[LANE] = (e < s) ? 1.0 : pow2neg(e);
    }
    __syncwarp();
  }
  __device__ HC_NI void apply_row_scaling() {  // :489-497
    __syncwarp();
    int nn = n * n;
    if (Aprec == 64) {
      c64* LU = (c64*)LUb;
      for (int e = LANE; e < nn; e += 32) LU[e] = LU[e] * rs[e % n];
    } else {
      // the scale factors rounded to FP32 once (staged in the fourth FP32 vector)
      float* rsf = (float*)(v32 + 3 * a->L.vn);
      if (LANE < n) rsf[LANE] = (float)rs[LANE];
      __syncwarp();
      c32* LU = (c32*)LUb;
      for (int e = LANE; e < nn; e += 32) LU[e] = LU[e] * rsf[e % n];
    }
    scaled = true;
    __syncwarp();
  }
  // ldiv!(x, J, b[, norm]) (:833-862)
  __device__ HC_NI c64 jac_ldiv(c64 b, const double* wv) {
    HC_PHASE(PH_SOLVE);
    if (wv && !factorized) {
      skeel_row_scaling(rs, wv, -30.0);
      apply_row_scaling();
    }
    return ws_ldiv(b);
  }
  // residual A x - b in double-double, x per LANE (mixed_precision_iterative_refinement!, :528-544)
  __device__ HC_NI double mp_refine_step(c64& xl, c64 b, const double* wv) {
    __syncwarp();
    cdd acc = cdd_of(C64(0.0));
    for (int j = 0; j < n; ++j) {
      c64 xj = shfl(xl, j);
      if (LANE < n) acc = acc + cdd_of(A_at(LANE, j)) * cdd_of(xj);
    }
    acc = acc - cdd_of(b);
    c64 rr = LANE < n ? round_c(acc) : C64(0.0);
    c64 dxl = ws_ldiv(rr);
    xl = xl - dxl;
    return vnorm(dxl, wv) / vnorm(xl, wv);
  }
  // fixed_precision_iterative_refinement! (:553-567)
  __device__ HC_NI double fp_refine_step(c64& xl, c64 b, const double* wv) {
    HC_PHASE(PH_REFINE);
    __syncwarp();
    c64 acc = C64(0.0);
    for (int j = 0; j < n; ++j) {
      c64 xj = shfl(xl, j);
      if (LANE < n) acc = acc + A_at(LANE, j) * xj;
    }
    acc = acc - b;
    c64 dxl = ws_ldiv(LANE < n ? acc : C64(0.0));
    xl = xl - dxl;
    return vnorm(dxl, wv) / vnorm(xl, wv);
  }
  // iterative_refinement! (:864-885)
  __device__ HC_NI double iterative_refinement(c64& xl, c64 b, const double* wv, double tol, int max_iters) {
    double delta = mp_refine_step(xl, b, wv);
    for (int i = 2; i <= max_iters; ++i) {
      double dp = mp_refine_step(xl, b, wv);
      if (dp < tol) return dp;
      if (dp > 0.5 * delta) return dp;
      delta = dp;
    }
    return delta;
  }
  // Higham estimator (:598-682)
  __device__ HC_NI double inverse_inf_norm_est(const double* dl, const double* dr) {
    if (!factorized) factorize();
    const double* rsv = scaled ? rs : nullptr;
    double xr = LANE < n ? 1.0 / n : 0.0;
    if (dr && LANE < n) xr /= dr[LANE];
    c64 y = lu_solve_adj(C64(xr));
    if (dl && LANE < n) y = y / dl[LANE];
    if (rsv && LANE < n) y = y * rsv[LANE];
    double g = wsum(LANE < n ? fast_abs(y) : 0.0);
    if (LANE < n) y = y / fast_abs(y);
    if (dl && LANE < n) y = y / dl[LANE];
    if (rsv && LANE < n) y = y / rsv[LANE];
    c64 z = lu_solve(LANE < n ? y : C64(0.0));
    xr = LANE < n ? (dr ? z.re / dr[LANE] : z.re) : 0.0;
    int k = 2;
    while (true) {
      // j = first index of max |x_i| (strict >)
      double av = LANE < n ? fabs(xr) : -1.0;
      int bi = LANE < n ? LANE : 1 << 30;
      double bv = av;
      double a0 = __shfl_sync(FULL, av, 0);
      if (isnan(a0)) {
        bv = -1.0;
        bi = (LANE == 0) ? 0 : 1 << 30;
      } else if (LANE > 0 && isnan(bv)) {
        bv = -1.0;
      }
#pragma unroll
      for (int o = 16; o; o >>= 1) {
        double ov = __shfl_xor_sync(FULL, bv, o);
        int oi = __shfl_xor_sync(FULL, bi, o);
        if (ov > bv || (ov == bv && oi < bi)) {
          bv = ov;
          bi = oi;
        }
      }
      int j = isnan(a0) ? 0 : bi;
      xr = (LANE == j) ? 1.0 : 0.0;
      if (dr && LANE < n) xr /= dr[LANE];
      y = lu_solve_adj(C64(xr));
      if (dl && LANE < n) y = y / dl[LANE];
      if (rsv && LANE < n) y = y * rsv[LANE];
      double gbar = g;
      g = wsum(LANE < n ? fast_abs(y) : 0.0);
      if (g <= gbar) {
        g = gbar;
        break;
      }
      if (LANE < n) y = y / fast_abs(y);
      if (dl && LANE < n) y = y / dl[LANE];
      if (rsv && LANE < n) y = y / rsv[LANE];
      z = lu_solve(LANE < n ? y : C64(0.0));
      xr = LANE < n ? (dr ? z.re / dr[LANE] : z.re) : 0.0;
      k += 1;
      double xinf = wjmax(fabs(xr), LANE, n);
      double xj = __shfl_sync(FULL, xr, j);
      if (xj == xinf || k > 2) break;
    }
    return nanmin(g, dINF());
  }
  // inf_norm (:684-707)
  __device__ HC_NI double inf_norm_mat(const double* dl, const double* dr) {
    __syncwarp();
    double ni = 0.0;
    if (LANE < n) {
      for (int j = 0; j < n; ++j) ni += dr ? fast_abs(A_at(LANE, j)) * dr[j] : fast_abs(A_at(LANE, j));
      if (dl) ni *= dl[LANE];
    }
    // sequential @fastmath max starting from -Inf
    double v = LANE < n ? ni : -dINF();
    int kn = wmax_int((LANE < n && isnan(v)) ? LANE : -1);
    if (kn == n - 1) return dNaN();
    return wmax_plain((LANE < n && LANE > kn) ? v : -dINF());
  }
  // cond of the current Jacobian (:745-774). FP64 decisions: an FP32 Jacobian is first
  // re-evaluated in FP64 at the point where it was last evaluated.
  __device__ HC_NI double ws_cond(const double* dl, const double* dr) {
    HC_PHASE(PH_COND);
    if (MIXED && Aprec == 32) {
      __syncwarp();
      H_eval_jac<c64>(xJ, tJ);
      updated();
    }
    if (n == 1) {
      double aa = cabs(A_at(0, 0));
      double d0 = dl ? dl[0] : 1.0, r0 = dr ? dr[0] : 1.0;
      if (!dl && !dr) return 1.0 / aa;
      if (!dl) return 1.0 / (aa * r0);
      if (!dr) return 1.0 / (d0 * aa);
      return 1.0 / (d0 * aa * r0);
    }
    return inverse_inf_norm_est(dl, dr) * inf_norm_mat(dl, dr);
  }
  // numerical rank, rtol 1e-14 (LA.rank in src/tracker.jl:711-737): one-sided Jacobi by LANE 0
  __device__ HC_NI int rank_rtol(double rtol) {
    __syncwarp();
    c64* B = (c64*)LUb;
    int nn = n * n;
    for (int e = LANE; e < nn; e += 32) B[e] = A_at(e % n, e / n);
    __syncwarp();
    int rnk = 0;
    if (LANE == 0) {
      for (int sweep = 0; sweep < 60; ++sweep) {
        bool rot = false;
        for (int p = 0; p < n - 1; ++p)
          for (int q = p + 1; q < n; ++q) {
            double al = 0, be = 0;
            c64 g = C64(0.0);
            for (int i = 0; i < n; ++i) {
              c64 ap = B[p * n + i], aq = B[q * n + i];
              al += abs2(ap);
              be += abs2(aq);
              g = g + conj(ap) * aq;
            }
            double ag = cabs(g);
            if (ag == 0.0 || ag <= 1e-15 * sqrt(al * be)) continue;
            rot = true;
            double zeta = (be - al) / (2.0 * ag);
            double tt = (zeta >= 0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1.0 + zeta * zeta));
            double cc = 1.0 / sqrt(1.0 + tt * tt), sn = cc * tt;
            c64 ph = g / ag;
            for (int i = 0; i < n; ++i) {
              c64 ap = B[p * n + i], aq = B[q * n + i];
              B[p * n + i] = cc * ap - sn * (conj(ph) * aq);
              B[q * n + i] = sn * (ph * ap) + cc * aq;
            }
          }
        if (!rot) break;
      }
      double smax = 0;
      for (int j = 0; j < n; ++j) {
        double sv = 0;
        for (int i = 0; i < n; ++i) sv += abs2(B[j * n + i]);
        smax = fmax(smax, sqrt(sv));
      }
      for (int j = 0; j < n; ++j) {
        double sv = 0;
        for (int i = 0; i < n; ++i) sv += abs2(B[j * n + i]);
        if (sqrt(sv) > rtol * smax) ++rnk;
      }
    }
    rnk = __shfl_sync(FULL, rnk, 0);
    factorized = false;  // the LU buffer was used as scratch
    __syncwarp();
    return rnk;
  }

  // ---------------------------------------------------------------- predictor
  // predictor Taylor coefficients: FP32 in mixed precision unless the FP32 rounding bound is
  // too large for this evaluation (then FP64) or the path already fell back to FP64
  __device__ __forceinline__ void taylor_path(int K, c64 t, c64* out) {
    if (MIXED && !j64) {
      if (!H_taylor<c32>(K, t, out)) {
        ++c_taylor64;
        H_taylor<c64>(K, t, out);
      }
    } else {
      H_taylor<c64>(K, t, out);
    }
  }
  __device__ void predictor_init() {  // src/predictor.jl:124-133
    cond_H_xd = 1.0;
    wnum = 1;
    pt = pprev_t = C64(dNaN(), 0.0);
    ps = pprev_s = C64(dNaN(), 0.0);
    trust_region = local_error = dNaN();
  }
  // :158-284 ; x = state x (vector), xhat may be nullptr
  __device__ HC_NI void predictor_update(c64 t, const c64* xhat) {
    int m = wnum;
    st(ptx0, ld(tx0));
    st(ptx1, ld(tx1));
    pprev_t = pt;
    pt = t;
    if (m > 1) {
      pprev_s = ps;
      ps = t_to_s_plane(t, m);
    }
    c64 xi = ld(x);
    double le0;
    if (!xhat) {
      le0 = dNaN();
    } else {
      double Ds = fast_abs(t - pprev_t);
      // norm(x̂, x): weighted distance
      double Ds2 = Ds * Ds;
      le0 = vnorm(ld(xhat) - xi, w) / (porder == 4 ? Ds2 * Ds2 : hc_pow(Ds, (double)porder));
    }
    predictor_compute(t, le0);
  }
  // Taylor coefficients x¹, x², x³ at the current (x, t) with the current Jacobian
  // factorization, trust region and local error (src/predictor.jl:202-284).
  // Mixed precision: the solves run on the FP32 LU; one refinement step with an FP64 residual
  // measures their relative error δ. Further refinement against an FP32 matrix cannot beat
  // its own rounding, so it is skipped; if δ > 1e-2 the FP32 Jacobian is unusable here and
  // the path switches to FP64 (Jacobian re-evaluated and refactored at x, coefficients redone).
  __device__ HC_NI void predictor_compute(c64 t, double le0) {
    HC_PHASE(PH_PREDICTOR);
    int m = wnum;
    c64 xi = ld(x);
    for (int attempt = 0; attempt < 2; ++attempt) {
      local_error = le0;
      const bool lu32 = MIXED && Aprec == 32;
      st(tx0, xi);
      tx_norm[0] = vnorm(xi, w);
      // ẋ
      taylor_path(1, t, u);
      c64 ul = -ld(u);
      c64 xt = jac_ldiv(ul, nullptr);
      double delta = fp_refine_step(xt, ul, w);
      cond_H_xd = delta / EPS;
      pred_delta = delta;
      if (lu32) {
        if (!(delta <= 1e-2)) {
          j64 = true;
          H_eval_jac<c64>(x, t);
          updated();
          continue;
        }
      } else if (delta > 1e-10) {
        iterative_refinement(xt, ul, nullptr, 1e-10, 5);
      }
      tx_norm[1] = vnorm(xt, w);
      st(tx1, xt);
      if (m > 1) {
        pmethod = HERMITE;
        porder = 4;
        trust_region = tx_norm[0] / tx_norm[1];
        if (isnan(local_error)) local_error = hc_pow(tx_norm[1] / tx_norm[0], 3.0);
        return;
      }
      taylor_path(2, t, u);
      ul = -ld(u);
      xt = jac_ldiv(ul, nullptr);
      if (!lu32 && delta > 1e-10) iterative_refinement(xt, ul, w, 1e-10, 4);
      tx_norm[2] = vnorm(xt, w);
      st(tx2, xt);
      taylor_path(3, t, u);
      ul = -ld(u);
      xt = jac_ldiv(ul, nullptr);
      if (!lu32 && delta > 1e-4) iterative_refinement(xt, ul, w, 1e-4, 3);
      tx_norm[3] = vnorm(xt, w);
      st(tx3, xt);
      break;
    }
    // trust region τ
    double taui = dINF();
    if (LANE < n) {
      double c1 = fast_abs(ld(tx1)), c2 = fast_abs(ld(tx2)), c3 = fast_abs(ld(tx3));
      double lam = jmax(1e-6, c1);
      c1 /= lam;
      c2 /= lam * lam;
      c3 /= lam * lam * lam;
      double tol = 1e-14 * jmax(c1, jmax(c2, c3));
      if (!((c1 <= tol && c2 <= tol && c3 <= tol) || c2 <= tol)) {
        double tv = (c2 / c3) / lam;
        if (!isnan(tv)) taui = tv;
      }
    }
#pragma unroll
    for (int o = 16; o; o >>= 1) taui = fmin(taui, __shfl_xor_sync(FULL, taui, o));
    double tau_ = taui;
    if (!isfinite(tau_)) tau_ = tx_norm[2] / tx_norm[3];
    if (!isfinite(tau_)) {
      double mx = jmax(jmax(tx_norm[0], tx_norm[1]), jmax(tx_norm[2], tx_norm[3]));
      tau_ = tx_norm[0] / mx;
    }
    pmethod = PADE21;
    porder = 4;
    trust_region = tau_;
    if (isnan(local_error)) {
      double it = 1.0 / tau_;
      local_error = (it * it) * (it * it);
    }
  }
  // :286-329
  __device__ HC_NI void predict(c64 t, c64 Dt) {
    HC_PHASE(PH_PREDICT);
    if (LANE >= n) return;
    c64 xi = tx0[LANE];
    if (pmethod == PADE21) {
      double lam = trust_region, lam2 = lam * lam, lam3 = lam * lam * lam;
      c64 x1 = tx1[LANE], x2 = tx2[LANE], x3 = tx3[LANE];
      double c = fast_abs(xi), c1 = fast_abs(x1), c2 = fast_abs(x2), c3 = fast_abs(x3);
      double a1 = c1 * lam, a2 = c2 * lam2, a3 = c3 * lam3;
      double tl = 1e-12 * sqrt(c * c + a1 * a1 + a2 * a2 + a3 * a3);
      if (c3 * lam3 <= tl || c2 * lam2 <= tl) {
        xh[LANE] = xi + Dt * (x1 + Dt * x2);
      } else {
        c64 di = C64(1.0) - cdiv(Dt * x3, x2);
        xh[LANE] = xi + Dt * (x1 + cdiv(Dt * x2, di));
      }
    } else {
      int m = wnum;
      c64 prev_s = t_to_s_plane(pprev_t, m), s = t_to_s_plane(t, m), sp = t_to_s_plane(t + Dt, m);
      c64 prev_sm, sm;
      if (m == 2) {
        prev_sm = 2.0 * prev_s;
        sm = 2.0 * s;
      } else {
        prev_sm = (double)m * cpow_int(prev_s, m - 1);
        sm = (double)m * cpow_int(s, m - 1);
      }
      xh[LANE] = cubic_hermite1(ptx0[LANE], prev_sm * ptx1[LANE], prev_s, xi, sm * tx1[LANE], s, sp);
    }
  }
  // cubic Hermite interpolation of one coordinate (src/predictor.jl:354-371)
  __device__ c64 cubic_hermite1(c64 y0, c64 yd0, c64 t0, c64 y1, c64 yd1, c64 t1, c64 tq) const {
    if (t0.im == 0.0 && t1.im == 0.0 && tq.im == 0.0) {
      double T0 = t0.re, T1 = t1.re, T = tq.re;
      double s = (T - T0) / (T1 - T0);
      double h00 = (1 + 2 * s) * ((1 - s) * (1 - s));
      double h10 = (T - T0) * ((1 - s) * (1 - s));
      double h01 = (s * s) * (3 - 2 * s);
      double h11 = (T - T0) * s * (s - 1);
      return h00 * y0 + h10 * yd0 + h01 * y1 + h11 * yd1;
    } else {
      c64 s = cdiv(tq - t0, t1 - t0);
      c64 one = C64(1.0), oms = one - s;
      c64 h00 = (one + 2.0 * s) * (oms * oms);
      c64 h10 = (tq - t0) * (oms * oms);
      c64 h01 = (s * s) * (C64(3.0) - 2.0 * s);
      c64 h11 = (tq - t0) * s * (s - one);
      return h00 * y0 + h10 * yd0 + h01 * y1 + h11 * yd1;
    }
  }

  // ---------------------------------------------------------------- Newton corrector
  // extended_prec_refinement_step! (src/newton_corrector.jl:55-78); xbar may alias xin
  __device__ HC_NI double ext_refine_step(c64* xbar, const c64* xin, c64 t, bool simple_newton_step) {
    H_eval_jac<c64>(xin, t);
    H_eval_dd(xin, t, r);
    updated();
    c64 rl = ld(r);
    c64 d = jac_ldiv(rl, w);
    iterative_refinement(d, rl, w, 1e-8, 3);
    c64 xn = ld(xin) - d;
    __syncwarp();
    st(xbar, xn);
    if (simple_newton_step) {
      H_eval_dd(xbar, t, r);
      d = jac_ldiv(ld(r), w);
    }
    return vnorm(d, w);
  }

  // newton! (:80-205); every iterate aliases x̄. JP = arithmetic of the Jacobian.
  template <class T>
  __device__ HC_NI NewtonResult newton(c64* xbar, const c64* x0v, c64 t, double mu_, double omega_, bool ext,
                                 bool accurate_mu, bool first_correction) {
    HC_PHASE(PH_NEWTON);
    const double a_ = ca, h_a = ch_a;
    c64 xi = ld(x0v);
    __syncwarp();
    st(xbar, xi);
    double mu_low = dNaN(), theta = dNaN(), norm_dxi = dNaN(), norm_dxim1 = dNaN(), norm_dx0 = dNaN();
    double abar = a_;
    double omega = omega_, mu = mu_;
    for (int i = 0; i <= 10; ++i) {
      H_eval_jac<T>(xbar, t);
      if (ext) H_eval_dd(xbar, t, r);
      updated();
      c64 rl = ld(r);
      c64 d = jac_ldiv(rl, w);
      if (ext) iterative_refinement(d, rl, w, abar * abar, 3);
      norm_dxi = vnorm(d, w);
      if (isnan(norm_dxi)) return NewtonResult{NEWT_SINGULARITY, norm_dxi, i + 1, omega, theta, mu_low, norm_dx0};
      xi = xi - d;
      st(xbar, xi);
      if (i == 0) norm_dx0 = norm_dxi;
      if (i == 1) omega = 2 * norm_dxi / (norm_dxim1 * norm_dxim1);
      if (i >= 1) theta = norm_dxi / norm_dxim1;
      if ((i >= 1 && theta > abar) || (i == 0 && !first_correction && 0.125 * norm_dx0 * omega > h_a)) {
        return NewtonResult{NEWT_TERMINATED, norm_dxi, i + 1, omega, theta, mu_low, norm_dx0};
      } else if (omega * norm_dxi * norm_dxi < 2 * mu * k_sq12ha) {
        H_eval_jac<T>(xbar, t);
        updated();
        rl = ld(r);
        if (ext) {
          c64 d2 = jac_ldiv(rl, nullptr);
          mu_low = vnorm(d2, w);
          H_eval_dd(xbar, t, r);
          rl = ld(r);
        }
        d = jac_ldiv(rl, nullptr);
        if (ext) iterative_refinement(d, rl, w, abar * abar, 3);
        xi = xi - d;
        st(xbar, xi);
        double norm_dxi1 = vnorm(d, w);
        if (isnan(norm_dxi1)) {
          return NewtonResult{NEWT_SINGULARITY, norm_dxi1, i + 1, omega, theta, mu_low, norm_dx0};
        } else if (norm_dxi1 > sqrt(norm_dxi)) {
          theta = norm_dxi1 / norm_dxi;
          return NewtonResult{NEWT_TERMINATED, norm_dxi1, i + 2, omega, theta, mu_low, norm_dx0};
        }
        if (norm_dxi1 > 2 * mu && ext) {
          H_eval_dd(xbar, t, r);
          d = jac_ldiv(ld(r), nullptr);
          norm_dxi = norm_dxi1;
          mu = norm_dxi1 = vnorm(d, w);
        } else if (norm_dxi1 > 2 * mu || accurate_mu) {
          H_eval(xbar, t, r);
          d = jac_ldiv(ld(r), nullptr);
          mu = vnorm(d, w);
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

  // init_newton! (:207-286) in FP64; x₁, x₂ alias x̄
  __device__ HC_NI void init_newton(bool& valid, double& omega_out, double& mu_out, const c64* x0v, c64 t, bool ext) {
    const double a_ = ca;
    H_eval_jac<c64>(x0v, t);
    if (ext) H_eval_dd(x0v, t, r);
    updated();
    c64 d = jac_ldiv(ld(r), w);
    double v = vnorm(d, w) + EPS;
    valid = false;
    double omega = dNaN(), mu = dNaN();
    double eps_ = sqrt(v);
    for (int k = 1; k <= 3; ++k) {
      c64 xbl = ld(x0v) + C64(eps_ * ldr(w));
      __syncwarp();
      st(xb, xbl);
      H_eval_jac<c64>(xb, t);
      if (ext) H_eval_dd(xb, t, r);
      updated();
      d = jac_ldiv(ld(r), w);
      xbl = xbl - d;
      st(xb, xbl);
      double norm_dx0_ = vnorm(d, w);
      if (ext)
        H_eval_dd(xb, t, r);
      else
        H_eval(xb, t, r);
      d = jac_ldiv(ld(r), w);
      xbl = xbl - d;
      st(xb, xbl);
      double norm_dx1 = vnorm(d, w) + EPS;
      if (norm_dx1 < a_ * norm_dx0_) {
        omega = 2 * norm_dx1 / (norm_dx0_ * norm_dx0_);
        mu = norm_dx1;
        double a7 = k_a7;
        if (omega * mu > a7) {
          NewtonResult rr = newton<c64>(xb, xb, t, a7 / omega, omega, ext, true, false);
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
        eps_ *= sqrt(eps_);
      }
    }
    omega_out = omega;
    mu_out = mu;
  }

  // ---------------------------------------------------------------- tracker
  __device__ long long steps() const { return accepted_steps + rejected_steps; }
  __device__ long long ext_steps() const { return ext_accepted_steps + ext_rejected_steps; }

  __device__ double initial_step_size() {  // src/tracker.jl:520-539
    int p = porder;
    double e = local_error;
    if (isinf(e)) e = 1e5;
    double Ds1 = nthroot(k_c1 / (omega * e), p) / O->beta_omega_p;
    double Ds2 = O->beta_tau * trust_region;
    double Ds = nanmin(Ds1, Ds2);
    return jmin(jmin(Ds, O->max_step_size), O->max_initial_step_size);
  }
  __device__ HC_NI void update_stepsize(const NewtonResult& res) {  // :541-588
    HC_PHASE(PH_STEPSIZE);
    int p = porder;
    double om = jclamp(omega + 2 * (omega - omega_prev), omega, 8 * omega);
    double Ds;
    if (res.code == NEWT_CONVERGED) {
      double e = local_error;
      double Ds1 = nthroot(k_c1 / (om * e), p) / O->beta_omega_p;
      double Ds2 = O->beta_tau * tau;
      if (use_strict_beta_tau || ss.dist_to_target() < Ds2) Ds2 = O->strict_beta_tau * tau;
      Ds = jmin(nanmin(Ds1, Ds2), O->max_step_size);
      if (use_strict_beta_tau && ss.dist_to_target() < Ds) Ds *= O->strict_beta_tau;
      Ds = jmin(Ds, 10 * Ds_prev);
      if (last_steps_failed > 0) Ds = jmin(Ds, Ds_prev);
    } else {
      int j = res.iters - 2;
      int N = (j >= 0 && j < 30) ? (1 << j) : 0;
      double Th = nthroot(res.theta, N);
      double hTh = h_fn(Th);
      double ha = k_hahalf;
      if (isnan(Th) || res.code == NEWT_SINGULARITY || isnan(res.accuracy) || res.iters == 1 || hTh < ha) {
        Ds = 0.25 * ss.Ds();
      } else {
        Ds = nthroot(k_c1half / (sqrt(1 + 2 * hTh) - 1), p) * ss.Ds();
      }
    }
    ss.propose(Ds);
  }
  __device__ HC_NI void check_terminated() {  // :591-619
    HC_PHASE(PH_STEPSIZE);
    double tol_acc;
    if (extended_prec || !O->extended_precision) {
      tol_acc = k_tolacc;
    } else {
      tol_acc = dINF();
    }
    c64 tp = ss.tp(), t = ss.t();
    double at = fast_abs(t);
    double eps_t = isinf(at) ? dNaN() : (nextafter(at, dINF()) - at);
    if (ss.is_done()) {
      tcode = TC_success;
    } else if (steps() >= O->max_steps) {
      tcode = TC_terminated_max_steps;
    } else if (omega * mu > tol_acc) {
      tcode = TC_terminated_accuracy_limit;
    } else if (ss.Ds() < O->min_step_size) {
      tcode = TC_terminated_step_size_too_small;
    } else if (fast_abs(tp - t) <= 2 * eps_t) {
      tcode = TC_terminated_step_size_too_small;
    } else if (O->min_rel_step_size > 0 && !(tp.re == ss.target.re && tp.im == ss.target.im) &&
               fast_abs(tp - t) < fast_abs(t) * O->min_rel_step_size) {
      tcode = TC_terminated_step_size_too_small;
    }
  }
  __device__ HC_NI void use_extended_precision() {  // :788-813
    if (!O->extended_precision) return;
    if (extended_prec) return;
    extended_prec = true;
    used_extended_prec = true;
    double m_ = mu;
    for (int i = 0; i < 2; ++i) m_ = ext_refine_step(x, x, ss.t(), false);
    mu = jmax(m_, EPS);
  }
  __device__ HC_NI void update_precision(double mu_low) {  // :768-786
    if (!O->extended_precision) return;
    if (extended_prec && !keep_extended_prec && !isnan(mu_low) && mu_low > mu) {
      if (mu_low * omega < k_a7h) {
        extended_prec = false;
        mu = mu_low;
      }
    } else if (mu * omega > k_a5h) {
      use_extended_precision();
    }
  }
  __device__ HC_NI double refine_current_solution(double min_tol, int nsteps) {  // :815-844
    double m_ = accuracy;
    c64 t = ss.t();
    double mub = ext_refine_step(xb, x, t, false);
    if (mub < m_) {
      st(x, ld(xb));
      m_ = mub;
    }
    int k = 1;
    while (m_ > min_tol && k <= nsteps) {
      mub = ext_refine_step(xb, x, t, true);
      if (mub < m_) {
        __syncwarp();
        st(x, ld(xb));
        m_ = mub;
      }
      k += 1;
    }
    __syncwarp();
    return m_;
  }

  // init! (:639-754); returns is_tracking
  // ω and μ given (not NaN) skip init_newton, as init!'s keywords do
  __device__ HC_NI bool tracker_init(c64 t1, c64 t0, double omega_in = dNaN(), double mu_in = dNaN()) {
    HC_PHASE(PH_INIT);
    phi_valid = false;
    step_logf = 0.f;
    ds_plain_cur = 0.0;
    acc_hist = 0xffu;
    cooldown = 0;
    j64 = false;
    omega_reseed = false;
    pred_delta = 0.0;
    ss.init(t1, t0);
    Ds_prev = 0.0;
    accuracy = EPS;
    omega = 1.0;
    keep_extended_prec = false;
    use_strict_beta_tau = false;
    refined_extended_prec = false;
    norm_init(ld(x));
    tcode = TC_tracking;
    accepted_steps = rejected_steps = ext_accepted_steps = ext_rejected_steps = 0;
    last_steps_failed = 0;
    c64 t = ss.t();
    bool valid = true;
    double om = omega_in, m_ = mu_in;
    bool ext = false;
    if (isnan(om) || isnan(m_)) {
      init_newton(valid, om, m_, x, t, false);
      if (!valid) {
        ext = true;
        init_newton(valid, om, m_, x, t, true);
      }
    }
    used_extended_prec = extended_prec = ext;
    if (!isnan(om)) omega = om;
    if (valid) {
      accuracy = m_;
      mu = jmax(m_, EPS);
    } else {
      H_eval_jac<c64>(x, t);
      bool anynan = false;
      for (int e = LANE; e < n * n; e += 32) anynan = anynan || isnanc(A_at(e % n, e / n));
      anynan = __any_sync(FULL, anynan);
      int corank = 0;
      if (!anynan) corank = n - rank_rtol(1e-14);
      tcode = corank > 0 ? TC_terminated_invalid_startvalue_singular_jacobian : TC_terminated_invalid_startvalue;
      return false;
    }
    tau = dINF();
    if (MIXED && !j64)
      H_eval_jac<c32>(x, t);
    else
      H_eval_jac<c64>(x, t);
    updated();
    predictor_init();
    predictor_update(ss.t(), nullptr);
    tau = trust_region;
    double Ds = initial_step_size();
    Ds = jmax(Ds, O->min_step_size);
    ss.propose(Ds);
    omega_prev = omega;
    return tcode == TC_tracking;
  }
  __device__ HC_NI void tracker_init_t0(c64 t0) {  // :756-766
    tcode = TC_tracking;
    ss.init(ss.t(), t0);
    double Ds = initial_step_size();
    ss.propose(Ds);
    Ds_prev = 0.0;
  }
  // step! (:851-926)
  __device__ HC_NI bool tracker_step() {
    HC_PHASE(PH_STEP);
    c64 t = ss.t(), Dt = ss.Dt(), tp = ss.tp();
    const bool logging = a->log && cur_path >= a->log_lo && cur_path < a->log_hi;
    double pre[8];
    if (logging) {
      pre[0] = ss.Ds();
      pre[1] = tau;
      pre[2] = local_error;
      pre[3] = omega;
      pre[4] = mu;
      pre[5] = vnorm(ld(x), nullptr);
      pre[6] = Ds_prev;
      pre[7] = trust_region;
    }
    predict(t, Dt);
    norm_update(ld(xh));
    NewtonResult res;
    if (MIXED && !j64 &&
        (ss.Ds() < 1e-6 * fast_abs(t) || pred_delta > 1e-3 || vnorm(ld(x), nullptr) > 1e4)) {
      // With an FP32 Jacobian Newton contracts only linearly (κ ≈ cond(J)·2^-23); the
      // quadratic model behind ω = 2‖Δx₁‖/‖Δx₀‖² then reads κ as curvature, ω grows as the
      // steps shrink and the steps shrink as ω grows. A tiny step relative to t, a predictor
      // solve error δ ≈ κ above 1e-3, or coordinates above 1e4 (FP32 loses range and accuracy
      // on |x|^d) move the path to FP64 for good.
      switch_to_fp64(t);
      predict(t, Dt);
    }
    if (MIXED && !j64) {
      res = newton<c32>(xb, xh, tp, mu, omega, extended_prec, false, accepted_steps == 0);
      if (res.code != NEWT_CONVERGED && step_logf <= 0.f) {
        // The FP32 Jacobian could not carry the correction: switch the path to FP64, redo the
        // predictor at the accepted point (its FP32 coefficients may be the culprit) and
        // retry this step with the same step size. A step enlarged beyond the plain proposal
        // (learned / explore step control) that fails is rejected instead: the step size, not
        // FP32, is the suspect, and the next attempt falls back to the plain proposal.
        switch_to_fp64(t);
        predict(t, Dt);
        res = newton<c64>(xb, xh, tp, mu, omega, extended_prec, false, accepted_steps == 0);
      }
    } else {
      res = newton<c64>(xb, xh, tp, mu, omega, extended_prec, false, accepted_steps == 0);
    }
    if (res.code == NEWT_CONVERGED) {
      __syncwarp();
      st(x, ld(xb));
      Ds_prev = ss.Ds();
      ss.step_success();
      accuracy = res.accuracy;
      mu = jmax(res.accuracy, EPS);
      omega_prev = omega;
      if (MIXED && omega_reseed) {
        omega = jmax(res.omega, 0.1);
        omega_reseed = false;
      } else {
        omega = jmax(jmax(res.omega, 0.5 * omega), 0.1);
      }
      update_precision(res.mu_low);
      if (ss.is_done() && O->extended_precision && accuracy > 1e-14) {
        accuracy = refine_current_solution(1e-14, 3);
        refined_extended_prec = true;
      }
      predictor_update(ss.t(), xh);
      tau = trust_region;
      accepted_steps += 1;
      ext_accepted_steps += extended_prec;
      last_steps_failed = 0;
    } else {
      rejected_steps += 1;
      ext_rejected_steps += extended_prec;
      last_steps_failed += 1;
    }
    norm_dx0 = res.norm_dx0;
    update_stepsize(res);
    if (O->step_control != HC_STEP_PLAIN) propose_next(res, t, logging, pre);
    else if (logging) log_step(t, pre, res);
    check_terminated();
    return last_steps_failed == 0;
  }

  // ---- learned / exploratory step proposals ---------------------------------------------
  // After a step, the plain rule (update_stepsize!, src/tracker.jl:541-588) has proposed Δs.
  //   explore: the proposal of the next step is multiplied by f = 6^u, u uniform from a hash of
  //            (path, step) — data for training;
  //   learned: f = exp(network(features)) ∈ [1, exp(logmax)];
  // both only while t > endgame_start when the endgame tracks the path (below).
  // A rejected enlarged proposal falls back to this step's plain proposal (then two accepted
  // plain steps before the next learned proposal); Newton's contraction test judges every step.
  // c_learned counts proposals the network enlarged, c_learned_rej those Newton rejected.
  __device__ HC_NI void propose_next(const NewtonResult& res, c64 t_prev, bool logging, const double* pre) {
    HC_PHASE(PH_STEPSIZE);
    const bool accepted = last_steps_failed == 0;
    acc_hist = (acc_hist << 1) | (accepted ? 1u : 0u);
    if (!accepted && step_logf > 0.f) {
      ss.propose(jmin(ds_plain_cur, ss.Ds()));
      if (O->step_control == HC_STEP_LEARNED) {
        ++c_learned_rej;
        cooldown = 2;
      }
    }
    if (logging) log_step(t_prev, pre, res);
    float lf = 0.f;
    bool valid = false;
    double dsp = ss.Ds();
    // Enlarged steps only before the endgame zone: for t < endgame_start the endgame samples
    // the path at every step (valuation, at-infinity and singular decisions), diverging paths
    // crowd together and the plain rule's step sequence is kept.
    const bool zone = a->mode != 1 || ss.t().re > O->endgame_start;
    if (accepted && !ss.is_done() && zone) {
      compute_features(res, dsp);
      valid = true;
      if (O->step_control == HC_STEP_EXPLORE) {
        unsigned long long z = (unsigned long long)cur_path * 0x9E3779B97F4A7C15ull + (unsigned long long)steps();
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        z ^= z >> 31;
        lf = (float)(uint32_t)(z >> 40) * 0x1p-24f * 1.7917595f;  // ln 6 · u, u uniform in [0, 1)
      } else if (O->step_control == HC_STEP_LEARNED && a->model) {
        if (cooldown > 0) {
          --cooldown;
        } else {
          lf = mlp_logf();
        }
      }
    }
    if (lf > 0.f) {
      // an enlarged step stays within 0.75 τ (β_τ of the reference's "fast" parameters,
      // src/tracker.jl:58-62), never below the plain proposal; the applied multiplier is kept
      double ds = jmin(dsp * (double)expf(lf), jmax(dsp, 0.75 * tau));
      ss.propose(ds);
      lf = logf((float)(ss.Ds() / dsp));
      if (!(lf > 0.f)) {
        lf = 0.f;
        ss.propose(dsp);
      } else if (O->step_control == HC_STEP_LEARNED) {
        ++c_learned;
      }
    }
    phi_valid = valid;
    step_logf = lf;
    ds_plain_cur = dsp;
  }
  // the 12 features of the step that was just accepted (all lanes hold the same values)
  __device__ HC_NI void compute_features(const NewtonResult& res, double dsp) {
    auto lg = [](double v) -> float {  // FP32 log: features are FP32 and clamped to ±40
      float l = log10f((float)v);
      if (!(l == l)) return 0.f;
      return fminf(40.f, fmaxf(-40.f, l));
    };
    double xnorm = vnorm(ld(x), nullptr);
    phi[0] = (float)ss.t().re;
    phi[1] = lg(Ds_prev);
    phi[2] = lg(tau);
    phi[3] = lg(fmax(res.theta == res.theta ? res.theta : 1e-20, 1e-20));
    phi[4] = lg(local_error);
    phi[5] = lg(xnorm);
    phi[6] = lg(omega);
    phi[7] = lg(dsp) - lg(tau);
    if (fabsf(phi[7]) >= 40.f || fabsf(lg(dsp)) >= 40.f || fabsf(lg(tau)) >= 40.f) phi[7] = lg(dsp / tau);
    phi[8] = (float)__popc(acc_hist & 0xffu) * 0.125f;
    phi[9] = (float)res.iters * 0.25f;
    phi[10] = lg(mu);
    phi[11] = lg(dsp);
  }
  // network inference: lane l computes hidden units l and l+32 (FP32 on BF16 weights)
  __device__ HC_NI float mlp_logf() {
    const StepModel* M = a->model;
    float xin[HC_NFEAT];
#pragma unroll
    for (int i = 0; i < HC_NFEAT; ++i) xin[i] = (phi[i] - M->mean[i]) * M->stdinv[i];
    auto bf = [](uint16_t v) { return __uint_as_float(((unsigned)v) << 16); };
    const int u0 = LANE, u1 = LANE + 32;
    float h0 = M->b1[u0], h1 = M->b1[u1];
#pragma unroll
    for (int i = 0; i < HC_NFEAT; ++i) {
      h0 += bf(M->W1T[i * 64 + u0]) * xin[i];
      h1 += bf(M->W1T[i * 64 + u1]) * xin[i];
    }
    h0 = fmaxf(h0, 0.f);
    h1 = fmaxf(h1, 0.f);
    float g0 = M->b2[u0], g1 = M->b2[u1];
#pragma unroll 4  // fully unrolled, this once-per-step loop is 20 KB of straight-line code
    for (int v = 0; v < 64; ++v) {
      float hv = __shfl_sync(FULL, v < 32 ? h0 : h1, v & 31);
      g0 += bf(M->W2T[v * 64 + u0]) * hv;
      g1 += bf(M->W2T[v * 64 + u1]) * hv;
    }
    g0 = fmaxf(g0, 0.f);
    g1 = fmaxf(g1, 0.f);
    float p1 = bf(M->W3[u0]) * g0 + bf(M->W3[u1]) * g1;
    float p2 = bf(M->W3[64 + u0]) * g0 + bf(M->W3[64 + u1]) * g1;
#pragma unroll
    for (int o = 16; o; o >>= 1) {
      p1 += __shfl_xor_sync(FULL, p1, o);
      p2 += __shfl_xor_sync(FULL, p2, o);
    }
    float o1 = p1 + M->b3[0], o2 = p2 + M->b3[1];
    float k = (o2 > 20.f ? o2 : log1pf(expf(o2))) + 0.05f;
    float lf = o1 - M->c / k;
    if (!(lf == lf)) return 0.f;
    return fminf(fmaxf(lf, 0.f), M->logmax);
  }
  // one record per attempted step (HC_LOG_FIELDS doubles), see include/hcgpu.h
  __device__ HC_NI void log_step(c64 t, const double* pre, const NewtonResult& res) {
    unsigned long long idx = 0;
    if (LANE == 0) idx = atomicAdd(a->log_count, 1ULL);
    idx = __shfl_sync(FULL, idx, 0);
    if (idx >= (unsigned long long)a->log_cap) return;
    double* rec = a->log + idx * HC_LOG_FIELDS;
    // fields 20..35: the features and multiplier that decided this step's size
    if (LANE < 16) {
      int f = 20 + LANE;
      double w2;
      if (LANE < HC_NFEAT)
        w2 = phi_valid ? (double)phi[LANE] : 0.0;
      else if (LANE == 12)
        w2 = step_logf;
      else if (LANE == 13)
        w2 = ds_plain_cur;
      else if (LANE == 14)
        w2 = phi_valid ? 1.0 : 0.0;
      else
        w2 = (double)O->step_control;
      rec[f] = w2;
    }
    double v = 0.0;
    switch (LANE) {
      case 0: v = (double)(cur_path + 1); break;
      case 1: v = t.re; break;
      case 2: v = t.im; break;
      case 3: v = pre[0]; break;
      case 4: v = pre[1]; break;
      case 5: v = pre[2]; break;
      case 6: v = pre[3]; break;
      case 7: v = pre[4]; break;
      case 8: v = last_steps_failed == 0 ? 1.0 : 0.0; break;
      case 9: v = res.iters; break;
      case 10: v = res.theta; break;
      case 11: v = res.norm_dx0; break;
      case 12: v = pre[5]; break;
      case 13: v = pre[6]; break;
      case 14: v = ss.Ds(); break;
      case 15: v = (double)((extended_prec ? 1 : 0) | (j64 ? 2 : 0) | (res.code << 2)); break;
      case 16: v = res.omega; break;
      case 17: v = res.accuracy; break;
      case 18: v = pre[7]; break;
      case 19: v = (double)accepted_steps; break;
      default: break;
    }
    if (LANE < 20) rec[LANE] = v;
  }
  // mixed precision: continue this path with an FP64 Jacobian, Taylor series and LU; the
  // predictor is recomputed at the accepted point and ω re-estimated by the next correction
  __device__ HC_NI void switch_to_fp64(c64 t) {
    j64 = true;
    omega_reseed = true;
    ++c_switch64;
    H_eval_jac<c64>(x, t);
    updated();
    predictor_compute(t, local_error);
    tau = trust_region;
  }
  // LA.cond(tracker, x, t, d_l, d_r) (src/tracker.jl:509-514), in FP64
  __device__ HC_NI double tracker_cond(const c64* xv, c64 t, const double* dl, const double* dr) {
    H_eval_jac<c64>(xv, t);
    updated();
    return ws_cond(dl, dr);
  }

  // ---------------------------------------------------------------- valuation
  __device__ void val_init() {  // src/valuation.jl:38-49
    double* vs[] = {vx, vtx, dvx, dvtx, nu2, nu1, lx2, lx1, lxd2, lxd1};
    for (int k = 0; k < 10; ++k) str(vs[k], 0.0);
    logt2 = logt1 = dNaN();
  }
  __device__ HC_NI void valuation_update(double t) {  // :82-124
    double logt = hc_log(t);
    bool diff = wnum > 1 && !isnan(logt2);
    if (LANE < n) {
      int i = LANE;
      c64 xi = tx0[i], xdi = tx1[i], x2i = tx2[i], x3i = tx3[i];
      double logxi = hc_log(fast_abs(xi)), logxdi = hc_log(fast_abs(xdi));
      auto fd = [](double nu, double s, double nu2_, double s2, double nu1_, double s1_) {
        double D1 = s - s1_, D2 = s - s2, D12 = s1_ - s2;
        return (D2 * nu1_) / (D12 * D1) - ((D12 + D2) * nu2_) / (D12 * D2) - (D12 * nu) / (D1 * D2);
      };
      if (diff) {
        double xx = abs2(xi);
        double nui = t * ((xi.re * xdi.re + xi.im * xdi.im) / xx);
        vx[i] = nui;
        dvx[i] = fd(nui, logt, nu2[i], logt2, nu1[i], logt1);
        double vxd = fd(logxdi, logt, lxd2[i], logt2, lxd1[i], logt1);
        double dvxd = fd(vxd, logt, 0.0, logt2, 0.0, logt1);
        vtx[i] = vxd + 1;
        dvtx[i] = dvxd;
      } else {
        auto nn1 = [](c64 X, c64 Xd, c64 X2, double tt, double& A, double& B) {
          double xx = abs2(X);
          double m_ = X.re * Xd.re + X.im * Xd.im;
          double l = m_ / xx;
          double m1 = X.re * X2.re + Xd.re * Xd.re + X.im * X2.im + Xd.im * Xd.im;
          double l1 = m1 / xx - 2 * l * l;
          A = tt * l;
          B = tt * l1 + l;
        };
        double nui, nu1v;
        nn1(xi, xdi, 2.0 * x2i, t, nui, nu1v);
        vx[i] = nui;
        dvx[i] = t * nu1v;
        double old = nu2[i];
        nu2[i] = nui;
        nu1[i] = old;
        double vxd;
        nn1(xdi, 2.0 * x2i, 6.0 * x3i, t, vxd, nu1v);
        vtx[i] = vxd + 1;
        dvtx[i] = t * nu1v;
      }
      double o = lx2[i];
      lx2[i] = logxi;
      lx1[i] = o;
      o = lxd2[i];
      lxd2[i] = logxdi;
      lxd1[i] = o;
    }
    logt1 = logt2;
    logt2 = logt;
    __syncwarp();
  }
  // at_infinity_tol! (:143-173) for LANE's coordinate
  __device__ double at_infinity_tol1(double finite_tol, bool zero_is_finite) const {
    if (LANE >= n) return dINF();
    double v = vx[LANE];
    double a1 = fabs(1.0 - vtx[LANE] / v), a2 = fabs(dvx[LANE] / v), a3 = fabs(dvtx[LANE] / vtx[LANE]);
    double e = jmax(jmax(a1, a2), a3);
    if (isnan(e)) return dINF();
    if (v + e < -finite_tol) return e;
    if (!zero_is_finite && v - e > -finite_tol) return e;
    return dINF();
  }
  __device__ HC_NI bool val_is_finite(double finite_tol, bool zero_is_finite, int max_wn) const {  // :175-205
    double delta = 1.0 / max_wn;
    bool ok = true;
    if (LANE < n) {
      double v = vx[LANE];
      if (fabs(v) < finite_tol) {
        if (!(fabs(dvx[LANE]) < finite_tol) || vtx[LANE] < 0.5 * delta) ok = false;
      } else if (zero_is_finite && v > (delta - finite_tol)) {
        double a1 = fabs(1.0 - vtx[LANE] / v), a2 = fabs(dvx[LANE] / v), a3 = fabs(dvtx[LANE] / vtx[LANE]);
        double e = jmax(jmax(a1, a2), a3);
        if (!(e < finite_tol)) ok = false;
      } else {
        ok = false;
      }
    }
    return __all_sync(FULL, ok);
  }
  __device__ HC_NI void estimate_winding_number(int max_wn, int& m, double& err_out) const {  // :207-228
    m = 1;
    double min_err = dINF();
    double vt = LANE < n ? vtx[LANE] : 0.0;
    for (int k = 1; k <= max_wn; ++k) {
      double mv = k * vt;
      double ei = LANE < n ? fabs(rint(mv) - mv) : 0.0;
      // err = max over lanes ignoring NaN (ifelse(errᵢ > err, errᵢ, err) from 0)
      double e2 = (isnan(ei) ? 0.0 : ei);
      double err = wmax_plain(e2);
      if (err < min_err) {
        m = k;
        min_err = err;
      }
    }
    err_out = min_err;
  }

  // ---------------------------------------------------------------- endgame
  __device__ c64* sample_val(int k) { return smp + (2 * sidx[k]) * a->L.vn; }
  __device__ c64* sample_der(int k) { return smp + (2 * sidx[k] + 1) * a->L.vn; }

  __device__ HC_NI void eg_init(double t1) {  // src/endgame_tracker.jl:260-294
    tracker_init(C64(t1), C64(0.0));
    ecode = ec_from_tc(tcode);
    singular_endgame = false;
    jtz0 = jtz1 = false;
    val_init();
    eg_wnum = 0;
    st(sol, C64(dNaN(), dNaN()));
    eg_accuracy = dNaN();
    eg_cond = dNaN();
    eg_singular = false;
    steps_eg = 0;
    ext_steps_eg_start = 0x7fffffffffffffffLL;
    str(egrs, 1.0);
    str(egcs, 1.0);
    str(ais, dNaN());
    singular_steps = 0;
    sidx[0] = 0;
    sidx[1] = 1;
    sidx[2] = 2;
    last_t = dNaN();
    __syncwarp();
  }
  __device__ HC_NI void tracking_stopped() {  // :695-721
    eg_accuracy = accuracy;
    if (ecode == EC_success && eg_accuracy > 1e-14) refine_current_solution(1e-14, O->refine_steps);
    __syncwarp();
    st(sol, ld(x));
    eg_wnum = 0;
    if (ecode == EC_success) {
      str(egcs, ldr(w));
      skeel_row_scaling(egrs, egcs, O->scaling_threshold);
      eg_cond = tracker_cond(sol, C64(0.0), egrs, egcs);
      eg_singular = eg_cond > O->sing_cond || eg_accuracy > O->sing_accuracy;
    }
  }
  __device__ HC_NI bool check_finite() {  // :402-422
    if (!val_is_finite(O->val_finite_tol, !O->zero_is_at_infinity, O->max_winding_number)) return false;
    int m;
    double merr;
    estimate_winding_number(O->max_winding_number, m, merr);
    if (merr < O->val_finite_tol) {
      if (m == 1 && !jtz0) return false;
      eg_wnum = m;
      return true;
    }
    return false;
  }
  __device__ HC_NI bool check_at_infinity() {  // :424-499
    if (!O->at_infinity_check) return false;
    double my_tol = at_infinity_tol1(O->val_finite_tol, !O->zero_is_at_infinity);
    str(ait, my_tol);
    __syncwarp();
    double kappa = dNaN();
    double t = ss.t().re;
    for (int i = 0; i < n; ++i) {
      double toli = ait[i];
      if (toli < O->val_at_infinity_tol) {
        if (MIXED && !j64) switch_to_fp64(ss.t());
        if (isnan(ais[i])) {
          bool allnan = __all_sync(FULL, LANE >= n || isnan(ais[LANE]));
          if (allnan) {
            str(egcs, ldr(w));
            skeel_row_scaling(egrs, egcs, O->scaling_threshold);
          }
          kappa = ws_cond(egrs, egcs);
          __syncwarp();
          if (LANE == 0) {
            aic[i] = kappa;
            aia[i] = fast_abs(x[i]);
            ais[i] = t;
          }
          __syncwarp();
        } else {
          if (isnan(kappa)) kappa = ws_cond(egrs, egcs);
          double vi = vx[i];
          bool at_zero = vx[i] > 0;
          double cond_growth = kappa / aic[i];
          double coord_growth = at_zero ? aia[i] / fast_abs(x[i]) : fast_abs(x[i]) / aia[i];
          double lim = jclamp(hc_pow(0.25, 4 * vi), 20.0, O->min_coord_growth);
          if (coord_growth > lim && (cond_growth > O->min_cond_growth || kappa > jmax(1e8, O->min_cond))) {
            ecode = at_zero ? EC_at_zero : EC_at_infinity;
            return true;
          }
        }
      } else if (!isnan(ais[i])) {
        __syncwarp();
        if (LANE == 0) ais[i] = dNaN();
        __syncwarp();
      }
    }
    return false;
  }
  __device__ HC_NI void add_sample(double t) {  // :630-662
    int m = eg_wnum;
    double s = nthroot(t, m);
    double mu_ = m * hc_pow(s, (double)(m - 1));
    double kappa = ws_cond(egrs, egcs);
    int k;
    if (singular_steps <= 2) {
      k = (int)singular_steps;
    } else {
      int t0 = sidx[0];
      sidx[0] = sidx[1];
      sidx[1] = sidx[2];
      sidx[2] = t0;
      sample_times[0] = sample_times[1];
      sample_conds[0] = sample_conds[1];
      sample_times[1] = sample_times[2];
      sample_conds[1] = sample_conds[2];
      k = 2;
    }
    __syncwarp();
    st(sample_val(k), ld(tx0));
    st(sample_der(k), mu_ * ld(tx1));
    sample_times[k] = s;
    sample_conds[k] = kappa;
    __syncwarp();
  }
  __device__ HC_NI double predict_endpoint() {  // :664-693
    if (singular_steps < 2) return dINF();
    __syncwarp();
    if (LANE < n) {
      if (singular_steps == 2)
        pred[LANE] = cubic_hermite1(sample_val(0)[LANE], sample_der(0)[LANE], C64(sample_times[0]),
                                    sample_val(1)[LANE], sample_der(1)[LANE], C64(sample_times[1]), C64(0.0));
      ppred[LANE] = pred[LANE];
      pred[LANE] = cubic_hermite1(sample_val(1)[LANE], sample_der(1)[LANE], C64(sample_times[1]),
                                  sample_val(2)[LANE], sample_der(2)[LANE], C64(sample_times[2]), C64(0.0));
    }
    __syncwarp();
    double p = sample_times[2] / sample_times[1];
    double err = inf_dist(ld(pred), ld(ppred)) / fabs((p * p) * (p * p) - 1);
    double norm_s = vnorm(ld(pred), nullptr);
    if (norm_s > 1e-8) err /= norm_s;
    return err;
  }
  __device__ HC_NI void switch_to_singular() {  // :501-524
    if (MIXED && !j64) switch_to_fp64(ss.t());
    singular_endgame = true;
    double t = ss.t().re;
    singular_start = t;
    bool allone = __all_sync(FULL, LANE >= n || egrs[LANE] == 1.0);
    if (allone) {
      str(egcs, ldr(w));
      skeel_row_scaling(egrs, egcs, O->scaling_threshold);
    }
    add_sample(t);
    singular_steps = 0;
    wnum = eg_wnum;
    __syncwarp();
    if (LANE == 0) aic[0] = sample_conds[0];
    __syncwarp();
    keep_extended_prec = true;
  }
  __device__ HC_NI void switch_to_regular() {  // :525-530
    singular_endgame = false;
    wnum = 1;
    tracker_init_t0(C64(0.0));
  }
  __device__ HC_NI int singular_endgame_step() {  // :533-628
    const double lambda = 0.25;
    double t = ss.t().re;
    tracker_init_t0(C64(lambda * t));
    bool max_steps = false;
    while (tcode == TC_tracking) {
      tracker_step();
      if ((steps_eg += 1) >= O->max_endgame_steps) {
        ecode = EC_terminated_max_steps;
        max_steps = true;
        break;
      } else if (ext_steps() - ext_steps_eg_start > O->max_endgame_extended_steps) {
        ecode = EC_terminated_max_extended_steps;
        max_steps = true;
        break;
      }
      if (cancelled()) return ecode = EC_terminated_unknown;
    }
    singular_steps += 1;
    if (!max_steps) {
      if (tcode != TC_success) {
        ecode = ec_from_tc(tcode);
        tracking_stopped();
        return ecode;
      }
      valuation_update(lambda * t);
      int mh;
      double mh_err;
      estimate_winding_number(O->max_winding_number, mh, mh_err);
      if (mh != eg_wnum || mh_err > 0.1) {
        switch_to_regular();
        return ecode;
      }
      add_sample(lambda * t);
      if (singular_steps < 2) return ecode;
      double acc = predict_endpoint();
      if (singular_steps == 2) {
        eg_accuracy = acc;
        st(sol, ld(pred));
        return ecode;
      } else if (acc < eg_accuracy && eg_accuracy > 1e-12) {
        eg_accuracy = acc;
        st(sol, ld(pred));
        return ecode;
      }
    }
    int m = eg_wnum;
    double kappa = sample_conds[2];
    double zero_cond = 1.0 / (m + 1);
    __syncwarp();
    if (LANE < n) sol[LANE] = (vx[LANE] < zero_cond) ? pred[LANE] : C64(0.0);
    __syncwarp();
    double kappa0 = tracker_cond(sol, C64(0.0), egrs, egcs);
    double J0_norm = inf_norm_mat(egrs, nullptr);
    if (eg_accuracy < O->singular_min_accuracy &&
        (((m > 1 && kappa > O->min_cond && nanmax(kappa0, 1.0 / J0_norm) > kappa) || (m == 1 && kappa0 > 1e12)) ||
         max_steps || (n == 1 && 1.0 / J0_norm < O->min_cond))) {
      eg_cond = jmax(kappa0, 1.0 / J0_norm);
      eg_singular = true;
      return ecode = EC_success;
    } else if (!max_steps) {
      switch_to_regular();
      return ecode;
    }
    return ecode;
  }
  __device__ HC_NI int eg_step() {  // :329-399
    HC_PHASE(PH_ENDGAME);
    if (steps_eg >= O->max_endgame_steps) {
      return ecode = EC_terminated_max_steps;
    } else if (ext_steps() - ext_steps_eg_start > O->max_endgame_extended_steps) {
      bool allfin = __all_sync(FULL, LANE >= n || !isnanc(sol[LANE]));
      if (allfin && eg_wnum != 0 && eg_accuracy < O->singular_min_accuracy) {
        eg_cond = tracker_cond(sol, C64(0.0), egrs, egcs);
        eg_singular = true;
        return ecode = EC_success;
      }
      return ecode = EC_terminated_max_extended_steps;
    }
    st(lastp, ld(x));
    last_t = ss.t().re;
    if (singular_endgame) return singular_endgame_step();
    c64 tp = ss.tp();
    bool is_jump_to_zero = (tp.re == 0.0 && tp.im == 0.0);
    bool step_success = tracker_step();
    ecode = ec_from_tc(tcode);
    if (ecode != EC_tracking) {
      tracking_stopped();
      return ecode;
    }
    jtz0 = jtz1;
    jtz1 = is_jump_to_zero;
    double t = ss.t().re;
    if (!(t <= O->endgame_start)) return ecode;
    // mixed precision: in the endgame a path whose coordinates grow (‖x‖∞ > 1e4: FP32 loses
    // range and accuracy on |x|^d) continues in FP64; so do paths flagged as diverging or
    // entering the singular endgame (see check_at_infinity, switch_to_singular)
    if (MIXED && !j64 && vnorm(ld(x), nullptr) > 1e4) switch_to_fp64(ss.t());
    if (steps_eg == 0) ext_steps_eg_start = ext_steps();
    steps_eg += 1;
    if (!step_success) return ecode;
    valuation_update(t);
    if (check_finite()) {
      switch_to_singular();
      return ecode;
    } else if (check_at_infinity()) {
      return ecode;
    }
    return ecode;
  }

  // ---------------------------------------------------------------- one path
  // One path in three parts, so that a kernel can also advance many paths one step at a time:
  // begin (start solution, tracker/endgame init), step (one endgame or tracker step; false once
  // the path stops), finish (result record and endpoint).
  __device__ HC_NI void begin(int64_t k) {
    cur_path = k;
    if (LANE < n) {
      double2 s = a->starts[k * n + LANE];
      x[LANE] = C64(s.x, s.y);
    }
    __syncwarp();
    if (a->mode == 1) {
      eg_init(a->t1_re);
    } else {
      c64 t1 = C64(a->t1_re, a->t1_im), t0 = C64(a->t0_re, a->t0_im);
      if (a->path_t1) t1 = C64(a->path_t1[k], 0.0);
      if (a->path_t0) t0 = C64(a->path_t0[k], 0.0);
      const double om_in = a->path_omega ? a->path_omega[k] : dNaN();
      const double mu_in = a->path_mu ? a->path_mu[k] : dNaN();
      if (toric) {
        const double* wr = a->tor_w + (size_t)a->tor_row[k] * a->L.tor_n;
        for (int j = LANE; j < a->L.tor_n; j += 32) tw[j] = wr[j];
        tc_t = dNaN();
        __syncwarp();
      }
      tracker_init(t1, t0, om_in, mu_in);
    }
  }
  __device__ __forceinline__ bool tracking() const {
    return a->mode == 1 ? ecode == EC_tracking : tcode == TC_tracking;
  }
  __device__ HC_NI bool step() {
    if (a->mode == 1) {
      eg_step();
      if (cancelled()) ecode = EC_terminated_unknown;
    } else {
      tracker_step();
      if (cancelled()) tcode = TC_terminated_unknown;
    }
    return tracking();
  }
  __device__ HC_NI void finish(int64_t k) {
    hc_path_result R;
    memset(&R, 0, sizeof(R));
    R.path_number = k + 1;
    c64 xs;
    if (a->mode == 1) {
      double t;
      const c64* xv;
      if (ecode == EC_success) {
        t = 0.0;
        xv = sol;
      } else {
        t = ss.t().re;
        xv = x;
      }
      H_eval(xv, C64(t), s1);
      R.residual = vnorm(ld(s1), nullptr);
      R.return_code = ecode;
      R.t_re = t;
      R.accuracy = eg_accuracy;
      R.cond = eg_cond;
      R.singular = eg_singular;
      R.winding_number = eg_wnum;
      R.omega = omega;
      R.mu = mu;
      R.tau = tau;
      R.extended_precision = extended_prec;
      R.extended_precision_used = used_extended_prec;
      R.accepted_steps = accepted_steps;
      R.rejected_steps = rejected_steps;
      R.steps_eg = steps_eg;
      R.last_t = last_t;
      xs = ld(xv);
      if (LANE < n) {
        if (a->val) a->val[k * n + LANE] = vx[LANE];
        if (a->last) a->last[k * n + LANE] = make_double2(lastp[LANE].re, lastp[LANE].im);
      }
    } else {
      c64 t = ss.t();
      R.return_code = tcode;
      R.t_re = t.re;
      R.t_im = t.im;
      R.accuracy = accuracy;
      R.omega = omega;
      R.mu = mu;
      R.tau = tau;
      R.extended_precision = extended_prec || refined_extended_prec;
      R.extended_precision_used = used_extended_prec || refined_extended_prec;
      R.accepted_steps = accepted_steps;
      R.rejected_steps = rejected_steps;
      H_eval(x, t, s1);
      R.residual = vnorm(ld(s1), nullptr);
      // valuation at the end point for the valuation known-answer tests
      val_init();
      if (tcode != TC_terminated_invalid_startvalue && tcode != TC_terminated_invalid_startvalue_singular_jacobian)
        valuation_update(t.re);
      xs = ld(x);
      if (LANE < n) {
        if (a->val) a->val[k * n + LANE] = vx[LANE];
        if (a->last) a->last[k * n + LANE] = make_double2(vtx[LANE], 0.0);
      }
    }
    if (LANE < n) a->sol[k * n + LANE] = make_double2(xs.re, xs.im);
    if (LANE == 0) a->res[k] = R;
    __syncwarp();
  }
  __device__ HC_NI void run(int64_t k) {
    HC_PHASE(PH_RUN);
    begin(k);
    while (tracking())
      if (!step()) break;
    finish(k);
  }
};

}  // namespace hcd
