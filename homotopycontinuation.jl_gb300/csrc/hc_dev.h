// hc_dev.h — data shared by the host launcher and the path-tracking kernel.
//
// A homotopy is compiled on the host into a "monomial program" (the GPU counterpart of
// ModelKit's InstructionSequence, src/model_kit/instruction_sequence.jl:1-27):
//   * a monomial table in degree order; monomial m = monomial[parent] * x[var], m = 0 is 1,
//   * "value rows": F_0..F_{n-1}, G_0..G_{n-1}; each a list of (coefficient, monomial),
//   * "Jacobian rows": ∂F_i/∂x_j (row j*n+i) then ∂G_i/∂x_j (row n*n + j*n+i); a Jacobian
//     term is (monomial, value term, exponent): its coefficient is exponent × the value term's,
//     so the tables stay small enough to live in shared memory,
// plus a static lane schedule: every row is cut into segments, segments are spread over the
// 32 lanes of a warp, and each segment writes one partial sum ("slot"); slots of one row are
// contiguous so the row total is a fixed-order sum.
//
// Shared memory of a CTA: [per-term tables, copied once per CTA][warp 0][warp 1]...
#pragma once
#include "hc_rtc.h"

#include "../../include/hcgpu.h"

namespace hcd {

struct DevRows {
  int nrows, nterms, nslots, nseg;
  const int4* seg;      // [nseg] (stride, term begin, term end, slot | mult << 24), grouped by lane
  const int* lane_seg;  // [33]
  const int* row_slot;  // [nrows + 1]
};

struct DevProg {
  int n, M, nlev, top;  // top: first monomial of the highest degree level
  const int2* mdef;     // [M] (parent, var)
  const int* lev;       // [nlev + 1] monomial ranges per degree level (level 0 = {0})
  DevRows val, jac;
  // per-term tables (global copies; the kernel stages them in shared memory)
  const double2* vcoef64;  // [val.nterms]
  const float2* vcoef32;   // [val.nterms]
  const uint16_t* vmono;   // [val.nterms]
  const uint32_t* jcode;   // [jac.nterms] monomial | value-term << 16
  // Jacobian segments carry their exponent multiplier in bits 24..31 of the slot field
  double gamma_re, gamma_im;
};

// Byte offsets of the CTA tables and of the per-warp regions
struct TableLayout {
  int bytes;
  int vcoef64, vcoef32, vmono, jcode, mdef;
  int n64, n32, nmono, njcode, nmdef;  // sizes in bytes (multiples of 16)
  int vc64_global;  // 1: the FP64 value coefficients are read from global memory (L1/L2), not staged
};
struct WarpLayout {
  int bytes;
  int state, mono, part, A, LU, xJ, dinv, ipiv;
  int vec;   // complex vectors (vn elements each, 16 B)
  int rvec;  // real vectors (vn elements each, 8 B)
  int vn;    // padded vector length (elements)
  int v32;   // FP32 staging: x (FP32 Jacobians) or tx0..tx2 (FP32 Taylor series), 4 × vn c32
  int tor;   // toric homotopy: coefficients u·t^w (c64), t^w and w (double) of the current path
  int tor_n; // value terms of the toric program (0: not a toric homotopy)
  // Mixed precision's rarely used FP64 working set — double-double monomials and partial
  // sums, FP64 Taylor series, FP64 Jacobian partial sums — may live in a per-warp slice of
  // global memory (Launch::cold) instead of shared memory: `cold` bytes per warp, the monomial
  // area at cmono and the partial sums at cpart. cold == 0: those areas alias mono and part.
  int cold, cmono, cpart;
  // cold layout: the last HC_NCVEC_COLD complex vectors (the endgame's solution estimate and
  // predictions and the singular endgame's samples), the last HC_NRVEC_COLD real vectors (the
  // endgame's scalings, condition estimates and valuation) and the point of the last Jacobian
  // (xJ) — each used once per endgame step or evaluation or less — at these offsets of the
  // global slice instead of shared memory; −1: in shared memory
  int cvec, crvec, cxj;
  // cold layout: A and LU in shared memory hold FP32 entries only (mixed precision's Jacobian);
  // FP64 Jacobians (path starts, condition numbers, the FP64 fallback) use A and LU at these
  // offsets of the global slice; −1: one shared A and LU of FP64 size serve both arithmetics
  int cA, cLU;
  // 1: mixed precision's FP32 Jacobian partial sums go to the FP64 monomial area (dead once the
  // value rows have been summed) instead of the partial-sum area
  int jmono;
};
// per-warp slot of the tracker state object (PathTracker: 1,264 bytes; 1,432 with the phase
// counters of profiling builds)
#ifdef HC_PHASE_CLOCKS
constexpr int HC_STATE_BYTES = 1536;
#else
constexpr int HC_STATE_BYTES = 1280;
#endif
constexpr int HC_NCVEC = 22, HC_NRVEC = 19, HC_NCVEC_COLD = 10, HC_NRVEC_COLD = 16;
constexpr int HC_LOG_FIELDS = 36;  // doubles per step-log record
constexpr int HC_NFEAT = 12;       // step features of the learned proposal
constexpr int HC_NSTATS = 11;      // device counters of a tracking call
// Cycle counters of the tracker's phases, accumulated per warp (lane 0, clock64) in builds
// compiled with -DHC_PHASE_CLOCKS and reported by hc_last_stats; zero otherwise. Phases nest
// (a solve includes the factorization it triggers), so the counts are inclusive.
enum HcPhase {
  PH_RUN, PH_STEP, PH_PREDICTOR, PH_PREDICT, PH_NEWTON, PH_EVALJ, PH_EVAL, PH_TAYLOR, PH_LU, PH_SOLVE,
  PH_NORM, PH_STEPSIZE, PH_ENDGAME, PH_MONO, PH_VALROWS, PH_JACROWS, PH_REFINE, PH_INIT, PH_COND, PH_DD,
  PH_WAIT,  // lockstep schedules: waits at the round barrier (PH_RUN then spans the warp's whole loop)
  HC_NPHASE
};

// Step-proposal network as the tracker reads it: normalisation, BF16 weights, FP32 biases
// (12→64→64→2; see hc_mlp.cu for the parameter layout and the loss).
struct StepModel {
  float mean[HC_NFEAT], stdinv[HC_NFEAT];
  float c;       // logit of the target acceptance probability
  float logmax;  // log of the largest step multiplier proposed
  float pad[6];
  uint16_t W1T[HC_NFEAT * 64];  // input-major: W1T[i*64 + u] = W1[u][i], so a warp reads 64 B
  float b1[64];
  uint16_t W2T[64 * 64];  // W2T[v*64 + u] = W2[u][v]
  float b2[64];
  uint16_t W3[2 * 64];
  float b3[2];
  float pad2[2];
};

struct Launch {
  DevProg P;
  hc_options O;
  TableLayout T;
  WarpLayout L;
  int64_t npaths;
  const double2* starts;
  hc_path_result* res;
  double2* sol;
  double* val;
  double2* last;
  int mode;  // 1 endgame, 0 plain tracker
  double t1_re, t1_im, t0_re, t0_im;
  unsigned long long* counter;  // work queue head
  volatile int* cancel;
  unsigned long long* stats;  // [9] device counters
  // optional step log: records of the paths in [log_lo, log_hi)
  double* log;
  unsigned long long* log_count;
  long long log_cap, log_lo, log_hi;
  const StepModel* model;  // learned step control (options.step_control == HC_STEP_LEARNED)
  unsigned long long* phase;  // [HC_NPHASE] phase cycle counters (profiling builds), may be null
  const int64_t* path_list;   // if set: queue item i tracks path path_list[i] (in-place re-tracking)
  // per-path overrides of the plain tracker (mode 0), each null or [npaths]: start and target
  // time (real), initial ω and μ (NaN: computed by init_newton)
  const double *path_t1, *path_t0, *path_omega, *path_mu;
  // toric homotopy of the polyhedral method: value-term weights, one row per mixed cell
  // (program term order, tor_n per row), and the row of each path
  const double* tor_w;
  const int32_t* tor_row;
  char* cold;  // per-warp global scratch of L.cold bytes (warp w of CTA b at (b·warps + w)·L.cold)
  // parameter homotopy of a straight-line program: p (start parameters) then q (target)
  const double2* slp_pq;
  int lockstep;  // 1: the CTA's warps advance their paths one step per round; 2: the same per
                 // sub-partition; 3: per two sub-partitions (hc_options::lockstep)
};

// A batch of independent homotopies tracked in one launch (hc_set_batch / hc_track_batch).
// Instance i has its own compiled program; its results start at path_off and its start and
// solution vectors at vec_off (complex elements). The CTAs of the persistent kernel take work
// units — (instance, path range) — from a device queue, stage that instance's tables in
// shared memory, and their warps pull the unit's paths from a shared-memory counter.
struct BatchInstance {
  DevProg P;
  TableLayout T;
  WarpLayout L;
  int64_t npaths, path_off, vec_off;
};
struct BatchUnit {
  int inst, lo, hi, pad;
};
struct BatchLaunch {
  Launch base;  // options, queue head (units), counters, cancel flag, t range, output bases
  const BatchInstance* inst;
  const BatchUnit* units;
  int nunits;
  int tbytes;   // shared bytes reserved for the tables (maximum over the instances)
  int wstride;  // shared bytes per warp (maximum over the instances)
};
constexpr int HC_LAUNCH_SMEM = (int)((sizeof(Launch) + 127) & ~(size_t)127);
// warps per CTA at most: the single-homotopy kernel (track_kernel) and the batch kernel
constexpr int HC_MAX_WARPS = 16;
constexpr int HC_MAX_BATCH_WARPS = 16;

}  // namespace hcd
