/* hcgpu.h — C ABI of libhcgpu.so, a GB300 (sm_103a) path tracker for polynomial homotopy
 * continuation with the semantics of HomotopyContinuation.jl's total-degree hot path.
 *
 * The reference tracks one path at a time inside Julia:
 *   solve(F; start_system = :total_degree)            src/solve.jl:447-526
 *     → total_degree_variables(F; gamma)               src/total_degree.jl:32-117
 *     → threaded_solve: track(tracker, S[k])           src/solve.jl:628-709 (:669)
 *       → EndgameTracker track!/step!                  src/endgame_tracker.jl:297-399, 902-914
 *         → Tracker init!/step!                        src/tracker.jl:639-926
 *     → PathResult / Result counts                     src/path_result.jl:76-98, src/result.jl:102-212
 * This library replaces the per-path loop (serial_solve / threaded_solve, src/solve.jl:603-709)
 * with one batched call: every path of the batch is tracked by one warp of a persistent CUDA
 * kernel. Plain pointers and sizes only; the caller owns every host array it passes.
 *
 * Errors: every function returns an int status (HC_OK == 0). Per-path failures are not
 * errors: they are return codes inside hc_path_result, with the values of
 * EndgameTrackerCode (src/endgame_tracker.jl:100-117) or TrackerCode (src/tracker.jl:166-176).
 */
#ifndef HCGPU_H
#define HCGPU_H

#ifndef __CUDACC_RTC__
#include <stdint.h>
#endif

#ifdef __cplusplus
extern "C" {
#endif

enum hc_status {
  HC_OK = 0,
  HC_ERR_INVALID_ARG = 1,
  HC_ERR_CUDA = 2,
  HC_ERR_NO_SYSTEM = 3,
  HC_ERR_CANCELLED = 4,
  HC_ERR_UNSUPPORTED = 5,
  HC_ERR_TOO_LARGE = 6,
  HC_ERR_TIMEOUT = 7,
  HC_ERR_COMPILE = 8
};

/* Arithmetic of the corrector, predictor and LU.
 *   HC_PREC_FP64 : complex FP64 everywhere (the reference's arithmetic).
 *   HC_PREC_MIXED: Jacobian, Taylor coefficients and LU in complex FP32; Newton residual,
 *                  solution update, condition numbers and every threshold decision in FP64;
 *                  double-double residuals on near-singular steps as in the reference. */
enum hc_precision { HC_PREC_FP64 = 0, HC_PREC_MIXED = 1 };

/* Step-size control. HC_STEP_PLAIN is update_stepsize! (src/tracker.jl:541-588).
 * HC_STEP_LEARNED lets the loaded network (hc_set_step_model) enlarge the plain proposal after
 * each accepted step; a proposal the Newton contraction test rejects falls back to the plain
 * one. HC_STEP_EXPLORE multiplies the plain proposal by a pseudo-random factor in [1, 6] and
 * is used with the step log to collect training data. */
enum hc_step_control { HC_STEP_PLAIN = 0, HC_STEP_LEARNED = 1, HC_STEP_EXPLORE = 2 };

/* Mirrors TrackerOptions + TrackerParameters (src/tracker.jl:45-140) and EndgameOptions
 * (src/endgame_tracker.jl:47-72); hc_default_options fills in the reference defaults. */
typedef struct hc_options {
  int32_t max_steps;
  int32_t extended_precision;
  double max_step_size, max_initial_step_size, min_step_size, min_rel_step_size, terminate_cond;
  double a, beta_a, beta_omega_p, beta_tau, strict_beta_tau;
  int32_t min_newton_iters;
  int32_t max_endgame_steps, max_endgame_extended_steps, max_winding_number;
  int32_t zero_is_at_infinity, at_infinity_check, only_nonsingular, refine_steps;
  double endgame_start, min_cond, min_cond_growth, min_coord_growth, singular_min_accuracy;
  double val_finite_tol, val_at_infinity_tol, sing_cond, sing_accuracy, scaling_threshold;
  /* GPU-side knobs (no counterpart in the reference) */
  int32_t precision;      /* enum hc_precision */
  int32_t step_control;   /* enum hc_step_control */
  int32_t warps_per_cta;  /* 0 = as many as fit in shared memory (at most 16), 1..16 */
  int32_t ctas_per_sm;    /* 0 = as many as fit */
  /* scheduling of a CTA's warps: 1 = lockstep (every warp advances its path by one step, then
   * the CTA waits for all, so the warps run the same code together and share the instruction
   * cache), 2 = lockstep of the warps that share an SM sub-partition (warps w, w + 4), 3 = of the
   * warps of two sub-partitions, 0 = each warp on its own, -1 = automatic (1 with 8 or more
   * warps per CTA, except 3 for mixed-precision homotopies of 2,000 value terms or more; 2 for
   * mixed precision with 6 or 7 warps; batches 1 with 8 or more). Results are identical in every mode. */
  int32_t lockstep;
  int32_t reserved;
} hc_options;

/* Per-path record. Mirrors PathResult (src/path_result.jl:76-98) for endgame tracking and
 * TrackerResult (src/tracker.jl:235-247) for plain tracking. */
typedef struct hc_path_result {
  int32_t return_code;     /* EndgameTrackerCode (endgame) / TrackerCode (plain) value */
  int32_t winding_number;  /* 0 == nothing */
  double t_re, t_im;       /* t where tracking stopped (0 on success with the endgame) */
  double accuracy, residual, cond, omega, mu, tau;
  int32_t singular, extended_precision, extended_precision_used, _pad;
  int64_t accepted_steps, rejected_steps, steps_eg, path_number;
  double last_t;           /* t of last_path_point */
} hc_path_result;

typedef struct hc_handle hc_handle;

/* Fill *opts with the reference defaults (DEFAULT_TRACKER_PARAMETERS, EndgameOptions()). */
int hc_default_options(hc_options* opts);

/* Create a tracker on the current CUDA device. Replaces EndgameTracker(H; options)
 * (src/endgame_tracker.jl:243-254). */
int hc_create(const hc_options* opts, hc_handle** out);
/* Same on CUDA device `device` (the caller's current device is left unchanged). Every entry
 * point taking a handle runs on the handle's device, so one host thread may drive handles on
 * several devices: the per-device shards of a batch (src/solve.jl:628-709 shards the paths over
 * threads; here contiguous path ranges go to devices). */
int hc_create_on_device(const hc_options* opts, int device, hc_handle** out);
void hc_destroy(hc_handle* h);
int hc_set_options(hc_handle* h, const hc_options* opts);

/* Set the straight-line homotopy H(x,t) = γ t G(x) + (1-t) F(x)
 * (src/homotopies/straight_line_homotopy.jl:10-68) from term tables:
 *   *_eq[k]        equation of term k (0-based),
 *   *_exps[k*n+j]  exponent of variable j in term k,
 *   *_coef[2k..]   coefficient (re, im).
 * For the total-degree start system G_i = s_i (x_i^{D_i} - 1) (src/total_degree.jl:62,102-106).
 * n ≤ 32. Replaces the ModelKit compile step (src/model_kit/compiled_system_homotopy.jl:15-58):
 * the tables become a monomial program evaluated by the kernel. */
int hc_set_homotopy(hc_handle* h, int n, int nG, const int32_t* G_eq, const int32_t* G_exps,
                    const double* G_coef, int nF, const int32_t* F_eq, const int32_t* F_exps,
                    const double* F_coef, double gamma_re, double gamma_im);

/* ---- Straight-line programs -----------------------------------------------------------
 * A target system F given as a straight-line program instead of term tables: ModelKit's
 * InstructionSequence (src/model_kit/instruction_sequence.jl:1-27) with 0-based tape slots.
 * Ops carry the values of ModelKit's OpType (src/model_kit/operations.jl:5-49) and its
 * semantics (:183-248); POW_INT's second input is the integer exponent itself, not a slot.
 * The GPU evaluator supports the algebraic ops (not ACOS .. TANH, POW). */
enum hc_op {
  HC_OP_STOP = 0, HC_OP_CB, HC_OP_ACOS, HC_OP_ASIN, HC_OP_COS, HC_OP_COSH, HC_OP_EXP, HC_OP_INV,
  HC_OP_INV_NOT_ZERO, HC_OP_INVSQR, HC_OP_NEG, HC_OP_SIN, HC_OP_SINH, HC_OP_SQR, HC_OP_SQRT, HC_OP_TAN,
  HC_OP_TANH, HC_OP_IDENTITY, HC_OP_ADD, HC_OP_DIV, HC_OP_MUL, HC_OP_SUB, HC_OP_POW_INT, HC_OP_POW,
  HC_OP_ADD3, HC_OP_MUL3, HC_OP_MULADD, HC_OP_MULSUB, HC_OP_SUBMUL, HC_OP_ADD4, HC_OP_MUL4,
  HC_OP_MULMULADD, HC_OP_MULMULSUB
};
/* Instruction (instruction_sequence.jl:1-5): output slot = op(input[0..arity-1]). */
typedef struct hc_instruction {
  int32_t input[4];
  int32_t op;
  int32_t output;
} hc_instruction;
/* The tape: slots [0, nconstants) hold the constants (complex, re/im interleaved), slots
 * [variables_offset, variables_offset + n) the variables x_1..x_n; instructions run in order,
 * each reading slots already written and writing any other slot below tape_size (a slot may
 * be written again, as in ModelKit's compacted tapes); HC_OP_STOP ends the program.
 * outputs[i] is the slot holding F_{i+1} at the end. With 1-based Julia indices this is the
 * reference's InstructionSequence of a system without parameters, every index minus one. */
typedef struct hc_slp {
  int32_t n;
  int32_t ninstructions;
  const hc_instruction* instructions;
  int32_t nconstants;
  const double* constants;
  int32_t variables_offset;
  int32_t tape_size;
  const int32_t* outputs;
} hc_slp;

/* Set the straight-line homotopy H = γ t G + (1 - t) F with F given as a straight-line
 * program and G the total-degree start system G_i = s_i (x_i^{D_i} - 1) (degrees D, scaling
 * s; src/total_degree.jl:62,102-106). Replaces ModelKit's compile step for this system
 * (src/model_kit/compiled_system_homotopy.jl:178-243: the program becomes source code that is
 * compiled, and compiled systems are cached by hash, :39-57): the program is emitted as CUDA C
 * — values, values with forward-mode derivatives (the Jacobian column of direction j in warp
 * lane j), double-double values and Taylor series of orders 1..3, every tape value a register
 * — and compiled with NVRTC together with the tracking kernel for this device's architecture;
 * the cubin is cached by a hash of its source (in memory, and on disk under $HCGPU_CACHE or
 * ~/.cache/hcgpu). hc_track / hc_track_device then run that kernel; n ≤ 32. Fails with
 * HC_ERR_UNSUPPORTED for ops the evaluator lacks and HC_ERR_COMPILE when NVRTC fails. */
int hc_set_slp(hc_handle* h, const hc_slp* F, const int32_t* degrees, const double* scaling, double gamma_re,
               double gamma_im);
/* The CUDA C source hc_set_slp generates for a program (no GPU needed): up to capacity - 1
 * bytes and a terminating 0 into out (may be NULL); *length receives the full length. */
int hc_slp_source(const hc_slp* F, const int32_t* degrees, const double* scaling, char* out, int64_t capacity,
                  int64_t* length);
/* Parameter homotopy H(x, t) = F(x; t p + (1 - t) q) (src/homotopies/parameter_homotopy.jl:3-44)
 * of a program F(x; p) whose tape holds its nparameters parameters at slots
 * [parameters_offset, +nparameters) (after the variables in ModelKit's tapes,
 * src/model_kit/instruction_sequence.jl:1-27); p (start parameters) and q (target parameters)
 * are nparameters complex values each. The parameters may enter F in any way the program's
 * ops allow. Replaces the handle's homotopy; hc_track from start solutions of F(x; p) at t = 1
 * to t = 0 then solves F(x; q). */
int hc_set_slp_parameter_homotopy(hc_handle* h, const hc_slp* F, int nparameters, int32_t parameters_offset,
                                  const double* start_parameters, const double* target_parameters);
/* New (p, q) for the program of hc_set_slp_parameter_homotopy (parameters!, :56-62): no new
 * compilation. */
int hc_set_slp_parameters(hc_handle* h, const double* start_parameters, const double* target_parameters);
/* The CUDA C that hc_set_slp_parameter_homotopy compiles for F. */
int hc_slp_parameter_source(const hc_slp* F, int nparameters, int32_t parameters_offset, char* out,
                            int64_t capacity, int64_t* length);

/* Track npaths start solutions (host arrays, npaths×n complex interleaved).
 *   endgame = 1: EndgameTracker from t = t1_re to 0 (track(eg, x), src/endgame_tracker.jl:902-914),
 *   endgame = 0: Tracker from t1 to t0 (track(tracker, x, t1, t0), src/tracker.jl:1023-1026).
 * out_results[npaths], out_solutions[npaths×n complex]; out_valuation (npaths×n, may be NULL)
 * receives val_x (src/valuation.jl:6-22); out_last (npaths×n complex, may be NULL) receives
 * last_path_point with the endgame and val_tẋ (real parts) without it.
 * Copies in, runs and copies out on the handle's stream; returns when the results are on the host.
 * With learned step control (and the endgame), paths whose nonsingular endpoints coincide with
 * another path's — the mark of a path that jumped onto another path — are re-tracked in place
 * with the plain step rule before returning (hc_last_stats [40] counts them); the device entry
 * points return the tracker's results unchecked. */
int hc_track(hc_handle* h, int64_t npaths, const double* starts, int endgame, double t1_re,
             double t1_im, double t0_re, double t0_im, hc_path_result* out_results,
             double* out_solutions, double* out_valuation, double* out_last);

/* Same, on device pointers, asynchronous on `stream` (a cudaStream_t, or NULL for the
 * handle's stream). No host synchronisation; the caller synchronises the stream. */
int hc_track_device(hc_handle* h, int64_t npaths, const double* d_starts, int endgame,
                    double t1_re, double t1_im, double t0_re, double t0_im,
                    hc_path_result* d_results, double* d_solutions, double* d_valuation,
                    double* d_last, void* stream);

/* Toric homotopy of the polyhedral method (ToricHomotopy, src/homotopies/toric_homotopy.jl:9-278;
 * its tracking in PolyhedralTracker, src/polyhedral.jl:412-530):
 *   H(x, t) = F(x; c(t)),  c_k(t) = u_k t^{w_k}
 * with the base coefficients u of the term table (F_eq, F_exps, F_coef as in hc_set_homotopy;
 * no start system) and per-path weights w: `weights` holds `nrows` rows of nF finite,
 * non-negative weights in the table's term order (one row per mixed cell; 0 on the cell's
 * own terms). The handle then tracks this homotopy only (hc_set_homotopy switches back). */
int hc_set_toric(hc_handle* h, int n, int nF, const int32_t* F_eq, const int32_t* F_exps, const double* F_coef,
                 int nrows, const double* weights);

/* Track npaths start vectors of the toric homotopy with the plain Tracker in FP64 (track!,
 * src/tracker.jl:937-965): path p uses weight row rows[p] and runs from t1[p] to t0[p]
 * (real, ≥ 0); omega/mu (may be NULL; NaN entries allowed) are init!'s ω and μ keywords — both
 * given skip init_newton. max_initial_step_size and min_step_size come from the options
 * (stage 1 of the reference sets 0.2; its restart sets min_step_size 0).
 * out_results[npaths] holds TrackerResult fields (return_code: TrackerCode), out_solutions
 * the endpoints. Host buffers; returns when the results are on the host. */
int hc_track_toric(hc_handle* h, int64_t npaths, const double* starts, const int32_t* rows, const double* t1,
                   const double* t0, const double* omega, const double* mu, hc_path_result* out_results,
                   double* out_solutions);

/* Fine mixed cells of n supports under an integer lifting (host code, no GPU): the start
 * cells of the polyhedral homotopy, which the reference takes from MixedSubdivisions.jl
 * (fine_mixed_cells, called at src/polyhedral.jl:23). Support i has nterms[i] points; points
 * holds all supports' points (Σ nterms × n, row-major), lifting one integer per point. For
 * every cell (at most max_cells; *out_ncells receives the count, HC_ERR_TOO_LARGE when it
 * exceeds max_cells) out_indices holds the two point indices per support (max_cells × 2n),
 * out_normals the inner normal γ, out_beta β_i = min over support i of ⟨a, γ⟩ + ω(a)
 * (max_cells × n each) and out_volumes |det(a_i − b_i)|. A lifting that does not induce a fine
 * subdivision returns HC_ERR_INVALID_ARG ("not generic"); draw another. */
int hc_mixed_cells(int n, const int32_t* nterms, const int32_t* points, const int64_t* lifting, int64_t max_cells,
                   int32_t* out_indices, double* out_normals, double* out_beta, int64_t* out_volumes,
                   int64_t* out_ncells);

/* Request cancellation of a running hc_track, hc_track_batch or hc_track_toric on this handle
 * (thread-safe; the call's own start clears the request). The kernel stops at the next step:
 * paths not yet finished report terminated_unknown, finished paths keep their results, and the
 * call returns HC_ERR_CANCELLED with every output array filled. This is solve's
 * catch_interrupt = true (src/solve.jl:603-709: an interrupt stops the loop and the paths
 * tracked so far are returned). */
int hc_cancel(hc_handle* h);

/* Run time limit, in seconds, of each later hc_track / hc_track_batch / hc_track_toric call on
 * this handle (0 = none, the default). When a call runs past it, it stops as after hc_cancel and
 * returns HC_ERR_TIMEOUT. No counterpart in the reference's solve (its closest analogue is the
 * interrupt handling above). */
int hc_set_time_limit(hc_handle* h, double seconds);

/* Last error message of this handle (or of the library when h is NULL). */
const char* hc_last_error(hc_handle* h);

/* Device counters of the last tracking call on this handle, up to nout values: [0] paths,
 * [1] evaluations with Jacobian, [2] residual-only evaluations, [3] double-double residuals,
 * [4] Taylor orders, [5] LU factorizations, [6] triangular-solve pairs, [7] FP32 Taylor
 * evaluations redone in FP64, [8] paths moved to FP64; [9] monomials, [10] value terms,
 * [11] Jacobian terms of the last hc_set_homotopy program; [12] CTAs, [13] warps per CTA,
 * [14] shared bytes per warp, [15] shared bytes of the CTA tables, [16] top-degree monomial
 * offset; [17] learned step proposals, [18] of them rejected by Newton; [19..39] cycles per
 * tracker phase (run, step, predictor, predict, newton, eval+Jacobian, eval, taylor, LU,
 * solve, norm, step size, endgame, monomials, value rows, Jacobian rows, refinement, init,
 * cond, double-double, lockstep barrier waits; inclusive), nonzero only in libraries built with
 * -DHC_PHASE_CLOCKS; [40] paths re-tracked with plain step control by the jump check of
 * hc_track/hc_track_batch; [41] lockstep mode of the last launch (hc_options::lockstep).
 * No counterpart in the reference (its closest analogue is the Jacobian's factorization and
 * ldiv counters, src/linear_algebra.jl:809-862). */
int hc_last_stats(hc_handle* h, double* out, int nout);

/* Load the step-proposal network used with HC_STEP_LEARNED: `params` are the FP32 parameters
 * (hc_mlp_num_params() floats, layout in hc_mlp.cu; stored as BF16 weights), `mean`/`std`
 * normalise the 12 features, proposals target acceptance probability `confidence` and are
 * capped at `max_factor` times the plain proposal. No counterpart in the reference. */
int hc_set_step_model(hc_handle* h, const float* params, const float* mean, const float* std,
                      double confidence, double max_factor);

/* Step-proposal network kernels (BF16 tensor-core operands, FP32 accumulation), device
 * pointers: forward out[B×2] = net(X[B×12]); mean BCE loss and gradient of logged steps
 * (X, tried log-multipliers L, accepted flags Y); one Adam step. No reference counterpart. */
int hc_mlp_num_params(void);
int hc_mlp_forward(const float* d_X, int B, const float* d_params, float* d_out, void* stream);
int hc_mlp_grad(const float* d_X, const float* d_L, const float* d_Y, int B, const float* d_params,
                float* d_grad, float* d_loss, void* stream);
int hc_mlp_adam(float* d_params, float* d_m, float* d_v, const float* d_grad, int step, float lr,
                float weight_decay, void* stream);

/* Step log: after this call, every step attempted on a path whose 0-based index lies in
 * [path_lo, path_hi) appends one record of HC_STEP_LOG_FIELDS doubles to a device buffer of
 * `capacity` records (capacity 0 disables logging). The fields follow the reference's
 * PathInfo trace (src/path_info.jl:3-21): path number, t (re, im), Δs tried, trust region,
 * local error, ω, μ (before the step), accepted, Newton iterations, θ, ‖Δx₀‖, ‖x‖∞,
 * previous Δs, next Δs, flags (extended precision | FP64-fallback << 1 | Newton code << 2),
 * ω and accuracy returned by the corrector, trust region after the step, accepted steps;
 * then the 12 step features that decided this step's size, the log-multiplier applied, the
 * plain proposal, a features-valid flag and the step-control mode (fields 20..35).
 * It is the training data of the learned step proposal. */
#define HC_STEP_LOG_FIELDS 36
int hc_set_step_log(hc_handle* h, int64_t capacity, int64_t path_lo, int64_t path_hi);
/* Copy up to max_records records of the last call to `out`; *n_records receives the number
 * of records the call produced (which may exceed the capacity). */
int hc_get_step_log(hc_handle* h, double* out, int64_t max_records, int64_t* n_records);

/* Track a batch without allocating any device memory. No counterpart in the reference.
 * For callers that cannot call cudaMalloc (code running under an allocator that owns all
 * device memory, a memory-capped sandbox, or a hot path that must not allocate): options,
 * homotopy term tables (host arrays, as for hc_set_homotopy) and device buffers for the start
 * solutions, results and endpoints go in; the kernel's scratch (work-queue head, counters,
 * cancel flag, compiled tables) lives in a 1 MiB static device array of the library instead
 * of handle-owned allocations. Compiled tables above 1 MiB - 256 bytes are rejected with
 * HC_ERR_TOO_LARGE. All calls on a device share that array: calls whose kernels overlap on
 * the GPU race and must be serialised (e.g. one stream). The first call on a device looks up
 * the array's address; make it outside any stream capture. The compiled tables are copied
 * from a host buffer that lives only for the call, so a call on a stream that is being
 * captured is refused with HC_ERR_UNSUPPORTED. step_control must be HC_STEP_PLAIN or
 * HC_STEP_EXPLORE (learned steps need a handle's network). Asynchronous on `stream`
 * (a cudaStream_t, NULL = legacy default stream). */
int hc_track_noalloc(const hc_options* opts, int n, int nG, const int32_t* G_eq,
                     const int32_t* G_exps, const double* G_coef, int nF, const int32_t* F_eq,
                     const int32_t* F_exps, const double* F_coef, double gamma_re,
                     double gamma_im, int64_t npaths, const double* d_starts, int endgame,
                     double t1_re, double t1_im, double t0_re, double t0_im,
                     hc_path_result* d_results, double* d_solutions, void* stream);

/* ---- Batches of independent homotopies (one launch) ----------------------------------
 * Replaces one solve(F_i) per instance (src/solve.jl:447-526, each running threaded_solve,
 * src/solve.jl:628-709) by a single persistent launch over all instances' paths. An instance
 * is a straight-line homotopy given exactly as to hc_set_homotopy, plus its number of start
 * solutions. Results are stored instance after instance (instance i's first result at
 * Σ_{j<i} npaths_j, its first start/solution element at Σ_{j<i} npaths_j·n_j complex values);
 * path_number counts within the instance (1-based), as in the per-instance solve. */
typedef struct hc_instance_desc {
  int32_t n, nG, nF, reserved;
  const int32_t* G_eq;
  const int32_t* G_exps;
  const double* G_coef;
  const int32_t* F_eq;
  const int32_t* F_exps;
  const double* F_coef;
  double gamma_re, gamma_im;
  int64_t npaths;
} hc_instance_desc;

/* Compile and upload a batch (replacing any previous batch of the handle). The kernel's CTAs
 * take work units of at most unit_paths[n] paths of one instance with n variables
 * (unit_paths: 33 entries indexed by n, NULL or 0 = one path per warp of a CTA); units are
 * queued largest estimated cost first. `total_paths` and `total_elements` (optional) receive
 * Σ npaths_i and Σ npaths_i·n_i. */
int hc_set_batch(hc_handle* h, int ninstances, const hc_instance_desc* instances,
                 const int32_t* unit_paths, int64_t* total_paths, int64_t* total_elements);
/* Re-plan the current batch's launch without recompiling it, per system size n (33 entries
 * each, indexed by n; NULL = all 0):
 *   unit_paths[n]  paths per work unit, 0 = one per warp of a CTA;
 *   staging[n]     mixed precision only (FP64 batches have one staging): 0 or 2 = the FP64 value
 *                  coefficients are read through L1/L2 and the FP64 areas of the rare
 *                  double-double and FP64 steps sit in per-warp global slices (about half the
 *                  shared memory per warp); 1 = every table and per-warp area in shared memory.
 * Results are identical for every plan; only the time differs. The staging also applies to
 * later hc_set_batch calls on the handle. */
int hc_set_batch_launch(hc_handle* h, const int32_t* unit_paths, const int32_t* staging);
/* The launch-plan autotuner: for every n in the batch, tracks `sample` instances of that n (0 =
 * all) from `starts` (all instances' start solutions, as hc_track_batch takes them) with each
 * unit size in candidates[0..ncandidates-1] (1..16 entries) and, in mixed precision, each
 * staging, times `repeats` launches after one warm-up with CUDA events on the handle's stream,
 * and keeps the fastest. Every launch has the shape the full batch will have (tables and
 * per-warp strides of all instances). Applies the chosen plan (hc_set_batch_launch) and writes
 * it to unit_paths_out[33] / staging_out[33] (optional); ms_out (optional, 33·2·ncandidates)
 * receives the milliseconds per launch, [(n·2 + s)·ncandidates + c] with s = 0 for global slices
 * and 1 for shared staging (FP64: s = 0), NaN where nothing ran. */
int hc_autotune_batch(hc_handle* h, const double* starts, int sample, const int32_t* candidates, int ncandidates,
                      int repeats, int32_t* unit_paths_out, int32_t* staging_out, double* ms_out);
/* Track every path of the batch from t=1 to t=0 (endgame != 0: EndgameTracker) on device
 * buffers; asynchronous on `stream` (NULL = the handle's stream). The launch is recorded in a
 * CUDA graph the first time a set of buffers is used and replayed afterwards. */
int hc_track_batch_device(hc_handle* h, const double* d_starts, int endgame,
                          hc_path_result* d_results, double* d_solutions, void* stream);
/* Same with host arrays; blocks until the results are in `out_results`/`out_solutions`. With
 * learned step control, applies hc_track's jump check within every instance. */
int hc_track_batch(hc_handle* h, const double* starts, int endgame, hc_path_result* out_results,
                   double* out_solutions);

/* ---- Certification -------------------------------------------------------------------
 * certify(F, solutions) (src/certification.jl:691-745): Krawczyk certificates for approximate
 * solutions of F, the target system of the handle's homotopy (H at t = 0). Per candidate:
 * certified = 1 if the polydisc B(center, radius) provably holds exactly one solution, which lies
 * in the polydisc B(enclosure center, enclosure); realness = 1 if that solution is provably real
 * (requires real_coefficients != 0, i.e. F has real coefficients), 2 if provably non-real, 0 if
 * undecided. center is the candidate after Newton refinement. Ball arithmetic with upward rounded
 * radii, one warp per candidate: first with FP64 centres (precision = 53), then, for the
 * candidates that pass fails, with double-word centres (precision = 106; the reference's Arb step,
 * src/certification.jl:1120-1200). */
typedef struct hc_certificate {
  int32_t certified, realness;
  double radius, enclosure;
  int32_t precision; /* bits of the centres of the pass that decided: 53 or 106 */
  int32_t reserved;
} hc_certificate;
int hc_certify(hc_handle* h, int64_t ncandidates, const double* candidates, int real_coefficients,
               hc_certificate* out, double* out_centers, double* out_enclosure_centers);

/* FP64 and FP32 CUDA-core FMA throughput of the current GPU in TFLOP/s, measured by a
 * short microbenchmark: the roofline denominators of this FP-pipe-bound path. No
 * counterpart in the reference. */
int hc_fma_peak(double* fp64_tflops, double* fp32_tflops);

#ifdef __cplusplus
}
#endif
#endif /* HCGPU_H */
