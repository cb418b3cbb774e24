"""Host-side mirror of HomotopyContinuation.jl's path-tracking API over libhcgpu.so.

    tracker, starts = total_degree(F; gamma=...)       # src/total_degree.jl:19-117
    r = track(tracker, starts[k]; path_number=k)       # src/endgame_tracker.jl:902-914
    res = solve(F; start_system="total_degree", ...)   # src/solve.jl:447-526
    nnonsingular(res), nsingular(res), nat_infinity(res), nfailed(res)   # src/result.jl:789-824

Every call goes through the C ABI; there is no CPU path.
"""
from __future__ import annotations

import ctypes as ct
from dataclasses import dataclass, field, fields
from typing import Optional

import numpy as np

from . import _lib
from .systems import System, TotalDegreeHomotopy, random_gamma, total_degree_homotopy, total_degree_start_solutions

# EndgameTrackerCode (src/endgame_tracker.jl:100-117) and TrackerCode (src/tracker.jl:166-176)
ENDGAME_CODES = [
    "tracking", "success", "at_infinity", "at_zero", "terminated_accuracy_limit",
    "terminated_invalid_startvalue", "terminated_invalid_startvalue_singular_jacobian",
    "terminated_ill_conditioned", "terminated_max_steps", "terminated_max_extended_steps",
    "terminated_max_winding_number", "terminated_step_size_too_small", "terminated_unknown",
    "post_check_failed", "excess_solution", "polyhedral_failed",
]
TRACKER_CODES = [
    "tracking", "success", "terminated_max_steps", "terminated_accuracy_limit",
    "terminated_ill_conditioned", "terminated_invalid_startvalue",
    "terminated_invalid_startvalue_singular_jacobian", "terminated_step_size_too_small",
    "terminated_unknown",
]

_PARAMETER_PRESETS = {  # src/tracker.jl:58-62
    "default": dict(beta_omega_p=3.0, beta_tau=0.4),
    "fast": dict(beta_omega_p=2.0, beta_tau=0.75),
    "conservative": dict(beta_omega_p=4.0, beta_tau=0.25),
}


@dataclass
class TrackerOptions:
    """TrackerOptions + TrackerParameters (src/tracker.jl:45-140)."""

    max_steps: int = 10_000
    max_step_size: float = np.inf
    max_initial_step_size: float = np.inf
    extended_precision: bool = True
    min_step_size: float = 1e-48
    min_rel_step_size: float = 0.0
    terminate_cond: float = 1e13
    parameters: str = "default"
    # GPU knobs (no reference counterpart)
    precision: str = "fp64"  # "fp64" | "mixed"
    step_control: str = "plain"  # "plain" | "learned" | "explore"
    step_model: Optional[object] = None  # learn.StepModel for "learned"; None: the shipped model
    warps_per_cta: int = 0  # 0: as many as fit in shared memory (at most 16)
    ctas_per_sm: int = 0
    lockstep: int = -1  # lockstep of a CTA's warps: 1 all, 2 per sub-partition, 3 per two, 0 none, -1 auto


@dataclass
class EndgameOptions:
    """EndgameOptions (src/endgame_tracker.jl:47-72)."""

    endgame_start: float = 0.1
    max_endgame_steps: int = 2000
    max_endgame_extended_steps: int = 400
    min_cond: float = 1e6
    min_cond_growth: float = 1e4
    min_coord_growth: float = 100.0
    zero_is_at_infinity: bool = False
    at_infinity_check: bool = True
    only_nonsingular: bool = False
    singular_min_accuracy: float = 1e-6
    max_winding_number: int = 6
    val_finite_tol: float = 0.05
    val_at_infinity_tol: float = 0.01
    sing_cond: float = 1e14
    sing_accuracy: float = 1e-12
    scaling_threshold: float = -30.0
    refine_steps: int = 3


def make_options(tracker_options: Optional[TrackerOptions] = None,
                 endgame_options: Optional[EndgameOptions] = None) -> _lib.Options:
    to = tracker_options or TrackerOptions()
    eo = endgame_options or EndgameOptions()
    if to.parameters not in _PARAMETER_PRESETS:
        raise ValueError(f"Unsupported `parameters` value {to.parameters}")
    o = _lib.default_options()
    for f in ("max_steps", "max_step_size", "max_initial_step_size", "min_step_size", "min_rel_step_size",
              "terminate_cond", "warps_per_cta", "ctas_per_sm", "lockstep"):
        setattr(o, f, getattr(to, f))
    o.extended_precision = int(to.extended_precision)
    for k, v in _PARAMETER_PRESETS[to.parameters].items():
        setattr(o, k, v)
    o.strict_beta_tau = min(0.75 * o.beta_tau, 0.4)
    o.precision = {"fp64": _lib.PREC_FP64, "mixed": _lib.PREC_MIXED}[to.precision]
    o.step_control = {"plain": _lib.STEP_PLAIN, "learned": _lib.STEP_LEARNED,
                      "explore": _lib.STEP_EXPLORE}[to.step_control]
    for f in fields(EndgameOptions):
        v = getattr(eo, f.name)
        setattr(o, f.name, int(v) if isinstance(v, bool) else v)
    return o


@dataclass
class PathResult:
    """src/path_result.jl:76-98"""

    return_code: str
    solution: np.ndarray
    t: float
    accuracy: float
    residual: float
    singular: bool
    condition_jacobian: float
    winding_number: Optional[int]
    extended_precision: bool
    path_number: Optional[int]
    start_solution: Optional[np.ndarray]
    last_path_point: tuple
    valuation: Optional[np.ndarray]
    omega: float
    mu: float
    accepted_steps: int
    rejected_steps: int
    steps_eg: int
    extended_precision_used: bool
    multiplicity: int = 1

    # predicates (src/path_result.jl:215-298)
    def is_success(self):
        return self.return_code == "success"

    def is_at_infinity(self):
        return self.return_code in ("at_infinity", "at_zero")

    def is_excess_solution(self):
        return self.return_code == "excess_solution"

    def is_failed(self):
        return not (self.is_at_infinity() or self.is_success() or self.is_excess_solution())

    def is_singular(self):
        return bool(self.singular)

    def is_nonsingular(self):
        return not self.is_singular() and self.is_success()

    def is_real(self, atol=1e-6, rtol=0.0):
        m = np.max(np.abs(self.solution.imag))
        if m < atol:
            return True
        if rtol == 0:
            return False
        return m < rtol * np.sum(np.abs(self.solution))

    def steps(self):
        return self.accepted_steps + self.rejected_steps


@dataclass
class TrackerResult:
    """src/tracker.jl:235-247"""

    return_code: str
    solution: np.ndarray
    t: complex
    accuracy: float
    accepted_steps: int
    rejected_steps: int
    extended_precision: bool
    extended_precision_used: bool
    omega: float
    mu: float
    tau: float

    def is_success(self):
        return self.return_code == "success"

    def is_invalid_startvalue(self):
        return self.return_code in ("terminated_invalid_startvalue", "terminated_invalid_startvalue_singular_jacobian")


class _Handle:
    def __init__(self, options: _lib.Options, device: Optional[int] = None):
        self.L = _lib.load()
        self.h = ct.c_void_p()
        if device is None:
            _lib.check(self.L.hc_create(ct.byref(options), ct.byref(self.h)))
        else:
            _lib.check(self.L.hc_create_on_device(ct.byref(options), int(device), ct.byref(self.h)))
        self.n = 0

    def set_homotopy(self, H):
        from .slp import SLPHomotopy, SLPParameterHomotopy, c_program

        if isinstance(H, SLPParameterHomotopy):  # F(x; t p + (1 - t) q), F a program
            p = np.ascontiguousarray(H.start_parameters)
            q = np.ascontiguousarray(H.target_parameters)
            if getattr(self, "_param_program", None) is H.program:  # same program: new (p, q) only
                _lib.check(self.L.hc_set_slp_parameters(self.h, _lib.ptr(p), _lib.ptr(q)), self.h)
                return
            s, deg, sc, keep = c_program(H.program)
            self._keep = (s, deg, sc, keep)
            _lib.check(self.L.hc_set_slp_parameter_homotopy(self.h, ct.byref(s), H.program.nparams, H.program.poff,
                                                            _lib.ptr(p), _lib.ptr(q)), self.h)
            self._param_program = H.program
            self.n = H.n
            return
        self._param_program = None
        if isinstance(H, SLPHomotopy):  # F as a straight-line program (hc_set_slp)
            s, deg, sc, keep = c_program(H.program)
            self._keep = (s, deg, sc, keep)
            _lib.check(self.L.hc_set_slp(self.h, ct.byref(s), _lib.ptr(deg), _lib.ptr(sc), H.gamma.real,
                                         H.gamma.imag), self.h)
            self.n = H.n
            return
        Ge, Gx, Gc = H.G.term_arrays()
        Fe, Fx, Fc = H.F.term_arrays()
        self._keep = (Ge, Gx, Gc, Fe, Fx, Fc)
        P = _lib.ptr
        rc = self.L.hc_set_homotopy(self.h, H.n, len(Ge), P(Ge), P(Gx), P(Gc), len(Fe), P(Fe), P(Fx), P(Fc),
                                    H.gamma.real, H.gamma.imag)
        _lib.check(rc, self.h)
        self.n = H.n

    def set_options(self, options):
        _lib.check(self.L.hc_set_options(self.h, ct.byref(options)), self.h)

    def track(self, starts, endgame=True, t1=1.0, t0=0.0):
        starts = np.ascontiguousarray(np.asarray(starts, dtype=np.complex128).reshape(-1, self.n))
        npaths = starts.shape[0]
        res = np.zeros(npaths, dtype=_lib.RESULT_DTYPE)
        sol = np.zeros((npaths, self.n), dtype=np.complex128)
        val = np.zeros((npaths, self.n), dtype=np.float64)
        last = np.zeros((npaths, self.n), dtype=np.complex128)
        t1 = complex(t1)
        t0 = complex(t0)
        P = _lib.ptr
        rc = self.L.hc_track(self.h, npaths, P(starts), 1 if endgame else 0, t1.real, t1.imag, t0.real, t0.imag,
                             P(res), P(sol), P(val), P(last))
        _lib.check(rc, self.h)
        return res, sol, val, last

    def set_step_log(self, capacity, path_lo=0, path_hi=2**62):
        _lib.check(self.L.hc_set_step_log(self.h, int(capacity), int(path_lo), int(path_hi)), self.h)

    def get_step_log(self, max_records=None):
        cnt = np.zeros(1, dtype=np.int64)
        if max_records is None:
            _lib.check(self.L.hc_get_step_log(self.h, None, 0, _lib.ptr(cnt)), self.h)
            max_records = int(cnt[0])
        out = np.zeros((max(int(max_records), 1), _lib.STEP_LOG_FIELDS), dtype=np.float64)
        _lib.check(self.L.hc_get_step_log(self.h, _lib.ptr(out), int(max_records), _lib.ptr(cnt)), self.h)
        return out[: min(int(cnt[0]), int(max_records))]

    STAT_NAMES = ["paths", "evals_jac", "evals", "evals_dd", "taylor_orders", "lu", "solves", "taylor_fp64_redo",
                  "paths_to_fp64", "monomials", "value_terms", "jacobian_terms", "blocks", "warps_per_block",
                  "smem_per_warp", "smem_tables", "top", "learned_proposals", "learned_rejected"] + [
        "clk_" + p for p in ("run", "step", "predictor", "predict", "newton", "eval_jac", "eval", "taylor", "lu",
                             "solve", "norm", "stepsize", "endgame", "mono", "val_rows", "jac_rows", "refine",
                             "init", "cond", "dd", "wait")] + ["paths_retracked", "lockstep"]

    def stats(self):
        out = np.zeros(len(self.STAT_NAMES))
        _lib.check(self.L.hc_last_stats(self.h, _lib.ptr(out), len(out)), self.h)
        return dict(zip(self.STAT_NAMES, out.tolist()))

    def set_step_model(self, model):
        """Load a learn.StepModel (network parameters and feature normalisation)."""
        P = _lib.ptr
        params = np.ascontiguousarray(model.params, dtype=np.float32)
        mean = np.ascontiguousarray(model.mean, dtype=np.float32)
        std = np.ascontiguousarray(model.std, dtype=np.float32)
        _lib.check(self.L.hc_set_step_model(self.h, P(params), P(mean), P(std), float(model.confidence),
                                            float(model.max_factor)), self.h)

    def setup_step_control(self, to):
        if to.step_control == "learned":
            from . import learn
            self.set_step_model(to.step_model if to.step_model is not None else learn.default_model())

    def cancel(self):
        self.L.hc_cancel(self.h)

    def set_time_limit(self, seconds):
        _lib.check(self.L.hc_set_time_limit(self.h, float(seconds)), self.h)

    def __del__(self):
        try:
            if self.h:
                self.L.hc_destroy(self.h)
                self.h = ct.c_void_p()
        except Exception:
            pass


def _path_results(res, sol, val, last, starts, endgame_start):
    out = []
    for k in range(len(res)):
        r = res[k]
        t = float(r["t_re"])
        wn = int(r["winding_number"])
        out.append(PathResult(
            return_code=ENDGAME_CODES[int(r["return_code"])],
            solution=sol[k].copy(),
            t=t,
            accuracy=float(r["accuracy"]),
            residual=float(r["residual"]),
            singular=bool(r["singular"]),
            condition_jacobian=float(r["cond"]),
            winding_number=None if wn == 0 else wn,
            extended_precision=bool(r["extended_precision"]),
            path_number=int(r["path_number"]),
            start_solution=None if starts is None else starts[k].copy(),
            last_path_point=(last[k].copy(), float(r["last_t"])),
            valuation=None if t > endgame_start else val[k].copy(),
            omega=float(r["omega"]),
            mu=float(r["mu"]),
            accepted_steps=int(r["accepted_steps"]),
            rejected_steps=int(r["rejected_steps"]),
            steps_eg=int(r["steps_eg"]),
            extended_precision_used=bool(r["extended_precision_used"]),
        ))
    return out


class EndgameTracker:
    """src/endgame_tracker.jl:236-254: tracks from t=1 to t=0 with the valuation and
    singular endgames. ``track_batch`` tracks many start solutions in one GPU call."""

    def __init__(self, H: TotalDegreeHomotopy, tracker_options=None, endgame_options=None, devices=None):
        """``devices``: CUDA device indices; with more than one, every call splits its paths into
        contiguous ranges, one per device (handles on each), tracked concurrently."""
        self.homotopy = H
        self.tracker_options = tracker_options or TrackerOptions()
        self.options = endgame_options or EndgameOptions()
        o = make_options(self.tracker_options, self.options)
        self._hs = [_Handle(o, d) for d in devices] if devices else [_Handle(o)]
        self._h = self._hs[0]
        for h in self._hs:
            h.setup_step_control(self.tracker_options)
            h.set_homotopy(H)

    def set_homotopy(self, H):
        """Track another homotopy with the same options (e.g. new parameters)."""
        self.homotopy = H
        for h in self._hs:
            h.set_homotopy(H)

    def track_arrays(self, starts, t1: float = 1.0):
        if len(self._hs) > 1:
            from .parallel import track_on_handles

            return track_on_handles(self._hs, starts, endgame=True, t1=t1)
        return self._h.track(starts, endgame=True, t1=t1)

    def track_batch(self, starts, t1: float = 1.0, path_numbers=None):
        starts = np.asarray(starts, dtype=np.complex128).reshape(-1, self.homotopy.n)
        res, sol, val, last = self.track_arrays(starts, t1=t1)
        if path_numbers is not None:
            res["path_number"] = np.asarray(path_numbers)
        return _path_results(res, sol, val, last, starts, self.options.endgame_start)

    def track(self, x, t1: float = 1.0, path_number=None) -> PathResult:
        r = self.track_batch(np.asarray(x)[None, :], t1)[0]
        r.path_number = path_number
        return r

    def stats(self):
        if len(self._hs) > 1:
            from .parallel import merge_stats

            return merge_stats([h.stats() for h in self._hs])
        return self._h.stats()

    def cancel(self):
        """Stop a track_* call running in another thread (catch_interrupt, src/solve.jl:603-709)."""
        for h in self._hs:
            h.cancel()

    def set_time_limit(self, seconds):
        """Run time limit of each later track_* call (0 = none); past it the call raises
        HCError(HC_ERR_TIMEOUT)."""
        for h in self._hs:
            h.set_time_limit(seconds)


class Tracker:
    """src/tracker.jl:452-479: tracks x from t₁ to t₀ without the endgame."""

    def __init__(self, H: TotalDegreeHomotopy, options: Optional[TrackerOptions] = None):
        self.homotopy = H
        self.options = options or TrackerOptions()
        self._h = _Handle(make_options(self.options, None))
        self._h.setup_step_control(self.options)
        self._h.set_homotopy(H)

    def set_homotopy(self, H):
        self.homotopy = H
        self._h.set_homotopy(H)

    def track_arrays(self, starts, t1=1.0, t0=0.0):
        return self._h.track(starts, endgame=False, t1=t1, t0=t0)

    def track_batch(self, starts, t1=1.0, t0=0.0):
        res, sol, val, last = self._h.track(starts, endgame=False, t1=t1, t0=t0)
        out = []
        for k in range(len(res)):
            r = res[k]
            out.append(TrackerResult(
                return_code=TRACKER_CODES[int(r["return_code"])],
                solution=sol[k].copy(),
                t=complex(r["t_re"], r["t_im"]),
                accuracy=float(r["accuracy"]),
                accepted_steps=int(r["accepted_steps"]),
                rejected_steps=int(r["rejected_steps"]),
                extended_precision=bool(r["extended_precision"]),
                extended_precision_used=bool(r["extended_precision_used"]),
                omega=float(r["omega"]),
                mu=float(r["mu"]),
                tau=float(r["tau"]),
            ))
        return out

    def track(self, x, t1=1.0, t0=0.0) -> TrackerResult:
        return self.track_batch(np.asarray(x)[None, :], t1, t0)[0]


def total_degree(F: System, gamma=None, tracker_options=None, endgame_options=None, seed=None, devices=None):
    """(EndgameTracker, start solutions) for the total-degree homotopy of F
    (src/total_degree.jl:32-117). γ defaults to cis(2π u) drawn from ``seed``; ``devices``
    spreads every call's paths over several GPUs."""
    if gamma is None:
        gamma = random_gamma(np.random.default_rng(seed))
    H = total_degree_homotopy(F, gamma)
    T = EndgameTracker(H, tracker_options, endgame_options, devices=devices)
    return T, total_degree_start_solutions(H.degrees)


def track(tracker, x, t1=1.0, path_number=None):
    return tracker.track(x, t1, path_number=path_number)


# ------------------------------------------------------------------------------------------
# Result (src/result.jl) and multiplicity clustering (src/unique_points.jl:314-341)
# ------------------------------------------------------------------------------------------
def multiplicities(vectors, atol=1e-14, rtol=1e-8):
    """Clusters of indices whose Euclidean distance to an earlier representative is at most
    max(atol, rtol·‖v‖) (src/unique_points.jl:280-341)."""
    reps, rep_ids = [], []
    mults = {}
    for i, v in enumerate(vectors):
        rad = max(atol, rtol * np.linalg.norm(v))
        found = None
        for k, p in zip(rep_ids, reps):
            if np.linalg.norm(v - p) <= rad:
                found = k
                break
        if found is None:
            reps.append(v)
            rep_ids.append(i)
        else:
            mults.setdefault(found, [found]).append(i)
    return list(mults.values())


@dataclass
class Result:
    path_results: list
    seed: Optional[int] = None
    start_system: Optional[str] = None
    multiple_indicator: set = field(default_factory=set)

    def __post_init__(self):
        sing = [r for r in self.path_results if r.is_singular()]
        clusters = multiplicities([r.solution for r in sing])
        for cl in clusters:
            for i in cl[1:]:
                self.multiple_indicator.add(sing[i].path_number)
            for i in cl:
                sing[i].multiplicity = max(len(cl), sing[i].winding_number or 1)

    def __len__(self):
        return len(self.path_results)

    def is_multiple_result(self, r):
        return r.path_number in self.multiple_indicator

    def nresults(self, only_real=False, real_atol=1e-6, real_rtol=0.0, only_nonsingular=False,
                 only_singular=False, only_finite=True, multiple_results=False):
        c = 0
        for r in self.path_results:
            if ((not only_real or r.is_real(real_atol, real_rtol)) and (not only_nonsingular or r.is_nonsingular())
                    and (not only_singular or r.is_singular()) and (not only_finite or r.is_success())
                    and (multiple_results or not self.is_multiple_result(r))):
                c += 1
        return c

    def nsolutions(self, only_nonsingular=True, **kw):
        return self.nresults(only_nonsingular=only_nonsingular, **kw)

    def solutions(self, only_nonsingular=True):
        return [r.solution for r in self.path_results
                if r.is_success() and (not only_nonsingular or r.is_nonsingular()) and not self.is_multiple_result(r)]


def nnonsingular(R: Result):
    return sum(1 for r in R.path_results if r.is_nonsingular())


def nsingular(R: Result, counting_multiplicities=False):
    return R.nresults(only_singular=True, multiple_results=counting_multiplicities)


def nat_infinity(R: Result):
    return sum(1 for r in R.path_results if r.is_at_infinity())


def nfailed(R: Result):
    return sum(1 for r in R.path_results if r.is_failed())


def solve(F, starts=None, start_system: str = "total_degree", *, start_parameters=None, target_parameters=None,
          transform_result=None, transform_parameters=None, flatten: bool = False, gamma=None, seed=None,
          tracker_options=None, endgame_options=None, precision: str = "fp64", step_control: str = "plain",
          devices=None):
    """solve(F; start_system = :total_degree | :polyhedral) (src/solve.jl:447-526): one batched
    GPU call replaces threaded_solve's per-path loop (src/solve.jl:628-709); the polyhedral start
    system tracks its toric stage and its coefficient homotopy as one launch each.

    With ``start_parameters`` (F a parameters.ParametricSystem or an slp.Program with parameters,
    ``starts`` its solutions at the start parameters): the parameter homotopy to
    ``target_parameters``; a list of target parameter vectors runs the many-parameter solver
    (src/solve.jl:747-880), in one launch for term tables."""
    if start_parameters is not None:
        from . import parameters

        if starts is None:
            raise ValueError("a parameter homotopy needs start solutions")
        return parameters.solve(F, starts, start_parameters, target_parameters, tracker_options=tracker_options,
                                endgame_options=endgame_options, transform_result=transform_result,
                                transform_parameters=transform_parameters, flatten=flatten,
                                precision=precision, step_control=step_control)
    if start_system == "polyhedral":
        from .polyhedral_homotopy import solve_polyhedral

        if starts is not None:
            raise NotImplementedError("start solutions without start_parameters (a start system G) are not supported")
        to = tracker_options or TrackerOptions()
        to.precision = precision
        to.step_control = step_control
        return solve_polyhedral(F, seed=seed, tracker_options=to, endgame_options=endgame_options)
    if start_system != "total_degree":
        raise NotImplementedError("start_system must be 'total_degree' or 'polyhedral'")
    if starts is not None:
        raise NotImplementedError("start solutions without start_parameters (a start system G) are not supported")
    to = tracker_options or TrackerOptions()
    to.precision = precision
    to.step_control = step_control
    T, S = total_degree(F, gamma=gamma, tracker_options=to, endgame_options=endgame_options, seed=seed,
                        devices=devices)
    prs = T.track_batch(S)
    return Result(prs, seed=seed, start_system=start_system)
