"""ctypes harness for the CPU oracle (oracle/hc_oracle.cpp).

TEST INFRASTRUCTURE ONLY: imported by tests/, __graft_entry__.smoke() and bench.py's
cpu_baseline / reference legs as the checker. The product never imports this module.
"""
from __future__ import annotations

import ctypes as ct
import os
import subprocess

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "_build", "libhcoracle.so")
_lib = None


def build(force: bool = False) -> str:
    src = os.path.join(_HERE, "hc_oracle.cpp")
    if force or not os.path.exists(_LIB_PATH) or os.path.getmtime(_LIB_PATH) < os.path.getmtime(src):
        subprocess.run(["make", "-s", "-C", _HERE], check=True)
    return _LIB_PATH


class Options(ct.Structure):
    _fields_ = [
        ("max_steps", ct.c_int32),
        ("extended_precision", ct.c_int32),
        ("max_step_size", ct.c_double),
        ("max_initial_step_size", ct.c_double),
        ("min_step_size", ct.c_double),
        ("min_rel_step_size", ct.c_double),
        ("terminate_cond", ct.c_double),
        ("a", ct.c_double),
        ("beta_a", ct.c_double),
        ("beta_omega_p", ct.c_double),
        ("beta_tau", ct.c_double),
        ("strict_beta_tau", ct.c_double),
        ("min_newton_iters", ct.c_int32),
        ("max_endgame_steps", ct.c_int32),
        ("max_endgame_extended_steps", ct.c_int32),
        ("max_winding_number", ct.c_int32),
        ("zero_is_at_infinity", ct.c_int32),
        ("at_infinity_check", ct.c_int32),
        ("only_nonsingular", ct.c_int32),
        ("refine_steps", ct.c_int32),
        ("endgame_start", ct.c_double),
        ("min_cond", ct.c_double),
        ("min_cond_growth", ct.c_double),
        ("min_coord_growth", ct.c_double),
        ("singular_min_accuracy", ct.c_double),
        ("val_finite_tol", ct.c_double),
        ("val_at_infinity_tol", ct.c_double),
        ("sing_cond", ct.c_double),
        ("sing_accuracy", ct.c_double),
        ("scaling_threshold", ct.c_double),
    ]


class PathResult(ct.Structure):
    _fields_ = [
        ("return_code", ct.c_int32),
        ("winding_number", ct.c_int32),
        ("t_re", ct.c_double),
        ("t_im", ct.c_double),
        ("accuracy", ct.c_double),
        ("residual", ct.c_double),
        ("cond", ct.c_double),
        ("omega", ct.c_double),
        ("mu", ct.c_double),
        ("tau", ct.c_double),
        ("singular", ct.c_int32),
        ("extended_precision", ct.c_int32),
        ("extended_precision_used", ct.c_int32),
        ("_pad", ct.c_int32),
        ("accepted_steps", ct.c_int64),
        ("rejected_steps", ct.c_int64),
        ("steps_eg", ct.c_int64),
        ("path_number", ct.c_int64),
        ("last_t", ct.c_double),
    ]


RESULT_DTYPE = np.dtype(
    [
        ("return_code", np.int32),
        ("winding_number", np.int32),
        ("t_re", np.float64),
        ("t_im", np.float64),
        ("accuracy", np.float64),
        ("residual", np.float64),
        ("cond", np.float64),
        ("omega", np.float64),
        ("mu", np.float64),
        ("tau", np.float64),
        ("singular", np.int32),
        ("extended_precision", np.int32),
        ("extended_precision_used", np.int32),
        ("_pad", np.int32),
        ("accepted_steps", np.int64),
        ("rejected_steps", np.int64),
        ("steps_eg", np.int64),
        ("path_number", np.int64),
        ("last_t", np.float64),
    ]
)
assert RESULT_DTYPE.itemsize == ct.sizeof(PathResult)


def lib():
    global _lib
    if _lib is None:
        build()
        L = ct.CDLL(_LIB_PATH)
        P = ct.c_void_p
        L.hco_default_options.argtypes = [ct.POINTER(Options)]
        L.hco_track.restype = ct.c_int
        L.hco_track.argtypes = [
            ct.c_int, ct.c_int, P, P, P, ct.c_int, P, P, P, ct.c_double, ct.c_double,
            ct.c_int64, P, ct.c_int, ct.c_double, ct.c_double, ct.c_double, ct.c_double,
            ct.POINTER(Options), ct.c_int, P, P, P, P,
        ]
        L.hco_track_toric.restype = ct.c_int
        L.hco_track_toric.argtypes = [
            ct.c_int, ct.c_int, P, P, P, ct.c_int, P, ct.c_int64, P, P, P, P, P, P,
            ct.POINTER(Options), ct.c_int, P, P,
        ]
        L.hco_ldiv.argtypes = [ct.c_int, P, P, P]
        L.hco_inverse_inf_norm_est.argtypes = [ct.c_int, P, P, P, P, P]
        L.hco_dd_op.argtypes = [ct.c_int, P, P, P]
        L.hco_norm.restype = ct.c_double
        L.hco_norm.argtypes = [ct.c_int, P, P]
        L.hco_homotopy_eval.argtypes = [
            ct.c_int, ct.c_int, P, P, P, ct.c_int, P, P, P, ct.c_double, ct.c_double,
            ct.c_int, P, ct.c_double, ct.c_double, P,
        ]
        _lib = L
    return _lib


def default_options(**kw) -> Options:
    o = Options()
    lib().hco_default_options(ct.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    return o


def _ptr(a):
    return a.ctypes.data_as(ct.c_void_p) if a is not None else None


def _cplx(a):
    a = np.ascontiguousarray(np.asarray(a, dtype=np.complex128))
    return a


def track(G_terms, F_terms, gamma, starts, *, endgame=True, t1=1.0, t0=0.0, options=None, nthreads=0):
    """Track each row of ``starts`` (paths × n complex) with the oracle.

    G_terms / F_terms: (eq int32[T], exps int32[T×n], coef float64[T×2]).
    Returns (results structured array, endpoints complex[paths×n], extra1, extra2) where
    extra1 = valuation val_x and extra2 = last_path_point (endgame) or val_tẋ (plain tracker).
    """
    starts = _cplx(starts)
    npaths, n = starts.shape
    Ge, Gx, Gc = G_terms
    Fe, Fx, Fc = F_terms
    opts = options if options is not None else default_options()
    res = np.zeros(npaths, dtype=RESULT_DTYPE)
    xs = np.zeros((npaths, n), dtype=np.complex128)
    val = np.zeros((npaths, n), dtype=np.float64)
    last = np.zeros((npaths, n), dtype=np.complex128)
    t1 = complex(t1)
    t0 = complex(t0)
    lib().hco_track(
        n, len(Ge), _ptr(Ge), _ptr(Gx), _ptr(Gc), len(Fe), _ptr(Fe), _ptr(Fx), _ptr(Fc),
        gamma.real, gamma.imag, npaths, _ptr(starts), 1 if endgame else 0,
        t1.real, t1.imag, t0.real, t0.imag, ct.byref(opts), int(nthreads),
        _ptr(res), _ptr(xs), _ptr(val), _ptr(last),
    )
    return res, xs, val, last


def track_toric(F_terms, weights, starts, rows, t1, t0, omega=None, mu=None, options=None, nthreads=0):
    """Toric stage of the polyhedral method with the oracle: path k from t1[k] to t0[k] with
    weight row rows[k] (weights: rows × terms of F_terms, in their order). Returns (results,
    endpoints)."""
    starts = _cplx(starts)
    npaths, n = starts.shape
    Fe, Fx, Fc = F_terms
    W = np.ascontiguousarray(weights, dtype=np.float64)
    opts = options if options is not None else default_options()
    res = np.zeros(npaths, dtype=RESULT_DTYPE)
    xs = np.zeros((npaths, n), dtype=np.complex128)
    f64 = lambda a: None if a is None else np.ascontiguousarray(a, dtype=np.float64)
    rows = np.ascontiguousarray(rows, dtype=np.int32)
    t1, t0, omega, mu = f64(t1), f64(t0), f64(omega), f64(mu)
    lib().hco_track_toric(n, len(Fe), _ptr(Fe), _ptr(Fx), _ptr(Fc), W.shape[0], _ptr(W), npaths, _ptr(starts),
                          _ptr(rows), _ptr(t1), _ptr(t0), _ptr(omega), _ptr(mu), ct.byref(opts), int(nthreads),
                          _ptr(res), _ptr(xs))
    return res, xs


def set_slp(program=None, start_parameters=None, target_parameters=None):
    """Evaluate F as the straight-line program ``program`` (hcgpu.slp.Program) in the following
    track() / homotopy_eval() calls; None switches back to term tables. A program with
    parameters is tracked as the parameter homotopy F(x; t p + (1 - t) q)."""
    L = lib()
    L.hco_set_slp.argtypes = [ct.c_int, ct.c_int, ct.c_void_p, ct.c_int, ct.c_void_p, ct.c_int, ct.c_int,
                              ct.c_void_p]
    L.hco_set_slp_parameters.argtypes = [ct.c_int, ct.c_int, ct.c_void_p, ct.c_void_p]
    if program is None:
        L.hco_set_slp(0, -1, None, 0, None, 0, 0, None)
        return
    ins, consts, voff, tape, outs = program.arrays()
    flat = np.ascontiguousarray(np.column_stack([ins["input"], ins["op"], ins["output"]]).astype(np.int32))
    consts = np.ascontiguousarray(consts if consts.size else np.zeros(2))
    outs = np.ascontiguousarray(outs, dtype=np.int32)
    L.hco_set_slp(program.n, len(ins), _ptr(flat), len(consts) // 2 if len(program._tape.consts) else 0,
                  _ptr(consts), voff, tape, _ptr(outs))
    if getattr(program, "nparams", 0):
        p = _cplx(start_parameters)
        q = _cplx(target_parameters)
        assert p.shape[0] == q.shape[0] == program.nparams
        L.hco_set_slp_parameters(program.nparams, program.poff, _ptr(p), _ptr(q))


def track_slp(program, gamma, starts, **kw):
    """track() of γ t G + (1 - t) F with F = program and G_i = s_i (x_i^{D_i} - 1) from the
    program's degrees and scalings."""
    n = program.n
    eq, ex, cf = [], [], []
    for i, (d, sc) in enumerate(zip(program.degrees, program.scaling)):
        e = [0] * n
        e[i] = int(d)
        eq += [i, i]
        ex += [e, [0] * n]
        cf += [sc, -sc]
    G = (np.asarray(eq, np.int32), np.asarray(ex, np.int32).reshape(-1, n), np.asarray(cf, np.complex128))
    F = (np.zeros(0, np.int32), np.zeros((0, n), np.int32), np.zeros(0, np.complex128))
    set_slp(program)
    try:
        return track(G, F, gamma, starts, **kw)
    finally:
        set_slp(None)


def _no_terms(n):
    return (np.zeros(0, np.int32), np.zeros((0, n), np.int32), np.zeros(0, np.complex128))


def track_slp_parameter(program, start_parameters, target_parameters, starts, **kw):
    """track() of the parameter homotopy F(x; t p + (1 - t) q), F = program (with parameters),
    from start solutions of F(x; p) at t = 1 to t = 0."""
    set_slp(program, start_parameters, target_parameters)
    try:
        return track(_no_terms(program.n), _no_terms(program.n), 1.0 + 0j, starts, **kw)
    finally:
        set_slp(None)


def slp_parameter_eval(program, start_parameters, target_parameters, kind, x, t):
    """homotopy_eval() of the parameter homotopy of ``program`` (kinds as there)."""
    set_slp(program, start_parameters, target_parameters)
    try:
        return homotopy_eval(_no_terms(program.n), _no_terms(program.n), 1.0 + 0j, kind, x, t)
    finally:
        set_slp(None)


TRACE_FIELDS = ["t_re", "t_im", "ds", "tau", "omega", "mu", "accepted", "iters", "norm_x", "ds_next",
                "omega_after", "accuracy", "extended_prec", "code", "steps_eg"]


def trace_path(G_terms, F_terms, gamma, starts, path, **kw):
    """Track ``starts`` and return (results..., per-step trace of path index ``path``)."""
    L = lib()
    L.hco_set_trace.argtypes = [ct.c_int64]
    L.hco_get_trace.argtypes = [ct.c_void_p, ct.c_int64]
    L.hco_get_trace.restype = ct.c_int64
    L.hco_set_trace(int(path))
    try:
        out = track(G_terms, F_terms, gamma, starts, **kw)
    finally:
        L.hco_set_trace(-1)
    nrec = L.hco_get_trace(None, 0)
    buf = np.zeros((max(nrec, 1), len(TRACE_FIELDS)))
    L.hco_get_trace(_ptr(buf), nrec)
    return out, buf[:nrec]


def ldiv(A, b):
    A = np.asfortranarray(np.asarray(A, dtype=np.complex128))
    n = A.shape[0]
    Af = np.ascontiguousarray(A.reshape(-1, order="F"))
    b = _cplx(b)
    x = np.zeros(n, dtype=np.complex128)
    lib().hco_ldiv(n, _ptr(Af), _ptr(b), _ptr(x))
    return x


def inverse_inf_norm_est(A, d_l=None, d_r=None):
    A = np.asarray(A, dtype=np.complex128)
    n = A.shape[0]
    Af = np.ascontiguousarray(A.reshape(-1, order="F"))
    dl = None if d_l is None else np.ascontiguousarray(d_l, dtype=np.float64)
    dr = None if d_r is None else np.ascontiguousarray(d_r, dtype=np.float64)
    est = np.zeros(1)
    cond = np.zeros(1)
    lib().hco_inverse_inf_norm_est(n, _ptr(Af), _ptr(dl), _ptr(dr), _ptr(est), _ptr(cond))
    return float(est[0]), float(cond[0])


def dd_op(op, a, b):
    a = np.ascontiguousarray(a, dtype=np.float64)
    b = np.ascontiguousarray(b, dtype=np.float64)
    c = np.zeros(2)
    lib().hco_dd_op({"add": 0, "sub": 1, "mul": 2}[op], _ptr(a), _ptr(b), _ptr(c))
    return float(c[0]), float(c[1])


def norm(x, w=None):
    x = _cplx(x)
    ww = None if w is None else np.ascontiguousarray(w, dtype=np.float64)
    return lib().hco_norm(len(x), _ptr(x), _ptr(ww))


def homotopy_eval(G_terms, F_terms, gamma, kind, x, t):
    """kind: 'eval', 'eval_dd', 'jacobian', 'taylor1', 'taylor2', 'taylor3'.
    For taylorK, x is a (K × n) array of series coefficients (orders 0..K-1)."""
    k = {"eval": 0, "eval_dd": 1, "jacobian": 2, "taylor1": 3, "taylor2": 4, "taylor3": 5}[kind]
    x = _cplx(x)
    n = x.shape[-1]
    Ge, Gx, Gc = G_terms
    Fe, Fx, Fc = F_terms
    out = np.zeros(n * n if k == 2 else n, dtype=np.complex128)
    t = complex(t)
    lib().hco_homotopy_eval(
        n, len(Ge), _ptr(Ge), _ptr(Gx), _ptr(Gc), len(Fe), _ptr(Fe), _ptr(Fx), _ptr(Fc),
        gamma.real, gamma.imag, k, _ptr(x), t.real, t.imag, _ptr(out),
    )
    if k == 2:
        return out.reshape(n, n, order="F")
    return out
