"""Parameter homotopies of straight-line programs, on the CPU.

H(x, t) = F(x; t p + (1 - t) q) (src/homotopies/parameter_homotopy.jl:3-44) for a program F(x; p)
whose parameters enter in any way the ops allow:

* the oracle's H, ∂H/∂x and Taylor coefficients against exact symbolic differentiation (sympy)
  on the reference's own ParameterHomotopy test system (test/homotopies_test.jl:61-79:
  f = [(2x² + b²y³ + 2axy)³, (a + c)⁴x + y²], p = [5.2, -1.3, 9.3], q = [2.6, 3.3, 2.3]);
* oracle tracking from solutions of F(x; p₀) to F(x; p₁) against a total-degree solve of
  F(x; p₁);
* the program front end (evaluation, fixing the parameters, degree bounds, the choice between
  term tables and programs) and the generated CUDA C, compiled by NVRTC.
"""
import ctypes as ct
import os

import numpy as np
import pytest

import hcgpu as hc
from hcgpu import _lib, slp
from hcgpu.systems import variables as poly_variables

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "homotopycontinuation.jl_gb300", "csrc")
INCLUDE = os.path.join(ROOT, "include")

P_REF = [5.2, -1.3, 9.3]
Q_REF = [2.6, 3.3, 2.3]


def reference_system():
    (x, y), (a, b, c) = slp.variables_and_parameters(2, 3)
    return slp.Program([(2 * x ** 2 + b ** 2 * y ** 3 + 2 * a * x * y) ** 3, (a + c) ** 4 * x + y ** 2])


def _sympy_truth(kind, X, t0):
    sp = pytest.importorskip("sympy")
    x, y, a, b, c, t, s = sp.symbols("x y a b c t s")
    f = [(2 * x ** 2 + b ** 2 * y ** 3 + 2 * a * x * y) ** 3, (a + c) ** 4 * x + y ** 2]
    sub = {v: t * sp.nsimplify(pv) + (1 - t) * sp.nsimplify(qv) for v, pv, qv in zip((a, b, c), P_REF, Q_REF)}
    H = [sp.expand(e.subs(sub)) for e in f]
    R = lambda z: sp.nsimplify(z.real) + sp.I * sp.nsimplify(z.imag)  # exact inputs
    T0 = R(t0)
    if kind == "eval":
        vals = [h.subs({x: R(X[0]), y: R(X[1]), t: T0}) for h in H]
    elif kind == "jacobian":
        J = [[sp.diff(h, v) for v in (x, y)] for h in H]
        vals = [[e.subs({x: R(X[0]), y: R(X[1]), t: T0}) for e in row] for row in J]
    else:
        K = int(kind[-1])
        xs = sum(R(X[k][0]) * s ** k for k in range(K))
        ys = sum(R(X[k][1]) * s ** k for k in range(K))
        vals = []
        for h in H:
            e = sp.expand(h.subs({x: xs, y: ys, t: T0 + s}, simultaneous=True))
            vals.append(sp.Poly(e, s).coeff_monomial(s ** K))
    return np.array(sp.N(sp.Matrix(vals), 30).tolist(), dtype=np.complex128).reshape(np.shape(vals))


@pytest.mark.parametrize("kind", ["eval", "jacobian", "taylor1", "taylor2", "taylor3"])
def test_oracle_parameter_homotopy_matches_symbolic(kind):
    import hco

    P = reference_system()
    rng = np.random.default_rng(7)
    for t0 in (0.375, 0.25 + 0.125j):
        if kind in ("eval", "jacobian"):
            X = np.round(rng.normal(size=2) * 8 + 1j * rng.normal(size=2) * 8) / 8
        else:
            K = int(kind[-1])
            X = np.round((rng.normal(size=(K, 2)) + 1j * rng.normal(size=(K, 2))) * 8) / 8
        got = hco.slp_parameter_eval(P, P_REF, Q_REF, kind, X, t0)
        want = _sympy_truth(kind, X, t0)
        if kind == "jacobian":
            want = want.reshape(2, 2)
        err = np.abs(got - want).max() / max(np.abs(want).max(), 1.0)
        assert err <= 1e-13, (kind, t0, got, want)


def _family():
    """F(x; a, b) = [x₁² + a² x₂ - b³, x₂² - a b x₁ - 1]: parameters enter non-affinely."""
    (x1, x2), (a, b) = slp.variables_and_parameters(2, 2)
    return slp.Program([x1 * x1 + a * a * x2 - b ** 3, x2 * x2 - a * b * x1 - 1.0])


def _solve_fixed(P, p, seed):
    import hco

    F = P.fixed(p)
    rng = np.random.default_rng(seed)
    g = complex(np.exp(2j * np.pi * rng.random()))
    S = hc.total_degree_start_solutions(F.degrees)
    res, x, _, _ = hco.track_slp(F, g, S)
    ok = (res["return_code"] == 1) & (res["singular"] == 0)
    return x[ok]


def test_oracle_parameter_tracking_reaches_the_target_solutions():
    import hco

    P = _family()
    rng = np.random.default_rng(11)
    p0 = rng.normal(size=2) + 1j * rng.normal(size=2)
    p1 = rng.normal(size=2) + 1j * rng.normal(size=2)
    S0 = _solve_fixed(P, p0, 1)
    assert S0.shape[0] == 4  # Bézout 2·2, generic parameters
    res, x, _, _ = hco.track_slp_parameter(P, p0, p1, S0)
    assert (res["return_code"] == 1).all() and (res["singular"] == 0).all()
    for xi in x:
        r = P.evaluate(xi, p1)
        assert np.abs(r).max() <= 1e-10 * max(1.0, np.abs(xi).max() ** 3)
    S1 = _solve_fixed(P, p1, 2)
    # the same four solutions (distinct endpoints, each within 1e-8 of a total-degree solution)
    d = np.abs(x[:, None, :] - S1[None, :, :]).max(axis=2)
    assert (d.min(axis=1) <= 1e-8 * np.abs(S1).max()).all()
    assert len(set(d.argmin(axis=1).tolist())) == 4


def test_parameter_program_front_end():
    P = reference_system()
    assert (P.n, P.nparams) == (2, 3)
    assert P.degrees == [9, 2]  # degree bounds in x
    X = np.array([1 + 1j, 0.5 - 0.25j])
    xx, yy = X
    aa, bb, cc = P_REF
    want = [(2 * xx ** 2 + bb ** 2 * yy ** 3 + 2 * aa * xx * yy) ** 3, (aa + cc) ** 4 * xx + yy ** 2]
    assert np.allclose(P.evaluate(X, P_REF), want, rtol=1e-14)
    F0 = P.fixed(P_REF)
    assert F0.nparams == 0 and F0.degrees == [9, 2]
    assert np.allclose(F0.evaluate(X), want, rtol=1e-14)
    with pytest.raises(ValueError):
        P.evaluate(X)  # parameters missing
    ins, consts, voff, tape, outs = P.arrays()
    assert P.poff == voff + P.n and tape == P.poff + P.nparams + len(ins)
    H = hc.parameter_homotopy(P, P_REF, Q_REF)
    assert isinstance(H, slp.SLPParameterHomotopy)
    assert np.allclose(H.evaluate(X, 1.0), want)
    assert np.allclose(H.parameters(Q_REF, P_REF).evaluate(X, 0.0), want)
    # polynomials in (x, p): term tables when affine in p, a program otherwise
    V = poly_variables(4)  # x1, x2, a, b
    affine = hc.parametric_system([V[0] * V[0] - V[2], V[1] * V[0] - V[3] + 1.0], 2, 2)
    assert isinstance(affine, hc.ParametricSystem)
    general = hc.parametric_system([V[0] * V[0] - V[2] * V[2], V[1] * V[0] - V[3] ** 3 + 1.0], 2, 2)
    assert isinstance(general, slp.Program) and general.nparams == 2 and general.degrees == [2, 2]
    x = np.array([0.3 + 0.1j, -0.7j])
    pv = np.array([1.5 - 0.5j, 0.25 + 2j])
    assert np.allclose(general.evaluate(x, pv), [x[0] ** 2 - pv[0] ** 2, x[1] * x[0] - pv[1] ** 3 + 1])
    with pytest.raises(NotImplementedError):
        hc.ParametricSystem.from_polys([V[0] * V[0] - V[2] * V[2], V[1] - V[3]], 2, 2)


def _nvrtc():
    for path in ("/usr/local/cuda/lib64/libnvrtc.so", "libnvrtc.so"):
        try:
            return ct.CDLL(path)
        except OSError:
            continue
    pytest.skip("NVRTC not found")


def test_parameter_source_compiles_with_nvrtc():
    P = reference_system()
    src = slp.source(P)
    assert "constexpr int NP = 3;" in src and "param_at(pq[0], pq[3], t)" in src and "p2_1 = pq[2] - pq[5]" in src
    src += "template __global__ void hcd::track_kernel<false>(const __grid_constant__ hcd::Launch la);\n"
    L = _nvrtc()
    prog = ct.c_void_p()
    assert L.nvrtcCreateProgram(ct.byref(prog), src.encode(), b"slp_param.cu", 0, None, None) == 0
    opts = [b"--gpu-architecture=sm_103a", b"-std=c++17", b"-default-device", b"-diag-suppress=39,177",
            b"-I" + CSRC.encode(), b"-I" + INCLUDE.encode()]
    rc = L.nvrtcCompileProgram(prog, len(opts), (ct.c_char_p * len(opts))(*opts))
    n = ct.c_size_t()
    L.nvrtcGetProgramLogSize(prog, ct.byref(n))
    log = ct.create_string_buffer(n.value)
    L.nvrtcGetProgramLog(prog, log)
    assert rc == 0, log.value.decode()[:2000]
    L.nvrtcDestroyProgram(ct.byref(prog))


def _raw_param(instrs, consts, voff, poff, np_, tape, outs, n):
    ins = np.zeros(len(instrs), dtype=slp.INSTR_DTYPE)
    for k, (inp, op, out) in enumerate(instrs):
        ins[k]["input"] = list(inp) + [0] * (4 - len(inp))
        ins[k]["op"] = slp.OP[op]
        ins[k]["output"] = out
    c = np.asarray(consts, dtype=np.float64)
    o = np.asarray(outs, dtype=np.int32)
    s = slp.hc_slp(n, len(ins), ins.ctypes.data, len(consts) // 2, c.ctypes.data, voff, tape, o.ctypes.data)
    L = _lib.load()
    ln = ct.c_int64()
    rc = L.hc_slp_parameter_source(ct.byref(s), np_, poff, None, 0, ct.byref(ln))
    return rc, L.hc_last_error(None).decode()


def test_parameter_program_validation():
    # slot 0 constant 1; slots 1, 2 variables x, y; slot 3 parameter a; F = (x y - a, x + y - 1)
    ok = [((1, 2), "MUL", 4), ((4, 3), "SUB", 5), ((1, 2), "ADD", 6), ((6, 0), "SUB", 7)]
    assert _raw_param(ok, [1.0, 0.0], 1, 3, 1, 8, [5, 7], 2)[0] == 0
    rc, msg = _raw_param(ok, [1.0, 0.0], 1, 2, 1, 8, [5, 7], 2)  # parameter on a variable's slot
    assert rc == 1 and "parameters must occupy" in msg
    rc, msg = _raw_param(ok[:3] + [((6, 0), "SUB", 3)], [1.0, 0.0], 1, 3, 1, 8, [5, 3], 2)  # overwrites a
    assert rc == 1 and "parameter" in msg
    rc, msg = _raw_param(ok, [1.0, 0.0], 1, 3, 0, 8, [5, 7], 2)
    assert rc == 1 and "nparameters" in msg
