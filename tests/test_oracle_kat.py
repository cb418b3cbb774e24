"""The CPU oracle against the reference's own known-answer tests (pinning the oracle).

Each case cites the reference test it restates; systems and fixed γ come from
tests/golden/kat_systems.json (generated from the reference test files)."""
import fractions

import numpy as np
import pytest

import hco
import hcgpu as hc
from _kat import KAT, gamma, system, winding_family


def track(H, S=None, **kw):
    S = hc.total_degree_start_solutions(H.degrees) if S is None else S
    return hco.track(H.G.term_arrays(), H.F.term_arrays(), H.gamma, S, **kw)


def nonsingular(res):
    return int(((res["return_code"] == 1) & (res["singular"] == 0)).sum())


def test_endgame_tracker_quadrics():
    # test/endgame_tracker_test.jl:2-31
    H = hc.total_degree_homotopy(system("quadrics_2x2"), gamma("quadrics_2x2"))
    res, x, val, last = track(H)
    assert [hc.ENDGAME_CODES[c] for c in res["return_code"]] == KAT["quadrics_2x2"]["expect"]["codes"]
    assert (res["accuracy"][:2] < 1e-12).all() and (res["residual"][:2] < 1e-12).all()
    assert (res["accepted_steps"][:2] + res["rejected_steps"][:2] < 20).all()
    assert (res["rejected_steps"][:2] == 0).all()
    assert res["cond"][1] < 1e3 and res["singular"][1] == 0
    np.testing.assert_allclose(val[2], [-1, -1], rtol=1e-3)
    np.testing.assert_allclose(val[3], [-1, -1], rtol=1e-3)


@pytest.mark.parametrize("d", [2, 4, 6])
def test_winding_number_family(d):
    # test/endgame_test.jl:62-69: d + 1 successful paths
    for k in range(3):
        H = hc.total_degree_homotopy(winding_family(d), np.exp(2j * np.pi * (k + 0.37) / 3))
        res, *_ = track(H)
        assert (res["return_code"] == 1).sum() == d + 1


def test_wilkinson_12():
    # test/endgame_test.jl:38-45: roots 1..12, tiny imaginary parts
    (x,) = hc.variables(1)
    p = hc.Poly.const(1.0, 1)
    for i in range(1, 13):
        p = p * (x - i)
    H = hc.total_degree_homotopy(hc.System.from_polys([p]), np.exp(2j * np.pi * 0.21))
    res, xs, _, _ = track(H)
    assert (res["return_code"] == 1).all()
    assert np.round(np.sort(xs[:, 0].real)).astype(int).tolist() == list(range(1, 13))
    assert np.abs(xs[:, 0].imag).max() < 1e-4


def test_mohab_fixed_gamma():
    # test/endgame_test.jl:76-107: 693 nonsingular, including the γ that used to jump paths
    H = hc.total_degree_homotopy(system("mohab"), gamma("mohab"))
    res, *_ = track(H)
    assert nonsingular(res) == KAT["mohab"]["expect"]["nnonsingular"]


def test_cyclic7():
    # test/endgame_test.jl:2-5: cyclic(7) via total degree has 924 nonsingular solutions
    H = hc.total_degree_homotopy(hc.cyclic(7), np.exp(2j * np.pi * 0.31))
    res, *_ = track(H)
    assert nonsingular(res) == KAT["cyclic7"]["expect"]["nsolutions"]


@pytest.mark.parametrize("k", range(3))
def test_dynamic_polynomials_18(k):
    # test/solve_test.jl:338-344: f₁ = (x⁴ + y⁴ − 1)(x² + y² − 2) + x⁵y, f₂ = x² + 2xy² − 2y² − 1/2
    # has 18 solutions (total degree 6·3 = 18: every path ends at a nonsingular solution), for
    # any generic γ
    H = hc.total_degree_homotopy(system("dynamic_polynomials_18"), np.exp(2j * np.pi * (0.13 + k / 3)))
    res, *_ = track(H)
    assert nonsingular(res) == KAT["dynamic_polynomials_18"]["expect"]["nsolutions"] == 18


@pytest.mark.parametrize("k", range(3))
def test_beyond_polyhedral_example(k):
    # test/endgame_test.jl:54-60: the 2×2 quadrics by total degree: 2 successes, 2 at infinity
    e = KAT["beyond_polyhedral"]["expect"]
    H = hc.total_degree_homotopy(system("beyond_polyhedral"), np.exp(2j * np.pi * (0.07 + k / 3)))
    res, *_ = track(H)
    codes = [hc.ENDGAME_CODES[int(c)] for c in res["return_code"]]
    assert codes.count("success") == e["success"] and codes.count("at_infinity") == e["at_infinity"]


def test_straight_line_tracker():
    # test/tracker_test.jl:93-105: Tracker on t G + (1 - t) F from G's roots succeeds; from
    # [100, -100] (not a root of G) the start value is invalid
    from _kat import straight_line_homotopy

    d = KAT["straight_line_tracker"]
    H = straight_line_homotopy()
    S = np.array(d["starts"] + [d["invalid_start"]], dtype=np.complex128)
    res, x, _, _ = track(H, S, endgame=False, t1=1.0, t0=0.0)
    assert [hc.TRACKER_CODES[int(c)] for c in res["return_code"]] == ["success", "success",
                                                                      "terminated_invalid_startvalue"]
    F = H.F
    for xi in x[:2]:
        assert np.abs(F.evaluate(xi)).max() < 1e-12


def test_valuation_examples():
    # test/valuation_test.jl:20-44 (Example 2) and :46-74 (Example 3), conservative parameters
    o = hco.default_options(beta_omega_p=4.0, beta_tau=0.25, strict_beta_tau=0.1875)
    H = hc.total_degree_homotopy(system("quadrics_2x2"), gamma("quadrics_2x2"))
    S = hc.total_degree_start_solutions(H.degrees)
    tf = 1e-10
    res, x, val, vtx = track(H, S[2:3], endgame=False, t1=1.0, t0=tf, options=o)
    assert res["return_code"][0] == 1
    np.testing.assert_allclose(val[0], [-1, -1], atol=10 * tf ** 0.5)
    np.testing.assert_allclose(vtx[0].real, [-1, -1], atol=tf ** 0.5)
    a = KAT["valuation_example3_a"]
    x_, y_ = hc.variables(2)
    f1 = (a[0] * x_**2 + a[1] * y_) * (a[2] * x_ + a[3] * y_) + 1
    f2 = (a[0] * x_**2 + a[1] * y_) * (a[4] * x_ + a[5] * y_) + 1
    H = hc.total_degree_homotopy(hc.System.from_polys([f1, f2]), gamma("quadrics_2x2"))
    S = hc.total_degree_start_solutions(H.degrees)
    res, x, val, vtx = track(H, S[2:3], endgame=False, t1=1.0, t0=tf, options=o)
    np.testing.assert_allclose(val[0], [-1 / 6, -2 / 6], atol=tf ** (1 / 6))
    np.testing.assert_allclose(vtx[0].real, [-1 / 6, -2 / 6], atol=tf ** (1 / 6))


@pytest.mark.parametrize("n", [3, 13, 31])
def test_ldiv(n):
    # test/linear_algebra_test.jl:51-64: ldiv! matches lu(A) \ b
    rng = np.random.default_rng(n)
    A = rng.normal(size=(n, n)) + 1j * rng.normal(size=(n, n))
    b = rng.normal(size=n) + 1j * rng.normal(size=n)
    x = hco.ldiv(A, b)
    ref = np.linalg.solve(A, b)
    assert np.linalg.norm(x - ref) / np.linalg.norm(ref) < 1e-13 * np.linalg.cond(A)


def test_inverse_inf_norm_estimator():
    # test/linear_algebra_test.jl:66-109: Higham estimate within 10x, with scalings
    rng = np.random.default_rng(5)
    d_r = rng.random() * 10.0 ** np.linspace(-6, 6, 6)
    d_l = rng.random() * 10.0 ** np.linspace(6, -6, 6)
    A = rng.normal(size=(6, 6)).astype(complex)
    inf = lambda M: np.abs(M).sum(axis=1).max()
    B = A @ np.diag(1 / d_r)
    est, cnd = hco.inverse_inf_norm_est(B)
    assert 0.1 <= inf(np.linalg.inv(B)) / est <= 10
    assert 0.1 <= np.linalg.cond(B, np.inf) / cnd <= 10
    est, _ = hco.inverse_inf_norm_est(B, None, d_r)
    assert 0.1 <= inf(np.linalg.inv(B @ np.diag(d_r))) / est <= 10
    est, _ = hco.inverse_inf_norm_est(B, d_r, None)
    assert 0.1 <= inf(np.linalg.inv(np.diag(d_r) @ B)) / est <= 10
    D = np.diag(1 / d_l) @ A @ np.diag(1 / d_r)
    est, cnd = hco.inverse_inf_norm_est(D, d_l, d_r)
    assert 0.1 <= inf(np.linalg.inv(np.diag(d_l) @ D @ np.diag(d_r))) / est <= 10
    assert hco.inverse_inf_norm_est(D, d_r, d_l)[0] > 100 * est


def test_double_double_arithmetic():
    # test/double_double_test.jl:67-95: +, −, × against exact rationals
    rng = np.random.default_rng(1)
    F = fractions.Fraction
    for _ in range(50):
        a = (rng.random() * 20 - 10, rng.random() * 1e-16)
        b = (rng.random() * 20 - 10, rng.random() * 1e-16)
        fa, fb = F(a[0]) + F(a[1]), F(b[0]) + F(b[1])
        for op, exact, tol in (("add", fa + fb, 1e-30), ("sub", fa - fb, 1e-30), ("mul", fa * fb, 1e-29)):
            hi, lo = hco.dd_op(op, np.array(a), np.array(b))
            assert abs(float(F(hi) + F(lo) - exact)) < tol


def test_norms_with_overflow():
    # test/norm_test.jl
    x = np.array([2.0j, 3.0 - 1j, 5.0 + 2.0j])
    y = np.array([-2.0j, 3.0 - 1j, 5.0 + 2.0j])
    assert np.isclose(hco.norm(x), abs(5 + 2j))
    assert np.isclose(hco.norm(x - y), 4)
    huge = 2.0**700
    assert np.isclose(hco.norm(huge * x), huge * abs(5 + 2j))
    w = np.array([4.0, 2.0, 2.0])
    assert np.isclose(hco.norm(x, w), 0.5 * abs(5 + 2j))
    assert np.isclose(hco.norm(huge * x, w), huge * 0.5 * abs(5 + 2j))


def _series_coeffs(H, tx, K):
    """Exact-order Taylor coefficients of γ t G + (1-t) F along x(ε)=Σ tx_k ε^k, computed
    independently with numpy polynomial products."""
    P = np.polynomial.polynomial

    def sys_series(S):
        out = []
        for e, c in zip(S.exponents, S.coefficients):
            acc = np.zeros(K + 1, dtype=complex)
            for row, cf in zip(e, c):
                term = np.array([cf], dtype=complex)
                for j, p in enumerate(row):
                    xs = np.array([tx[k][j] for k in range(len(tx))], dtype=complex)
                    for _ in range(p):
                        term = P.polymul(term, xs)[: K + 1]
                acc[: len(term)] += term
            out.append(acc)
        return np.array(out)

    return sys_series(H.G), sys_series(H.F)


def test_taylor_coefficients():
    # test/model_kit/e2e_test.jl:66-91: taylor! order K equals the series coefficient
    F, g = hc.dense_random_system(3, 3, seed=11)
    H = hc.total_degree_homotopy(F, g)
    rng = np.random.default_rng(2)
    tx = [rng.normal(size=3) + 1j * rng.normal(size=3) for _ in range(3)]
    t = 0.3 + 0.1j
    for K in (2, 3):
        u = hco.homotopy_eval(H.G.term_arrays(), H.F.term_arrays(), H.gamma, f"taylor{K}", np.array(tx[:K]), t)
        dg, df = _series_coeffs(H, tx[:K], K)
        ref = H.gamma * (dg[:, K - 1] + t * dg[:, K]) + (1 - t) * df[:, K] - df[:, K - 1]
        np.testing.assert_allclose(u, ref, rtol=1e-12, atol=1e-12 * np.abs(ref).max())
    u1 = hco.homotopy_eval(H.G.term_arrays(), H.F.term_arrays(), H.gamma, "taylor1", np.array(tx[:1]), t)
    np.testing.assert_allclose(u1, H.gamma * H.G.evaluate(tx[0]) - H.F.evaluate(tx[0]), rtol=1e-12)
    # double-double residual equals the plain one to FP64 rounding
    ue = hco.homotopy_eval(H.G.term_arrays(), H.F.term_arrays(), H.gamma, "eval", np.array([tx[0]]), t)
    ud = hco.homotopy_eval(H.G.term_arrays(), H.F.term_arrays(), H.gamma, "eval_dd", np.array([tx[0]]), t)
    np.testing.assert_allclose(ud, ue, rtol=1e-13)
    J = hco.homotopy_eval(H.G.term_arrays(), H.F.term_arrays(), H.gamma, "jacobian", np.array([tx[0]]), t)
    eps = 1e-7
    for j in range(3):
        e = np.zeros(3, complex)
        e[j] = eps
        fd = (hco.homotopy_eval(H.G.term_arrays(), H.F.term_arrays(), H.gamma, "eval", np.array([tx[0] + e]), t)
              - hco.homotopy_eval(H.G.term_arrays(), H.F.term_arrays(), H.gamma, "eval", np.array([tx[0] - e]), t)) / (2 * eps)
        np.testing.assert_allclose(J[:, j], fd, rtol=1e-6)


def _oracle_result(name, g):
    from hcgpu.tracking import Result, _path_results

    H = hc.total_degree_homotopy(system(name), g)
    S = hc.total_degree_start_solutions(H.degrees)
    res, x, val, last = track(H, S)
    return res, Result(_path_results(res, x, val, last, S, 0.1))


@pytest.mark.parametrize("k", range(3))
def test_hyperbolic_6_6_multiplicity(k):
    # test/endgame_test.jl:7-22: 12 paths of winding number 3, 2 singular results of multiplicity 6
    e = KAT["hyperbolic_6_6"]["expect"]
    res, R = _oracle_result("hyperbolic_6_6", np.exp(2j * np.pi * (0.1 + k / 3)))
    assert int((res["winding_number"] == e["winding_number"]).sum()) == e["n_winding"]
    assert R.nresults() == e["nresults"]
    assert hc.nsingular(R) == e["nsingular"]
    assert all(r.multiplicity == e["multiplicity"] for r in R.path_results)


@pytest.mark.parametrize("k", range(3))
def test_singular_1_multiplicity(k):
    # test/endgame_test.jl:24-36: one singular solution (multiplicity 3) and one nonsingular
    e = KAT["singular_1"]["expect"]
    res, R = _oracle_result("singular_1", np.exp(2j * np.pi * (0.1 + k / 3)))
    assert hc.nsingular(R) == e["nsingular"]
    assert R.nresults(only_nonsingular=True) == e["nresults_nonsingular"]
    assert sorted(r.multiplicity for r in R.path_results if r.is_singular()) == [3, 3, 3]


def test_at_infinity_decision_depends_on_step_parameters():
    """On the endgame-heavy system (8 sparse quartics, seed 0) the reference's at-infinity
    heuristic (src/endgame_tracker.jl:424-499) decides two borderline paths differently when
    only its step parameters change (src/tracker.jl:58-62): path 61576 (a solution of norm
    2.8e6, cond 1.7e11) is found with the default parameters but declared at infinity with
    CONSERVATIVE_TRACKER_PARAMETERS; path 22314 is at infinity by default but a singular
    solution with FAST_TRACKER_PARAMETERS. Counts of two trackers whose step sequences differ
    (learned step control, or another evaluation order) can therefore differ on such paths."""
    F, g = hc.sparse_random_system(8, 8, 4, seed=0)
    H = hc.total_degree_homotopy(F, g)
    S = hc.total_degree_start_solutions(H.degrees)
    fast = dict(beta_omega_p=2.0, beta_tau=0.75, strict_beta_tau=0.4)
    conservative = dict(beta_omega_p=4.0, beta_tau=0.25, strict_beta_tau=0.1875)

    def code(p, **kw):
        res, x, _, _ = track(H, S[p:p + 1], options=hco.default_options(**kw))
        return hc.ENDGAME_CODES[res["return_code"][0]], bool(res["singular"][0]), float(np.abs(x[0]).max())

    c, sing, nx = code(61576)
    assert (c, sing) == ("success", False) and 1e6 < nx < 1e7
    c, sing, nx = code(61576, **conservative)
    assert c == "at_infinity" and 1e4 < nx < 1e5
    assert code(22314)[0] == "at_infinity"
    c, sing, nx = code(22314, **fast)
    assert (c, sing) == ("success", True) and nx > 1e10


@pytest.mark.parametrize("d", [2, 6])
def test_x_minus_10_power_as_program(d):
    # test/endgame_test.jl:47-52: count(r -> r.winding_number == d, res) == d. The reference
    # evaluates (x-10)^d as written; the oracle does the same through its program interpreter
    # (the expanded polynomial's residual is rounding noise near the 6-fold root)
    import math

    from hcgpu import slp

    (x,) = slp.variables(1)
    scale = max(float(math.comb(d, k)) * 10.0 ** (d - k) for k in range(d + 1))
    P = slp.Program([(x - 10.0) ** d], degrees=[d], scaling=[scale])
    for k in range(3):
        res, xs, _, _ = hco.track_slp(P, np.exp(2j * np.pi * (0.05 + k / 3)), hc.total_degree_start_solutions([d]))
        assert list(res["winding_number"]) == [d] * d
        assert (res["return_code"] == 1).all() and (res["singular"] == 1).all()
        assert np.abs(xs[:, 0] - 10).max() < 1e-6


def test_program_interpreter_matches_term_tables():
    # the oracle's straight-line-program evaluation (values, Jacobian, Taylor series) tracks the
    # structured systems to the endpoints its term-table evaluation of their expansions finds
    from hcgpu import slp

    for P, S in (slp.products_of_linear_forms(4, 3, 1), slp.determinantal(3, 3, 2), slp.disguised_ops(0)):
        P.scaling = [float(np.max(np.abs(c))) for c in S.coefficients]
        g = np.exp(2j * np.pi * 0.17)
        H = hc.total_degree_homotopy(S, g)
        starts = hc.total_degree_start_solutions(H.degrees)
        ro, xo, _, _ = track(H, starts)
        rp, xp, _, _ = hco.track_slp(P, g, starts)
        assert np.array_equal(ro["return_code"], rp["return_code"])
        ok = (ro["return_code"] == 1) & (ro["singular"] == 0)
        assert (np.abs(xp[ok] - xo[ok]).max(1) / np.abs(xo[ok]).max(1)).max() <= 1e-10
