"""The CUDA tracker (libhcgpu.so, through the C ABI) on the reference's own known-answer
systems and on samples of the benchmark configurations, against the CPU oracle.

Bar, for every case: the return code of every path equals the oracle's, and every path that
is nonsingular in both ends within 1e-10 relative (‖Δx‖∞/‖x‖∞) of the oracle's endpoint. The
KAT counts themselves (693, 924, winding numbers, multiplicities) are asserted as the
reference's tests assert them. Learned step control takes other steps than the oracle's plain
rule; its bar is the same per-path codes and endpoints.
"""
import numpy as np
import pytest

import hcgpu as hc
from _kat import KAT, gamma, system
from _parity import REL_TOL, counts, oracle_track, rel_err

pytestmark = pytest.mark.gpu

MODES = [("fp64", "plain"), ("mixed", "plain"), ("fp64", "learned"), ("mixed", "learned")]


def gpu_track(H, S, precision, step_control, endgame_options=None):
    to = hc.TrackerOptions(precision=precision, step_control=step_control)
    T = hc.EndgameTracker(H, to, endgame_options)
    out = T.track_arrays(S)
    return out, T.stats()


def assert_parity(ro, xo, rg, xg, tol=REL_TOL):
    bad = np.nonzero(ro["return_code"] != rg["return_code"])[0]
    assert bad.size == 0, (bad[:10], ro["return_code"][bad[:10]], rg["return_code"][bad[:10]])
    assert np.array_equal(ro["singular"], rg["singular"])
    both = (ro["return_code"] == 1) & (ro["singular"] == 0)
    if both.any():
        err = rel_err(xg[both], xo[both])
        assert err.max() <= tol, err.max()


_oracle_cache = {}


def oracle(key, H, S, **kw):
    if key not in _oracle_cache:
        _oracle_cache[key] = oracle_track(H, S, **kw)
    return _oracle_cache[key]


@pytest.mark.parametrize("precision,step_control", MODES)
def test_mohab_fixed_gamma(precision, step_control):
    # test/endgame_test.jl:76-107: 693 nonsingular with the γ that once made paths jump
    H = hc.total_degree_homotopy(system("mohab"), gamma("mohab"))
    S = hc.total_degree_start_solutions(H.degrees)
    ro, xo, _, _ = oracle("mohab", H, S)
    (rg, xg, _, _), st = gpu_track(H, S, precision, step_control)
    want = KAT["mohab"]["expect"]["nnonsingular"]
    assert counts(ro)["nonsingular"] == want
    assert counts(rg)["nonsingular"] == want
    assert counts(rg) == counts(ro)
    assert_parity(ro, xo, rg, xg)


@pytest.mark.parametrize("precision,step_control", MODES)
def test_cyclic7_total_degree(precision, step_control):
    # test/endgame_test.jl:2-5: 924 solutions
    H = hc.total_degree_homotopy(hc.cyclic(7), np.exp(2j * np.pi * 0.31))
    S = hc.total_degree_start_solutions(H.degrees)
    ro, xo, _, _ = oracle("cyclic7", H, S)
    (rg, xg, _, _), _ = gpu_track(H, S, precision, step_control)
    assert counts(rg)["nonsingular"] == KAT["cyclic7"]["expect"]["nsolutions"]
    assert counts(rg) == counts(ro)
    assert_parity(ro, xo, rg, xg)


@pytest.mark.parametrize("precision,step_control", MODES)
def test_dynamic_polynomials_18(precision, step_control):
    # test/solve_test.jl:338-344: 18 solutions of (x⁴ + y⁴ − 1)(x² + y² − 2) + x⁵y,
    # x² + 2xy² − 2y² − 1/2 by total degree (every one of the 18 paths)
    H = hc.total_degree_homotopy(system("dynamic_polynomials_18"), np.exp(2j * np.pi * 0.13))
    S = hc.total_degree_start_solutions(H.degrees)
    ro, xo, _, _ = oracle("dynamic_polynomials_18", H, S)
    (rg, xg, _, _), _ = gpu_track(H, S, precision, step_control)
    assert counts(rg)["nonsingular"] == KAT["dynamic_polynomials_18"]["expect"]["nsolutions"] == 18
    assert counts(rg) == counts(ro)
    assert_parity(ro, xo, rg, xg)


@pytest.mark.parametrize("precision,step_control", MODES)
def test_beyond_polyhedral_example(precision, step_control):
    # test/endgame_test.jl:54-60: the 2×2 quadrics by total degree: 2 successes, 2 at infinity
    e = KAT["beyond_polyhedral"]["expect"]
    for k in range(3):
        H = hc.total_degree_homotopy(system("beyond_polyhedral"), np.exp(2j * np.pi * (0.07 + k / 3)))
        S = hc.total_degree_start_solutions(H.degrees)
        ro, xo, _, _ = oracle_track(H, S)
        (rg, xg, _, _), _ = gpu_track(H, S, precision, step_control)
        codes = [hc.ENDGAME_CODES[int(c)] for c in rg["return_code"]]
        assert codes.count("success") == e["success"] and codes.count("at_infinity") == e["at_infinity"]
        assert_parity(ro, xo, rg, xg)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_straight_line_tracker(precision):
    # test/tracker_test.jl:93-105: Tracker on t G + (1 - t) F from G's roots succeeds; from
    # [100, -100] the start value is invalid (plain tracker, t from 1 to 0)
    from _kat import straight_line_homotopy

    d = KAT["straight_line_tracker"]
    H = straight_line_homotopy()
    S = np.array(d["starts"] + [d["invalid_start"]], dtype=np.complex128)
    ro, xo, _, _ = oracle_track(H, S, endgame=False)
    rg, xg, _, _ = hc.Tracker(H, hc.TrackerOptions(precision=precision)).track_arrays(S, t1=1.0, t0=0.0)
    assert [hc.TRACKER_CODES[int(c)] for c in rg["return_code"]] == ["success", "success",
                                                                     "terminated_invalid_startvalue"]
    assert list(rg["return_code"]) == list(ro["return_code"])
    assert rel_err(xg[:2], xo[:2]).max() <= REL_TOL


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_wilkinson_12(precision):
    # test/endgame_test.jl:38-45: roots 1..12 (only_nonsingular endgame), tiny imaginary parts.
    # The expanded polynomial's roots 5..11 have relative condition numbers of 1e8..1e9, so an
    # FP64 residual fixes them only to ~1e-8; whether the final double-double refinement runs
    # depends on a noise-level accuracy estimate. Both trackers are therefore held to the
    # exact roots (integers) rather than to each other at 1e-10.
    (x,) = hc.variables(1)
    p = hc.Poly.const(1.0, 1)
    for i in range(1, 13):
        p = p * (x - i)
    H = hc.total_degree_homotopy(hc.System.from_polys([p]), np.exp(2j * np.pi * 0.21))
    S = hc.total_degree_start_solutions(H.degrees)
    eo = hc.EndgameOptions(only_nonsingular=True)
    import hco

    ro, xo, _, _ = oracle_track(H, S, options=hco.default_options(only_nonsingular=1))
    (rg, xg, _, _), _ = gpu_track(H, S, precision, "plain", eo)
    assert list(rg["return_code"]) == list(ro["return_code"]) == [1] * 12
    assert np.round(np.sort(xg[:, 0].real)).astype(int).tolist() == list(range(1, 13))
    assert np.abs(xg[:, 0].imag).max() < 1e-4
    for xs in (xg[:, 0], xo[:, 0]):
        exact = np.round(xs.real)
        assert (np.abs(xs - exact) / exact).max() <= 1e-8


@pytest.mark.parametrize("k", range(3))
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_hyperbolic_6_6_multiplicity(k, precision):
    # test/endgame_test.jl:7-22: 12 paths of winding number 3 end at 2 singular solutions of
    # multiplicity 6 (the reference dehomogenises nothing: y = 1 there)
    e = KAT["hyperbolic_6_6"]["expect"]
    F = system("hyperbolic_6_6")
    g = np.exp(2j * np.pi * (0.1 + k / 3))
    H = hc.total_degree_homotopy(F, g)
    S = hc.total_degree_start_solutions(H.degrees)
    ro, xo, _, _ = oracle_track(H, S)
    (rg, xg, _, _), _ = gpu_track(H, S, precision, "plain")
    assert_parity(ro, xo, rg, xg)
    assert list(rg["winding_number"]) == list(ro["winding_number"])
    R = hc.solve(F, gamma=g, precision=precision)
    prs = R.path_results
    assert sum(1 for r in prs if r.winding_number == e["winding_number"]) == e["n_winding"]
    assert R.nresults() == e["nresults"]
    assert hc.nsingular(R) == e["nsingular"]
    assert all(r.multiplicity == e["multiplicity"] for r in prs if r.is_success() and not R.is_multiple_result(r))


@pytest.mark.parametrize("k", range(3))
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_singular_1_multiplicity(k, precision):
    # test/endgame_test.jl:24-36: one singular solution of multiplicity 3 and one nonsingular
    e = KAT["singular_1"]["expect"]
    F = system("singular_1")
    g = np.exp(2j * np.pi * (0.1 + k / 3))
    H = hc.total_degree_homotopy(F, g)
    S = hc.total_degree_start_solutions(H.degrees)
    ro, xo, _, _ = oracle_track(H, S)
    (rg, xg, _, _), _ = gpu_track(H, S, precision, "plain")
    assert_parity(ro, xo, rg, xg)
    R = hc.solve(F, gamma=g, precision=precision)
    assert hc.nsingular(R) == e["nsingular"]
    assert R.nresults(only_nonsingular=True) == e["nresults_nonsingular"]
    sing = [r for r in R.path_results if r.is_singular()]
    assert len(sing) == 3 and all(r.multiplicity == 3 for r in sing)


def test_dense_cubics_10x10_sample_mixed_learned():
    """The benchmark's homotopy (10 dense cubics in 10 variables, seed 0, 59,049 paths): 4,096
    evenly spaced paths in mixed precision with learned steps, against the FP64 oracle."""
    F, g = hc.dense_random_system(10, 3, seed=0)
    H = hc.total_degree_homotopy(F, g)
    S = hc.total_degree_start_solutions(H.degrees)
    idx = np.linspace(0, len(S) - 1, 4096).astype(np.int64)
    ro, xo, _, _ = oracle_track(H, S[idx])
    (rg, xg, _, _), st = gpu_track(H, S[idx], "mixed", "learned")
    assert counts(rg) == counts(ro)
    assert_parity(ro, xo, rg, xg)
    assert st["learned_proposals"] > 0
    assert st["evals_dd"] > 0  # near-singular steps ran the double-double residual


@pytest.mark.parametrize("precision,step_control", [("fp64", "plain"), ("mixed", "learned")])
def test_uneven_batch_n6_to_8_against_oracle(precision, step_control):
    """Instances with 6 ≤ n ≤ 8 of the 2,000-instance uneven workload (seed 0), tracked in one
    batched launch: per-path codes and endpoints against the oracle, instance by instance."""
    inst = [(F, g) for F, g in hc.uneven_instances(2000, 0) if 6 <= F.n <= 8]
    # one instance per n, the smallest Bézout number of that n (keeps the oracle in seconds)
    pick = {}
    for F, g in inst:
        b = int(np.prod([max(int(e.sum(axis=1).max()), 1) for e in F.exponents]))
        if F.n not in pick or b < pick[F.n][0]:
            pick[F.n] = (b, F, g)
    Hs = [hc.total_degree_homotopy(F, g) for _, F, g in (pick[n] for n in sorted(pick))]
    assert [H.n for H in Hs] == [6, 7, 8]
    B = hc.BatchTracker(Hs, hc.TrackerOptions(precision=precision, step_control=step_control))
    res, sol = B.track_arrays()
    for i, (r, x) in enumerate(B.split(res, sol)):
        S = hc.total_degree_start_solutions(Hs[i].degrees)
        ro, xo, _, _ = oracle_track(Hs[i], S)
        assert counts(r) == counts(ro)
        assert_parity(ro, xo, r, x)
