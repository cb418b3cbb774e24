"""GPU (libhcgpu.so, through the C ABI) versus the CPU oracle on the same homotopies, γ and
start solutions. Bar: identical return codes / counts, and every path that is nonsingular in
both within 1e-10 relative (‖Δx‖∞/‖x‖∞) of the oracle's endpoint."""
import numpy as np
import pytest

import hcgpu as hc
from _parity import REL_TOL, compare_endgame, counts, oracle_track, rel_err

pytestmark = pytest.mark.gpu


def quadrics_2x2():
    x, y = hc.variables(2)
    return hc.System.from_polys([2.3 * x**2 + 1.2 * y**2 + 3 * x - 2 * y + 3,
                                 2.3 * x**2 + 1.2 * y**2 + 5 * x + 2 * y - 5])


def test_quadrics_2x2_fixed_gamma():
    # reference test/endgame_tracker_test.jl:2-31 (γ = 0.4 + 1.3i)
    H = hc.total_degree_homotopy(quadrics_2x2(), 0.4 + 1.3j)
    S = hc.total_degree_start_solutions(H.degrees)
    (ro, xo, vo), (rg, xg, vg), err = compare_endgame(H, S)
    assert list(rg["return_code"]) == list(ro["return_code"]) == [1, 1, 2, 2]
    assert err.max() <= REL_TOL
    assert (rg["accuracy"][:2] < 1e-12).all() and (rg["residual"][:2] < 1e-12).all()
    assert (rg["rejected_steps"][:2] == 0).all() and (rg["accepted_steps"][:2] < 20).all()
    assert rg["cond"][1] < 1e3
    np.testing.assert_allclose(vg[2], [-1, -1], rtol=1e-3)
    np.testing.assert_allclose(vg[3], [-1, -1], rtol=1e-3)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_dense_quadrics_6x6(precision):
    # 6 dense quadrics in 6 variables (all 28 monomials), 64 paths
    F, g = hc.dense_random_system(6, 2, seed=1)
    H = hc.total_degree_homotopy(F, g)
    S = hc.total_degree_start_solutions(H.degrees)
    (ro, xo, _), (rg, xg, _), err = compare_endgame(H, S, precision=precision)
    assert counts(rg) == counts(ro)
    assert len(err) == counts(ro)["nonsingular"]
    assert err.max() <= REL_TOL


@pytest.mark.parametrize("seed", [3, 4])
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_dense_cubics_small(seed, precision):
    F, g = hc.dense_random_system(3, 3, seed=seed)
    H = hc.total_degree_homotopy(F, g)
    S = hc.total_degree_start_solutions(H.degrees)
    (ro, _, _), (rg, _, _), err = compare_endgame(H, S, precision=precision)
    assert counts(rg) == counts(ro)
    assert err.max() <= REL_TOL


@pytest.mark.parametrize("d", [2, 4])
def test_winding_number_family(d):
    # reference test/endgame_test.jl:62-69: d + 1 successes
    a = [0.257, -0.139, -1.73, -0.199, 1.79, -1.32]
    x, y = hc.variables(2)
    f1 = (a[0] * x**d + a[1] * y) * (a[2] * x + a[3] * y) + 1
    f2 = (a[0] * x**d + a[1] * y) * (a[4] * x + a[5] * y) + 1
    H = hc.total_degree_homotopy(hc.System.from_polys([f1, f2]), np.exp(2j * np.pi * 0.37))
    S = hc.total_degree_start_solutions(H.degrees)
    (ro, _, _), (rg, _, _), err = compare_endgame(H, S)
    assert (rg["return_code"] == 1).sum() == d + 1
    assert list(rg["return_code"]) == list(ro["return_code"])
    assert err.max() <= REL_TOL


def test_univariate_double_root():
    # reference test/endgame_tracker_test.jl:32-45: (x-10)^2 has winding number 2, singular
    (x,) = hc.variables(1)
    H = hc.total_degree_homotopy(hc.System.from_polys([(x - 10) ** 2]), np.exp(2j * np.pi * 0.3))
    S = hc.total_degree_start_solutions(H.degrees)
    ro, xo, _, _ = oracle_track(H, S)
    T = hc.EndgameTracker(H)
    prs = T.track_batch(S)
    assert [p.winding_number for p in prs] == [2, 2]
    assert all(p.is_singular() and p.is_real() for p in prs)
    assert all(0 < p.last_path_point[1] < 0.1 for p in prs)
    assert list(ro["winding_number"]) == [2, 2]
    for p in prs:
        assert abs(p.solution[0] - 10) < 1e-6


def test_plain_tracker_valuation():
    # reference test/valuation_test.jl:20-44 (Example 2): track S[3] to t = 1e-10 with
    # conservative parameters; valuation ≈ -1 for both coordinates
    H = hc.total_degree_homotopy(quadrics_2x2(), 0.4 + 1.3j)
    S = hc.total_degree_start_solutions(H.degrees)
    to = hc.TrackerOptions(parameters="conservative")
    T = hc.Tracker(H, to)
    tf = 1e-10
    rg, xg, vg, lg = T.track_arrays(S[2:3], t1=1.0, t0=tf)
    assert rg["return_code"][0] == 1
    np.testing.assert_allclose(vg[0], [-1, -1], atol=10 * tf ** 0.5)
    np.testing.assert_allclose(lg[0].real, [-1, -1], atol=tf ** 0.5)
    import hco

    o = hco.default_options(beta_omega_p=4.0, beta_tau=0.25, strict_beta_tau=0.1875)
    ro, xo, vo, lo = oracle_track(H, S[2:3], endgame=False, t1=1.0, t0=tf, options=o)
    assert ro["return_code"][0] == 1
    assert rel_err(xg, xo).max() <= 1e-8


def test_api_result_counts():
    F, g = hc.dense_random_system(4, 2, seed=7)
    res = hc.solve(F, gamma=g)
    assert len(res) == 16
    assert hc.nnonsingular(res) + hc.nsingular(res, counting_multiplicities=True) + hc.nat_infinity(res) + hc.nfailed(res) == 16
    assert hc.nnonsingular(res) == 16
