"""Parameter homotopies, host side and oracle (no GPU): the affine-parameter system type, its
errors, and the oracle pinned to the reference's parameter-homotopy known answers
(test/tracker_test.jl: Tracker(ParameterHomotopy(F, [1, 0], [2, 4])), track from [1, 1])."""
import numpy as np
import pytest

import hcgpu as hc
from _kat import KAT, parametric_system
from _parity import oracle_track


def _kat():
    d = KAT["parameter_tracker"]
    return parametric_system(d), d


def test_fixing_parameters_matches_substitution():
    F, d = _kat()
    rng = np.random.default_rng(0)
    for _ in range(5):
        x = rng.normal(size=2) + 1j * rng.normal(size=2)
        p = rng.normal(size=2) + 1j * rng.normal(size=2)
        xp = np.concatenate([x, p])
        direct = [sum(complex(*c) * np.prod(xp ** np.array(e)) for e, c in zip(eq["exponents"], eq["coefficients"]))
                  for eq in d["equations"]]
        np.testing.assert_allclose(F(p).evaluate(x), direct, rtol=1e-14)
    # all fixings share one support
    assert all((a == b).all() for a, b in zip(F([1, 0]).exponents, F([2, 4]).exponents))


def test_parameter_homotopy_is_the_straight_line_form():
    F, d = _kat()
    p, q = np.array([1.0, 0.3j]), np.array([2.0 - 1j, 4.0])
    H = hc.ParameterHomotopy(F, p, q)
    x = np.array([0.3 + 0.1j, -0.7j])
    for t in (0.0, 0.25, 1.0):
        lhs = H.gamma * t * H.G.evaluate(x) + (1 - t) * H.F.evaluate(x)
        np.testing.assert_allclose(lhs, F(t * p + (1 - t) * q).evaluate(x), rtol=1e-14, atol=1e-15)


def test_non_affine_parameters_and_underdetermined_systems_are_rejected():
    x, y, a, b = hc.variables(4)
    with pytest.raises(NotImplementedError):
        hc.ParametricSystem.from_polys([x**2 - a * b, x * y - a], 2, 2)
    with pytest.raises(NotImplementedError):
        hc.ParametricSystem.from_polys([x**2 - a**2, x * y - a], 2, 2)
    G = parametric_system(KAT["parameter_solve"]["underdetermined"])
    with pytest.raises(hc.FiniteException) as e:
        hc.ParameterHomotopy(G, [1, 0], [2, 4])
    assert e.value.dim == KAT["parameter_solve"]["expect"]["finite_exception_dim"]


def test_oracle_parameter_tracker_kat():
    F, d = _kat()
    H = hc.ParameterHomotopy(F, d["start_parameters"], d["target_parameters"])
    s = np.array([d["start"]], dtype=np.complex128)
    r, x, _, _ = oracle_track(H, s, endgame=False)
    assert hc.TRACKER_CODES[int(r["return_code"][0])] == "success"
    assert int(r["accepted_steps"][0] + r["rejected_steps"][0]) <= d["expect"]["max_steps"]
    np.testing.assert_allclose(x[0], d["expect"]["solution"], rtol=1e-12)
    # and back from t = 0 to t = 1
    rb, xb, _, _ = oracle_track(H, x, endgame=False, t1=0.0, t0=1.0)
    assert hc.TRACKER_CODES[int(rb["return_code"][0])] == "success"
    np.testing.assert_allclose(xb[0], d["start"], rtol=1e-12)


def test_oracle_parameter_endgame_kat():
    F, d = _kat()
    H = hc.ParameterHomotopy(F, d["start_parameters"], d["target_parameters"])
    r, x, _, _ = oracle_track(H, np.array([d["start"]], dtype=np.complex128))
    assert hc.ENDGAME_CODES[int(r["return_code"][0])] == "success"
    np.testing.assert_allclose(x[0], d["expect"]["solution"], rtol=1e-12)
