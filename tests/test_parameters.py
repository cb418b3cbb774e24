"""GPU tests of parameter homotopies (through the C ABI): the reference's known answers,
GPU-vs-oracle parity, and the many-parameter solver in one batched launch."""
import numpy as np
import pytest

import hcgpu as hc
from _kat import KAT, parametric_system
from _parity import REL_TOL, counts, oracle_track, rel_err

pytestmark = pytest.mark.gpu


def _kat():
    d = KAT["parameter_tracker"]
    return parametric_system(d), d


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_parameter_tracker_kat(precision):
    # test/tracker_test.jl: success within 5 steps at [√2, -√2], and back to the start
    F, d = _kat()
    H = hc.ParameterHomotopy(F, d["start_parameters"], d["target_parameters"])
    T = hc.Tracker(H, hc.TrackerOptions(precision=precision))
    r = T.track(np.array(d["start"], dtype=np.complex128), 1.0, 0.0)
    assert r.return_code == "success"
    assert r.accepted_steps + r.rejected_steps <= d["expect"]["max_steps"]
    np.testing.assert_allclose(r.solution, d["expect"]["solution"], rtol=1e-12)
    rb = T.track(r.solution, 0.0, 1.0)
    assert rb.return_code == "success"
    np.testing.assert_allclose(rb.solution, d["start"], rtol=1e-12)


def test_parameter_solve_kat():
    # test/solve_test.jl "solve (parameter homotopy)": nsolutions == 1
    F, d = _kat()
    R = hc.solve(F, [d["start"]], start_parameters=d["start_parameters"],
                 target_parameters=d["target_parameters"])
    assert R.nsolutions() == KAT["parameter_solve"]["expect"]["nsolutions"]
    np.testing.assert_allclose(R.solutions()[0], d["expect"]["solution"], rtol=1e-12)


def _circle_line():
    # f = x² + y² − 1, l = a x + b y + c with parameters (a, b, c) (test/solve_test.jl, "Many parameters")
    x, y, a, b, c = hc.variables(5)
    return hc.ParametricSystem.from_polys([x**2 + y**2 - 1, a * x + b * y + c], 2, 3)


def _generic_start(F, seed):
    rng = np.random.default_rng(seed)
    p0 = rng.normal(size=3) + 1j * rng.normal(size=3)
    R0 = hc.solve(F(p0), gamma=np.exp(2j * np.pi * rng.random()))
    S0 = np.array(R0.solutions())
    assert S0.shape == (2, 2)
    return p0, S0


def test_many_parameter_solver_in_one_launch():
    F = _circle_line()
    p0, S0 = _generic_start(F, 1)
    rng = np.random.default_rng(2)
    params = [rng.random(3) for _ in range(100)]
    out = hc.solve(F, S0, start_parameters=p0, target_parameters=params)
    assert len(out) == 100 and all(isinstance(R, hc.Result) and q is p for (R, q), p in zip(out, params))
    assert all(R.nsolutions() == 2 for R, _ in out)
    # every endpoint solves its target system, and matches a single-target run bit for bit
    for (R, q) in out[:10]:
        for s in R.solutions():
            assert np.abs(F(q).evaluate(s)).max() < 1e-12
    R1 = hc.solve(F, S0, start_parameters=p0, target_parameters=params[3])
    np.testing.assert_array_equal(np.array(R1.solutions()), np.array(out[3][0].solutions()))
    # GPU vs oracle on a few targets
    for q in params[:5]:
        H = hc.ParameterHomotopy(F, p0, q)
        ro, xo, _, _ = oracle_track(H, S0)
        rg, xg, _, _ = hc.EndgameTracker(H).track_arrays(S0)
        assert counts(rg) == counts(ro)
        assert rel_err(xg, xo).max() <= REL_TOL


def test_many_parameter_transforms():
    F = _circle_line()
    p0, S0 = _generic_start(F, 3)
    rng = np.random.default_rng(4)
    params = [rng.random(3) for _ in range(20)]
    real = lambda R, q: [np.real(s) for s in R.solutions() if np.abs(np.imag(s)).max() < 1e-8]
    flat = hc.solve(F, S0, start_parameters=p0, target_parameters=params, transform_result=real, flatten=True)
    nested = hc.solve(F, S0, start_parameters=p0, target_parameters=params, transform_result=real)
    assert len(flat) == sum(len(r) for r in nested) > 0
    for v in flat:
        assert v.shape == (2,) and abs(v[0] ** 2 + v[1] ** 2 - 1) < 1e-10
    idx = hc.solve(F, S0, start_parameters=p0, target_parameters=range(5),
                   transform_parameters=lambda k: params[k], transform_result=lambda R, k: (R.nsolutions(), k))
    assert idx == [(2, k) for k in range(5)]
