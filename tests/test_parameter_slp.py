"""Parameter homotopies of straight-line programs on the GPU (hc_set_slp_parameter_homotopy):
H(x, t) = F(x; t p + (1 - t) q) (src/homotopies/parameter_homotopy.jl:3-44) with parameters that
enter F non-affinely, against the oracle's restatement of the same homotopy.

Bar: identical return codes per path and nonsingular endpoints within 1e-10 relative of the
oracle's, in FP64 and mixed precision; new (p, q) on a tracker (hc_set_slp_parameters) give the
results of a fresh tracker bit for bit; on an affine family the program and the term-table
route (which tracks t F(x; p) + (1 - t) F(x; q), the same function) agree within 1e-10."""
import numpy as np
import pytest

import hcgpu as hc
from _parity import REL_TOL, oracle_track, rel_err
from hcgpu import slp
from hcgpu.systems import variables as poly_variables

pytestmark = pytest.mark.gpu


def _family():
    """n = 3, F(x; a, b, c) with squares, cubes and products of the parameters."""
    (x, y, z), (a, b, c) = slp.variables_and_parameters(3, 3)
    return slp.Program([x * x + a * a * y - b ** 3 + c * z,
                        y * z - a * b * x + (c - 1.0) ** 2,
                        z * z * x - (a + b * c) * y + 0.5])


def _start(P, p, seed):
    import hco

    F = P.fixed(p)
    rng = np.random.default_rng(seed)
    g = complex(np.exp(2j * np.pi * rng.random()))
    res, x, _, _ = hco.track_slp(F, g, hc.total_degree_start_solutions(F.degrees))
    ok = (res["return_code"] == 1) & (res["singular"] == 0)
    return x[ok]


def _params(seed):
    rng = np.random.default_rng(seed)
    return [rng.normal(size=3) + 1j * rng.normal(size=3) for _ in range(3)]


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_gpu_parameter_homotopy_matches_oracle(precision):
    import hco

    P = _family()
    p0, p1, _ = _params(3)
    S0 = _start(P, p0, 1)
    assert S0.shape[0] == 7  # the family's generic root count (Bézout 12)
    ro, xo, _, _ = hco.track_slp_parameter(P, p0, p1, S0)
    T = hc.EndgameTracker(hc.parameter_homotopy(P, p0, p1), hc.TrackerOptions(precision=precision))
    rg, xg, _, _ = T.track_arrays(S0)
    assert list(rg["return_code"]) == list(ro["return_code"])
    ok = (ro["return_code"] == 1) & (ro["singular"] == 0)
    assert ok.sum() == S0.shape[0]
    assert rel_err(xg[ok], xo[ok]).max() <= REL_TOL
    for xi in xg[ok]:
        assert np.abs(P.evaluate(xi, p1)).max() <= 1e-9 * max(1.0, np.abs(xi).max() ** 3)


def test_new_parameters_need_no_new_tracker():
    P = _family()
    p0, p1, p2 = _params(4)
    S0 = _start(P, p0, 2)
    H = hc.parameter_homotopy(P, p0, p1)
    T = hc.EndgameTracker(H)
    r1, x1, _, _ = T.track_arrays(S0)
    T.set_homotopy(H.parameters(p0, p2))  # two small device arrays, no compilation
    r2, x2, _, _ = T.track_arrays(S0)
    rf, xf, _, _ = hc.EndgameTracker(hc.parameter_homotopy(P, p0, p2)).track_arrays(S0)
    assert np.array_equal(r2["return_code"], rf["return_code"]) and np.array_equal(x2, xf)
    assert not np.allclose(x1, x2)
    # the many-parameter solver on a program: one tracker retargeted per target
    out = hc.parameters.solve(P, S0, p0, [p1, p2])
    for (R, q), xs in zip(out, (x1, x2)):
        got = np.array([r.solution for r in R.path_results])
        assert np.array_equal(got, xs)


def test_affine_family_program_equals_term_tables():
    """x₁² + a x₂ - b, x₁ x₂ - c x₁ + 1 - b: affine in (a, b, c), so the term-table route and the
    program route track the same homotopy."""
    V = poly_variables(5)
    polys = [V[0] * V[0] + V[2] * V[1] - V[3], V[0] * V[1] - V[4] * V[0] + 1.0 - V[3]]
    Fa = hc.parametric_system(polys, 2, 3)
    assert isinstance(Fa, hc.ParametricSystem)
    (x1, x2), (a, b, c) = slp.variables_and_parameters(2, 3)
    Pp = slp.Program([x1 * x1 + a * x2 - b, x1 * x2 - c * x1 + 1.0 - b])
    p0, p1, _ = _params(5)
    S0 = _start(Pp, p0, 3)
    assert S0.shape[0] == 3  # x₂ = (b - x₁²)/a leaves a cubic in x₁
    rt, xt, _, _ = hc.EndgameTracker(hc.parameter_homotopy(Fa, p0, p1)).track_arrays(S0)
    rp, xp, _, _ = hc.EndgameTracker(hc.parameter_homotopy(Pp, p0, p1)).track_arrays(S0)
    assert list(rt["return_code"]) == list(rp["return_code"]) == [1] * 3
    assert rel_err(xp, xt).max() <= REL_TOL
    # and the oracle's term-table form agrees
    H = hc.parameter_homotopy(Fa, p0, p1)
    ro, xo, _, _ = oracle_track(H, S0)
    assert rel_err(xp, xo).max() <= REL_TOL
