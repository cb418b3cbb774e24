"""GPU edge cases through the C ABI: the largest supported system size (n = 32), n = 1, empty
inputs, and a batch with an instance that has no paths."""
import numpy as np
import pytest

import hcgpu as hc
from _parity import REL_TOL, counts, oracle_track, rel_err
from hcgpu import _lib

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_largest_system_n32(precision):
    # f_i = x_i² + a_i x_{i+1} + b_i: leading forms x_i², no solutions at infinity, so every
    # one of the 2^32 total-degree paths ends at a finite nonsingular solution
    rng = np.random.default_rng(3)
    x = hc.variables(32)
    a = rng.normal(size=32) + 1j * rng.normal(size=32)
    b = rng.normal(size=32) + 1j * rng.normal(size=32)
    F = hc.System.from_polys([x[i] ** 2 + a[i] * x[(i + 1) % 32] + b[i] for i in range(32)])
    g = np.exp(0.9j)
    H = hc.total_degree_homotopy(F, g)
    S = hc.total_degree_start_solutions(H.degrees, np.arange(48))
    ro, xo, _, _ = oracle_track(H, S)
    T = hc.EndgameTracker(H, hc.TrackerOptions(precision=precision))
    rg, xg, _, _ = T.track_arrays(S)
    assert counts(rg) == counts(ro)
    both = (ro["return_code"] == 1) & (ro["singular"] == 0) & (rg["return_code"] == 1) & (rg["singular"] == 0)
    assert both.sum() == len(S)
    assert rel_err(xg[both], xo[both]).max() <= REL_TOL


def test_n33_is_rejected():
    x = hc.variables(33)
    F = hc.System.from_polys([xi**2 - 1 for xi in x])
    with pytest.raises(_lib.HCError, match="n <= 32"):
        hc.EndgameTracker(hc.total_degree_homotopy(F, 0.3 + 0.9j))


def test_univariate():
    (x,) = hc.variables(1)
    p = hc.Poly.const(1.0, 1)
    for r in (1, 2, 3, 4, 5):
        p = p * (x - r)
    F = hc.System.from_polys([p])
    R = hc.solve(F, gamma=np.exp(0.4j))
    sols = sorted(s[0].real for s in R.solutions())
    np.testing.assert_allclose(sols, [1, 2, 3, 4, 5], rtol=1e-12)
    H = hc.total_degree_homotopy(F, np.exp(0.4j))
    ro, xo, _, _ = oracle_track(H, hc.total_degree_start_solutions(H.degrees))
    rg, xg, _, _ = hc.EndgameTracker(H).track_arrays(hc.total_degree_start_solutions(H.degrees))
    assert (rg["return_code"] == ro["return_code"]).all()
    assert rel_err(xg, xo).max() <= REL_TOL


def test_empty_inputs():
    F, g = hc.dense_random_system(3, 2, seed=1)
    H = hc.total_degree_homotopy(F, g)
    T = hc.EndgameTracker(H)
    r, x, _, _ = T.track_arrays(np.zeros((0, 3), dtype=np.complex128))
    assert r.shape == (0,) and x.shape == (0, 3)
    # a batch where one instance has no paths
    G, h = hc.dense_random_system(2, 2, seed=2)
    Hs = [H, hc.total_degree_homotopy(G, h)]
    B = hc.BatchTracker(Hs, npaths=[0, 4])
    res, sol = B.track_arrays(hc.total_degree_start_solutions(Hs[1].degrees).reshape(-1))
    parts = B.split(res, sol)
    assert parts[0][0].shape == (0,) and parts[1][0].shape == (4,)
    r1, x1, _, _ = hc.EndgameTracker(Hs[1]).track_arrays(hc.total_degree_start_solutions(Hs[1].degrees))
    assert np.array_equal(parts[1][1], x1)
