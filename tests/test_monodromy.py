"""GPU monodromy: loops in the coefficient space of 3 dense quadrics (8 solutions) find the
same solution set as the total-degree solve at the base parameters."""
import numpy as np
import pytest

import hcgpu as hc

pytestmark = pytest.mark.gpu


def test_monodromy_finds_all_solutions():
    F0, _ = hc.dense_random_system(3, 2, seed=7)
    Fp = hc.ParametricSystem.coefficient_parameters(F0)
    R = hc.monodromy_solve(Fp, seed=3, target_solutions_count=8, max_loops_no_progress=20)
    assert R.is_success() and R.nsolutions() == 8
    assert R.tracked_paths > 0 and R.rounds >= 1
    # every solution solves the base system, and the set equals the total-degree solve's
    Fb = Fp(R.parameters)
    for x in R.solutions:
        assert np.abs(Fb.evaluate(x)).max() < 1e-9 * max(1, np.abs(x).max()) ** 2
    T = hc.solve(Fb, gamma=np.exp(0.7j))
    td = T.solutions()
    assert len(td) == 8
    for x in R.solutions:
        d = min(np.abs(x - y).max() / max(np.abs(y).max(), 1.0) for y in td)
        assert d < 1e-8


def test_monodromy_heuristic_stop_without_target():
    F0, _ = hc.dense_random_system(2, 2, seed=2)
    Fp = hc.ParametricSystem.coefficient_parameters(F0)
    R = hc.monodromy_solve(Fp, seed=4, max_loops_no_progress=6)
    assert R.is_heuristic_stop()
    assert R.nsolutions() == 4
