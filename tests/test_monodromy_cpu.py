"""Monodromy host logic (no GPU): start pairs and distinct-point bookkeeping."""
import numpy as np

import hcgpu as hc
from hcgpu.monodromy import _UniquePoints


def test_find_start_pair_solves_the_family():
    F0, _ = hc.dense_random_system(3, 2, seed=5)
    Fp = hc.ParametricSystem.coefficient_parameters(F0)
    assert Fp.nparams == 30
    np.testing.assert_allclose(Fp(np.concatenate(F0.coefficients)).evaluate([0.3, 0.1j, -1]),
                               F0.evaluate([0.3, 0.1j, -1]), rtol=1e-14)
    x, p = hc.find_start_pair(Fp, seed=1)
    assert np.abs(Fp(p).evaluate(x)).max() < 1e-10


def test_unique_points():
    U = _UniquePoints(1e-8)
    rng = np.random.default_rng(0)
    pts = [rng.normal(size=3) + 1j * rng.normal(size=3) for _ in range(50)]
    assert all(U.add(p) for p in pts)
    assert not any(U.add(p * (1 + 1e-12)) for p in pts)
    assert len(U) == 50
