"""GPU certification (hc_certify through the C ABI): the reference's known answers
(test/certification_test.jl "Simple 1"), agreement with the exact rational oracle on every
candidate, larger systems, and rejection of non-solutions."""
import numpy as np
import pytest

import certify_oracle as CO
import hcgpu as hc
from _kat import KAT, jacobian, system, term_lists

pytestmark = pytest.mark.gpu


def _solve_kat():
    F = system("certification_simple")
    R = hc.solve(F, gamma=np.exp(0.31j))
    return F, R


def test_certify_reference_example():
    F, R = _solve_kat()
    e = KAT["certification_simple"]["expect"]
    assert hc.nnonsingular(R) == e["nnonsingular"]
    C = hc.certify(F, R)
    assert C.ncertified() == e["ncertified"]
    assert C.ndistinct_certified() == e["ndistinct_certified"]
    assert C.nreal_certified() == e["nreal_certified"]
    assert C.ncomplex_certified() == e["ncomplex_certified"]
    assert C.ndistinct_real_certified() == e["nreal_certified"]
    assert C.ndistinct_complex_certified() == e["ncomplex_certified"]
    # the same solutions twice: twice the certificates, the same distinct solutions
    S = [r.solution for r in R.path_results if r.is_success()]
    D = hc.certify(F, S + S)
    d = e["doubled"]
    assert D.ncertified() == d["ncertified"] and D.ndistinct_certified() == d["ndistinct_certified"]
    assert D.nreal_certified() == d["nreal_certified"]
    assert D.ndistinct_real_certified() == d["ndistinct_real_certified"]


def test_certificates_agree_with_the_exact_oracle():
    """Every GPU certificate is confirmed by the exact rational Krawczyk test on the same box,
    and the realness verdicts agree."""
    F, R = _solve_kat()
    C = hc.certify(F, R)
    terms = term_lists(F)
    for c in C.certificates:
        assert c.certified
        Y = np.linalg.inv(jacobian(F, c.center))
        ok, realness = CO.krawczyk(terms, c.center, c.radius / np.sqrt(2), Y, True)
        assert ok
        assert realness == (1 if c.real else 2 if c.complex else 0)
        # the certified solution lies within the enclosure of the refined centre
        assert np.abs(c.enclosure_center - c.center).max() <= c.radius


def test_certify_dense_quadrics_and_reject_non_solutions():
    F, g = hc.dense_random_system(6, 2, seed=1)
    R = hc.solve(F, gamma=g)
    C = hc.certify(F, R)
    assert C.ncertified() == hc.nnonsingular(R) == 64
    assert C.ndistinct_certified() == 64
    assert C.nreal_certified() == 0  # complex coefficients: realness is not claimed
    rng = np.random.default_rng(0)
    bogus = [rng.normal(size=6) + 1j * rng.normal(size=6) for _ in range(16)]
    B = hc.certify(F, bogus)
    assert B.ncertified() == 0
