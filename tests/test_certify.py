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
    # random points: the double-word pass refines with Newton before certifying (as the
    # reference does, up to 8 iterations, src/certification.jl:1040-1056), so a point whose
    # iteration reaches a solution gets that solution's certificate; every certificate issued
    # is confirmed by the exact oracle, and the points that reach none are rejected
    rng = np.random.default_rng(0)
    bogus = [rng.normal(size=6) + 1j * rng.normal(size=6) for _ in range(16)]
    B = hc.certify(F, bogus)
    assert B.ncertified() < 16
    terms = term_lists(F)
    for c in B.certificates:
        if c.certified:
            assert c.precision == 106
            Y = np.linalg.inv(jacobian(F, c.center))
            assert CO.krawczyk(terms, c.center, c.radius / np.sqrt(2), Y, False)[0]


def test_ill_conditioned_roots_need_the_double_word_pass():
    """Wilkinson's polynomial ∏_{i=1..16} (x − i), expanded in FP64: in the middle the terms reach
    1e22 against |p'| ~ 1e11, so the FP64 residual's rounding radius forces boxes wider than the
    ball enclosure of p' allows (it grows like Σ k²|c_k||x|^(k-2) r): FP64 centres certify only
    the outer roots. The double-word pass (the reference's Arb step,
    src/certification.jl:1120-1200, here ~106 bits) certifies every root of the FP64 polynomial.
    (At degree 20 the middle roots need more than 106 bits; the reference goes on to 192 and 256,
    this library stops at double-word centres and leaves them uncertified.) Every certificate
    is confirmed by the exact rational Krawczyk test on the reported box."""
    N = 16
    (x,) = hc.variables(1)
    p = hc.Poly.const(1.0, 1)
    for i in range(1, N + 1):
        p = p * (x - i)
    F = hc.System.from_polys([p])
    e, c = F.exponents[0][:, 0], F.coefficients[0]
    dense = np.zeros(N + 1, dtype=np.complex128)
    dense[N - e] = c
    cands = [[complex(r)] for r in np.roots(dense)]  # accurate to ~1e-3 in the middle
    C = hc.certify(F, cands)
    assert C.ncertified() == N and C.ndistinct_certified() == N
    precs = [cc.precision for cc in C.certificates]
    assert 53 in precs and precs.count(106) >= N // 2, precs
    assert C.nreal_certified() == N  # real coefficients, real roots
    terms = term_lists(F)
    for cc in C.certificates:
        Y = np.linalg.inv(jacobian(F, cc.center))
        ok, realness = CO.krawczyk(terms, cc.center, cc.radius / np.sqrt(2), Y, True)
        assert ok and realness == 1, (cc.center, cc.radius, cc.precision)
        assert np.abs(cc.enclosure_center - cc.center).max() <= cc.radius
