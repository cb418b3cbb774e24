"""Certification oracle (exact rational Krawczyk test) pinned to the reference's certification
known answers (test/certification_test.jl "Simple 1": 18 nonsingular solutions, all certified,
4 real and 14 non-real), with the tracker oracle supplying the solutions."""
import numpy as np

import certify_oracle as CO
import hcgpu as hc
from _kat import KAT, jacobian, system, term_lists
from _parity import oracle_track


def _oracle_solutions():
    F = system("certification_simple")
    H = hc.total_degree_homotopy(F, np.exp(0.31j))
    S = hc.total_degree_start_solutions(H.degrees)
    r, x, _, _ = oracle_track(H, S)
    ok = (r["return_code"] == 1) & (r["singular"] == 0)
    return F, x[ok]


def test_oracle_certifies_the_reference_example():
    F, X = _oracle_solutions()
    e = KAT["certification_simple"]["expect"]
    assert len(X) == e["nnonsingular"]
    terms = term_lists(F)
    cert = real = nonreal = 0
    for x in X:
        Y = np.linalg.inv(jacobian(F, x))
        c, re = CO.krawczyk(terms, x, 1e-9 * max(1.0, np.abs(x).max()), Y, True)
        cert += c
        real += re == 1
        nonreal += re == 2
    assert (cert, real, nonreal) == (e["ncertified"], e["nreal_certified"], e["ncomplex_certified"])


def test_oracle_rejects_non_solutions():
    F, X = _oracle_solutions()
    terms = term_lists(F)
    for x in X[:4]:
        y = x + 1e-3
        Y = np.linalg.inv(jacobian(F, y))
        assert CO.krawczyk(terms, y, 1e-9, Y, True)[0] is False
