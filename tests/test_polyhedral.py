"""Polyhedral homotopy on the GPU (hc_set_toric / hc_track_toric, then the coefficient
homotopy): path counts of the reference's tests (test/polyhedral_test.jl,
test/solve_test.jl:94-124) and parity with the oracle's polyhedral tracker."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "homotopycontinuation.jl_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import hcgpu as hc  # noqa: E402
from hcgpu import polyhedral_homotopy as ph  # noqa: E402

pytestmark = pytest.mark.gpu

REL_TOL = 1e-10  # endpoint agreement with the oracle, ‖x_gpu − x_ref‖∞ / max(‖x_ref‖∞, 1)


def f_example():
    x, y = hc.variables(2)
    return hc.System.from_polys([2 * y + 3 * y ** 2 - x * y ** 3, x + 4 * x ** 2 - 2 * x ** 3 * y])


def sparse_system(seed):
    return hc.sparse_random_system(4, 5, 3, seed=seed)[0]


def _rel(a, b):
    return np.abs(a - b).max() / max(np.abs(b).max(), 1.0)


@pytest.mark.parametrize("torus,npaths,nsucc", [(False, 8, 6), (True, 3, 3)])
def test_polyhedral_counts_kat(torus, npaths, nsucc):
    # test/polyhedral_test.jl:2-21
    T, S = ph.polyhedral(f_example(), only_torus=torus, seed=1)
    assert len(S) == npaths
    rs = T.track_arrays(S)
    assert sum(r.is_success() for r in rs) == nsucc


def test_cyclic5_kat():
    # test/polyhedral_test.jl:38-42
    F = hc.cyclic(5)
    T, S = ph.polyhedral(F, seed=2)
    rs = T.track_arrays(S)
    assert sum(r.is_success() for r in rs) == 70
    for r in rs:
        assert np.abs(F.evaluate(r.solution)).max() < 1e-10


def test_cyclic7_kat():
    # test/polyhedral_test.jl:43-46: 924 solutions of cyclic-7
    F = hc.cyclic(7)
    T, S = ph.polyhedral(F, seed=6)
    assert len(S) == 924
    rs = T.track_arrays(S)
    assert sum(r.is_success() for r in rs) == 924


def test_univariate_and_zero_solutions():
    x, = hc.variables(1)
    F = hc.System.from_polys([x ** 5 - 3 * x ** 2 + 1])
    R = hc.solve(F, start_system="polyhedral", seed=1)
    assert R.nsolutions() == 5
    roots = np.roots([1, 0, 0, -3, 0, 1])
    for r in R.path_results:
        assert np.abs(roots - r.solution[0]).min() < 1e-10
    # y^2 + z = z^3 - y = 0: five solutions in the torus and (0, 0)
    y, z = hc.variables(2)
    H = hc.System.from_polys([y ** 2 + z, z ** 3 - y])
    T, S = ph.polyhedral(H, seed=2)
    assert len(S) == 6
    sols = [r.solution for r in T.track_arrays(S) if r.is_success()]
    assert len(sols) == 6
    assert min(np.abs(s).max() for s in sols) < 1e-10
    T, S = ph.polyhedral(H, only_non_zero=True, seed=2)
    assert sum(r.is_success() for r in T.track_arrays(S)) == 5


def test_polyhedral_solutions_certified():
    # every solution the polyhedral solve of cyclic-5 returns is certified, and all 70 distinct
    R = hc.solve(hc.cyclic(5), start_system="polyhedral", seed=2)
    C = hc.certify(hc.cyclic(5), R)
    assert C.ncertified() == 70
    assert C.ndistinct_certified() == 70


def test_toric_entry_point_argument_checks():
    from hcgpu import _lib
    from hcgpu.tracking import _Handle, make_options

    L = _lib.load()
    P = _lib.ptr
    F = f_example()
    eq, ex, cf = F.term_arrays()
    h = _Handle(make_options())
    nT = len(eq)
    W = np.zeros((1, nT))
    Wbad = W.copy()
    Wbad[0, 0] = -1.0
    assert L.hc_set_toric(h.h, 2, nT, P(eq), P(ex), P(cf), 1, P(Wbad)) == 1
    assert L.hc_set_toric(h.h, 2, nT, P(eq), P(ex), P(cf), 1, P(W)) == 0
    x = np.ones((1, 2), dtype=np.complex128)
    res = np.zeros(1, dtype=_lib.RESULT_DTYPE)
    sol = np.zeros((1, 2), dtype=np.complex128)
    t0, t1 = np.zeros(1), np.ones(1)
    row_bad = np.array([1], dtype=np.int32)
    row_ok = np.array([0], dtype=np.int32)
    assert L.hc_track_toric(h.h, 1, P(x), P(row_bad), P(t0), P(t1), None, None, P(res), P(sol)) == 1
    assert L.hc_track_toric(h.h, 1, P(x), P(row_ok), P(-t1), P(t1), None, None, P(res), P(sol)) == 1
    # a handle holding a toric homotopy refuses the straight-line entry points
    assert L.hc_track(h.h, 1, P(x), 1, 1.0, 0.0, 0.0, 0.0, P(res), P(sol), None, None) == 1
    assert b"toric" in L.hc_last_error(h.h)


def test_solve_polyhedral_affine_sqr():
    # test/solve_test.jl:95-100: 2 solutions
    x, y = hc.variables(2)
    F = hc.System.from_polys([2.3 * x ** 2 + 1.2 * y ** 2 + 3 * x - 2 * y + 3,
                              2.3 * x ** 2 + 1.2 * y ** 2 + 5 * x + 2 * y - 5])
    R = hc.solve(F, start_system="polyhedral", seed=3)
    assert R.nsolutions() == 2


@pytest.mark.parametrize("case", ["f", "f_torus", "cyclic5", "sparse0", "sparse1"])
def test_toric_stage_matches_oracle(case):
    import polyhedral_oracle as po

    if case.startswith("f"):
        T, S = ph.polyhedral(f_example(), only_torus=case == "f_torus", seed=1)
    elif case == "cyclic5":
        T, S = ph.polyhedral(hc.cyclic(5), seed=2)
    else:
        T, S = ph.polyhedral(sparse_system(int(case[-1])), seed=4)
    codes, x1, acc, rej, _ = T.track_toric(S)
    ocodes, ox1, oacc, orej = po.track_toric(T, S)
    assert (codes == ocodes).all()
    for k in np.nonzero(codes == 1)[0]:
        assert _rel(x1[k], ox1[k]) <= REL_TOL
    # the same algorithm: step counts agree up to rounding-level decisions
    assert abs(int(acc.sum()) - int(oacc.sum())) <= max(3, 0.01 * int(oacc.sum()))


@pytest.mark.parametrize("case", ["cyclic5", "sparse0", "sparse1", "sparse2"])
def test_polyhedral_matches_oracle(case):
    import polyhedral_oracle as po

    if case == "cyclic5":
        F = hc.cyclic(5)
        T, S = ph.polyhedral(F, seed=2)
    else:
        F = sparse_system(int(case[-1]))
        T, S = ph.polyhedral(F, seed=4)
    rs = T.track_arrays(S)
    ocodes, ox, _ = po.track(T, S)
    codes = np.array([{"success": 1, "polyhedral_failed": -1}.get(r.return_code, 0) for r in rs])
    assert ((codes == 1) == (ocodes == 1)).all()
    for k, r in enumerate(rs):
        if r.is_success() and not r.is_singular():
            assert _rel(r.solution, ox[k]) <= REL_TOL
    # no more paths than the mixed volume, and every nonsingular solution found twice by
    # neither: the solutions are distinct
    sols = [r.solution for r in rs if r.is_success() and not r.is_singular()]
    for i in range(len(sols)):
        for j in range(i + 1, len(sols)):
            assert _rel(sols[i], sols[j]) > 1e-6


def test_polyhedral_vs_total_degree_solutions():
    # the same finite solutions as the total-degree solve of the same system
    F = sparse_system(0)
    Rp = hc.solve(F, start_system="polyhedral", seed=5)
    Rt = hc.solve(F, gamma=np.exp(0.7j))
    sp = [r.solution for r in Rp.path_results if r.is_success() and not r.is_singular()]
    st = [r.solution for r in Rt.path_results if r.is_success() and not r.is_singular()]
    assert len(sp) == len(st)
    for x in sp:
        assert min(_rel(x, y) for y in st) <= 1e-8
