"""Polyhedral start systems on the CPU: mixed volumes, Hermite normal form and binomial systems
against the reference's known answers (test/polyhedral_test.jl, test/solve_test.jl:94-176,
test/binomial_system_test.jl), and the whole polyhedral tracker on the oracle
(test/polyhedral_test.jl:2-48 path counts)."""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "homotopycontinuation.jl_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import hcgpu as hc  # noqa: E402
from hcgpu import polyhedral_homotopy as ph  # noqa: E402


def f_example():
    x, y = hc.variables(2)
    return hc.System.from_polys([2 * y + 3 * y ** 2 - x * y ** 3, x + 4 * x ** 2 - 2 * x ** 3 * y])


def hc_i():
    x1, x2, s = hc.variables(3)
    return hc.System.from_polys([
        x1 ** 3 * s ** 15 + x1 * x2 * s + x2 ** 3 + s ** 12,
        x1 ** 2 * s ** 9 + x1 * x2 ** 2 + x2 * s ** 3,
        x1 ** 2 * x2 * s ** 5 + x1 * s ** 8 + x2 ** 2,
    ])


def test_paths_to_track_kat():
    # test/solve_test.jl:162-171: 8 polyhedral paths, 3 in the torus (mixed volume)
    f = f_example()
    assert ph.paths_to_track(f) == 8
    assert ph.paths_to_track(f, only_non_zero=True) == 3
    assert ph.mixed_volume(f) == 3


def test_only_torus_kat():
    # test/polyhedral_test.jl:23-36
    F = hc_i()
    assert ph.paths_to_track(F, only_torus=False) == 92
    assert ph.paths_to_track(F, only_torus=True) == 54


@pytest.mark.parametrize("n,mv", [(5, 70), (6, 156), (7, 924), (8, 2560)])
def test_cyclic_mixed_volume(n, mv):
    # cyclic-5: 70, cyclic-7: 924 (test/polyhedral_test.jl:39-46); cyclic-6: 156, cyclic-8: 2560
    assert ph.mixed_volume(hc.cyclic(n)) == mv


def test_small_systems_by_hand():
    # x^5 - 3x^2 + 1: 5 roots; y z = 1, y + z = 3: 2; y^2 + z = z^3 - y = 0: z = -y^2 and
    # y (y^5 + 1) = 0, so 5 solutions in the torus and (0, 0) besides
    x, = hc.variables(1)
    assert ph.mixed_volume(hc.System.from_polys([x ** 5 - 3 * x ** 2 + 1])) == 5
    y, z = hc.variables(2)
    assert ph.mixed_volume(hc.System.from_polys([y * z - 1, y + z - 3])) == 2
    H = hc.System.from_polys([y ** 2 + z, z ** 3 - y])
    assert ph.paths_to_track(H, only_non_zero=True) == 5
    assert ph.paths_to_track(H) == 6


def test_mixed_cells_are_fine_and_lifting_independent():
    sup = ph.support_coefficients(hc.cyclic(5))[0]
    vols = []
    for seed in range(3):
        cells, lift = ph.fine_mixed_cells(sup, seed=seed)
        vols.append(sum(c.volume for c in cells))
        for c in cells:
            # the normal is minimised exactly on the cell's edge in every support
            for i, (a, b) in enumerate(c.indices):
                vals = sup[i] @ c.normal + lift[i]
                assert abs(vals[a] - c.beta[i]) < 1e-8 and abs(vals[b] - c.beta[i]) < 1e-8
                others = np.delete(vals, [a, b])
                assert (others > c.beta[i] + 1e-9).all()
    assert vols == [70, 70, 70]


def test_hnf_kat():
    # test/binomial_system_test.jl:24-35
    A = np.array([[0, 3, 1, 0], [-2, 2, -1, 2], [1, -1, 2, 3], [-3, 3, 3, 2]])
    H, U = ph.hnf(A)
    assert (A.astype(object).dot(U) == H).all()
    assert all(H[i][j] == 0 for i in range(4) for j in range(i + 1, 4))
    assert abs(round(np.linalg.det(np.array(U, dtype=float)))) == 1
    H, U = ph.hnf(np.array([[-2]]))
    assert H[0][0] == 2 and U[0][0] == -1


def _binomial_err(A, b, X):
    return max(np.max(np.abs(np.array([np.prod(x ** a) for a in A.T]) - b) / np.abs(b)) for x in X.T)


def test_binomial_unit_b_kat():
    # test/binomial_system_test.jl:56-70: the reference's b vector
    A = np.array([[0, 1, 1, 0, -1], [0, 0, 0, 1, -1], [-1, 0, -1, 0, -1], [0, -1, 0, -1, -1], [1, 0, 0, 0, -1]])
    b = np.array([0.9053223983046926 + 0.4247250347316951j, 0.7000429487508004 - 0.7141007421255663j,
                  0.018811552539476483 - 0.9998230470893611j, -0.9983533473373446 + 0.057363698105327716j,
                  0.9999409355072137 - 0.010868555421874721j])
    X = ph.solve_binomial(A, b)
    assert X.shape == (5, 5)
    assert _binomial_err(A, b, X) < 1e-12


@pytest.mark.parametrize("unit", [True, False])
def test_binomial_general_kat(unit):
    # test/binomial_system_test.jl:72-106: |det A| = 6910 solutions
    A = np.array([[3, 2, 3, 4, 2, 5], [6, -3, 8, -3, 8, 7], [-2, -5, 7, 3, 6, 5], [1, 2, 3, 4, 5, 6],
                  [1, 0, 2, 0, 5, 0], [1, 2, 0, -3, 0, 5]])
    rng = np.random.default_rng(11)
    b = rng.standard_normal(6) + 1j * rng.standard_normal(6)
    if unit:
        b = b / np.abs(b)
    X = ph.solve_binomial(A, b)
    assert X.shape == (6, 6910)
    assert _binomial_err(A, b, X) < 1e-12
    assert len({tuple(np.round(x, 7)) for x in X.T}) == 6910


def test_binomial_univariate_and_unimodular():
    # x^3 = b: the three cube roots; a unimodular system has exactly one solution
    X = ph.solve_binomial(np.array([[3]]), np.array([2.0 + 1.0j]))
    assert X.shape == (1, 3)
    assert np.allclose(X[0] ** 3, 2.0 + 1.0j, rtol=1e-14)
    assert len({np.round(v, 10) for v in X[0]}) == 3
    A = np.array([[1, 1], [0, 1]])
    b = np.array([3.0 - 1.0j, 0.5j])
    X = ph.solve_binomial(A, b)
    assert X.shape == (2, 1)
    assert _binomial_err(A, b, X) < 1e-14


def test_cell_binomial_kat():
    # test/binomial_system_test.jl:108-121: a cell of cyclic-5 with random coefficients
    sup = ph.support_coefficients(hc.cyclic(5))[0]
    cells, lift = ph.fine_mixed_cells(sup, seed=0)
    rng = np.random.default_rng(5)
    coeffs = [rng.standard_normal(len(S)) + 1j * rng.standard_normal(len(S)) for S in sup]
    for c in cells[:5]:
        X = ph.cell_start_solutions(sup, coeffs, c)
        assert len(X) == c.volume
        for x in X:
            for i, (p, q) in enumerate(c.indices):
                lhs = coeffs[i][p] * np.prod(x ** sup[i][p]) + coeffs[i][q] * np.prod(x ** sup[i][q])
                scale = abs(coeffs[i][p] * np.prod(x ** sup[i][p]))
                assert abs(lhs) <= 1e-12 * scale


def test_underdetermined_raises():
    x, y = hc.variables(2)
    F = hc.System.from_polys([2.3 * x ** 2 + 1.2 * y ** 2 + 3 * x - 2 * y + 3])
    with pytest.raises(hc.FiniteException):
        ph.polyhedral(F)


@pytest.mark.parametrize("torus,npaths,nsucc", [(False, 8, 6), (True, 3, 3)])
def test_oracle_polyhedral_counts(torus, npaths, nsucc):
    # test/polyhedral_test.jl:2-21 on the oracle: 8 paths with 6 solutions, 3 in the torus
    import polyhedral_oracle as po

    T, S = ph.polyhedral(f_example(), only_torus=torus, seed=1)
    assert len(S) == npaths
    codes, xs, _ = po.track(T, S)
    assert (codes == 1).sum() == nsucc


def test_oracle_binomial_supports_only():
    # y^2 + z = z^3 - y = 0 with only_non_zero: both supports are binomials, so the cell is
    # the whole system and no toric weight is nonzero; 5 solutions in the torus
    import polyhedral_oracle as po

    y, z = hc.variables(2)
    H = hc.System.from_polys([y ** 2 + z, z ** 3 - y])
    T, S = ph.polyhedral(H, only_non_zero=True, seed=2)
    assert len(S) == 5
    codes, xs, _ = po.track(T, S)
    assert (codes == 1).all()
    for x in xs:
        assert np.abs(H.evaluate(x)).max() < 1e-12


def test_oracle_polyhedral_cyclic7():
    # test/polyhedral_test.jl:43-46: 924 solutions of cyclic-7, on the oracle
    import polyhedral_oracle as po

    T, S = ph.polyhedral(hc.cyclic(7), seed=6)
    assert len(S) == 924
    codes, xs, _ = po.track(T, S)
    assert (codes == 1).sum() == 924


def test_oracle_polyhedral_cyclic5():
    # test/polyhedral_test.jl:38-42: 70 solutions of cyclic-5
    import polyhedral_oracle as po

    F = hc.cyclic(5)
    T, S = ph.polyhedral(F, seed=2)
    assert len(S) == 70
    codes, xs, _ = po.track(T, S)
    assert (codes == 1).sum() == 70
    for x in xs:
        assert np.abs(F.evaluate(x)).max() < 1e-10
